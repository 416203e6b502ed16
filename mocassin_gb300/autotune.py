"""Autotuner of the persistent march's scheduling parameters.

The march (wave_march_kernel) refills a warp's idle lanes from the
frequency-sorted queue once ``refill_min`` of them are free, and lets every
lane take ``inner_steps`` cell crossings between refill checks.  The best
pair depends on the grid (cells per chord, absorption per crossing) and on
how many packets a round holds, so it is measured: each candidate runs a
sample of the model's packets on the resident grid and the fastest by
device time wins.  The physics does not depend on the choice (each packet
consumes its own random stream in the reference order); only the order of
the FP64 estimator sums does.
"""
import itertools

DEFAULT_CANDIDATES = tuple(itertools.product((2, 4, 8, 16), (2, 4, 8, 16)))


def autotune(ctx, n_packets, candidates=DEFAULT_CANDIDATES, repeats=2, seed=77, precision="fp32", form="wave"):
    """Sets and returns the fastest (refill_min, inner_steps) for ``ctx``'s grid
    with ``n_packets`` per trial, and the table of timings (crossings/s)."""
    table = {}
    best, best_rate = None, -1.0
    for k, (rm, ins) in enumerate(candidates):
        ctx.set_tuning(rm, ins)
        rate = 0.0
        for r in range(repeats):
            st = ctx.run(n_packets=n_packets, seed=seed + r, precision=precision, zero_first=True, form=form)
            rate = max(rate, st["crossings"] / (st["kernel_ms"] / 1e3))
        table[(rm, ins)] = rate
        if rate > best_rate:
            best, best_rate = (rm, ins), rate
    ctx.set_tuning(*best)
    ctx.zero()
    return best, table
