"""One persistent march over many models (mc_batch_run) gives each model the
transport of its own mc_ctx_run: the same draws, counters and rounds; Jste and
escapedPackets to 1e-12 in FP64 (only the order of the FP64 sums differs) and
to 1e-5 in FP32, where the warp-private FP32 accumulators flush in an order
that depends on scheduling."""
import pytest

from mocassin_gb300 import nebula, transport
from tests import helpers

pytestmark = pytest.mark.gpu

KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")
GAS = [s for s in nebula.small_cases() if not s.dust]
DUST = [s for s in nebula.small_cases() if s.dust]


def _own_runs(nebs, seeds, precision):
    out = []
    for neb, seed in zip(nebs, seeds):
        ctx = transport.TransportContext(neb)
        try:
            st = ctx.run(seed=seed, precision=precision)
            js, _, es = ctx.download()
        finally:
            ctx.close()
        out.append((st, js, es))
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("group", ["gas", "dust"])
def test_batch_matches_each_models_own_run(gpu_lib, precision, group):
    specs = GAS if group == "gas" else DUST
    nebs = [nebula.build(s) for s in specs]
    seeds = [11 + 7 * i for i in range(len(nebs))]
    ctxs = [transport.TransportContext(n) for n in nebs]
    try:
        stats = transport.batch_run(ctxs, seeds=seeds, precision=precision)
        got = [c.download() for c in ctxs]
    finally:
        for c in ctxs:
            c.close()
    tol = 1e-12 if precision == "fp64" else 1e-5
    for (st, (js, _, es)), (ref, rjs, res) in zip(zip(stats, got), _own_runs(nebs, seeds, precision)):
        for k in KEYS:
            assert st[k] == ref[k], (k, st[k], ref[k])
        assert st["rounds"] == ref["rounds"]
        assert st["crossings"] > 0
        assert helpers.rel_err(js, rjs) < tol
        assert helpers.rel_err(es, res) < tol


def test_batch_of_uneven_models_and_repeated_calls(gpu_lib):
    """Models of very different packet counts share the launches; a second
    call accumulates like a second mc_ctx_run."""
    nebs = [nebula.build(GAS[0]), nebula.build(GAS[1]), nebula.build(GAS[3])]
    npk = [20000, 300, 5000]
    ctxs = [transport.TransportContext(n) for n in nebs]
    try:
        transport.batch_run(ctxs, n_packets=npk, seeds=[1, 2, 3], precision="fp64")
        transport.batch_run(ctxs, n_packets=npk, seeds=[4, 5, 6], precision="fp64")
        got = [c.download() for c in ctxs]
    finally:
        for c in ctxs:
            c.close()
    for i, neb in enumerate(nebs):
        ctx = transport.TransportContext(neb)
        try:
            ctx.run(n_packets=npk[i], seed=1 + i, precision="fp64")
            ctx.run(n_packets=npk[i], seed=4 + i, precision="fp64")
            rjs, _, res = ctx.download()
        finally:
            ctx.close()
        assert helpers.rel_err(got[i][0], rjs) < 1e-12
        assert helpers.rel_err(got[i][2], res) < 1e-12


def test_batch_rejects_gas_and_dust_together(gpu_lib):
    ctxs = [transport.TransportContext(nebula.build(GAS[0])), transport.TransportContext(nebula.build(DUST[0]))]
    try:
        with pytest.raises(transport.TransportError) as e:
            transport.batch_run(ctxs, seeds=[1, 2])
        assert e.value.status == 7  # MC_ERR_UNSUPPORTED
        # the contexts stay usable
        st = transport.batch_run(ctxs[:1], seeds=[1])
        assert st[0]["escaped"] + st[0]["lines"] > 0
    finally:
        for c in ctxs:
            c.close()


def test_lockstep_lambda_iteration_matches_each_models_own(gpu_lib):
    """iterate.batched_step: the models' transports in one mc_batch_run, then
    their own updates.  The first iteration draws as each model's own step
    (same crossings); the states after two iterations agree with the own
    iterations' to the FP32 noise of the accumulators' flush order."""
    import numpy as np

    from mocassin_gb300 import iterate
    specs = [GAS[0], GAS[2]]
    a = [iterate.LambdaIteration(nebula.build(s), form="wave") for s in specs]
    b = [iterate.LambdaIteration(nebula.build(s), form="wave") for s in specs]
    try:
        ra = iterate.batched_step(a, [50, 50])
        rb = [m.step(seed=50) for m in b]
        for x, y in zip(ra, rb):
            assert x["crossings"] == y["crossings"]
        iterate.batched_step(a, [51, 51])
        for m in b:
            m.step(seed=51)
        for x, y in zip(a, b):
            ta, tb = x.ctx.get_cell_state()[0], y.ctx.get_cell_state()[0]
            ok = (ta > 0) & (tb > 0)
            assert ok.sum() > 0
            assert float(np.median(np.abs(ta[ok] / tb[ok] - 1))) < 1e-3
    finally:
        for m in a + b:
            m.close()


def test_lockstep_server_serves_every_request(gpu_lib):
    from mocassin_gb300 import serve
    srv = serve.ModelServer(workers=2, iterations=2, lockstep=True, group=2)
    for s in (GAS[0], GAS[1], GAS[2]):
        srv.submit(s)
    rep = srv.run()
    assert rep["errors"] == [] and rep["models"] == 3 and rep["iterations"] == 6
    assert rep["latency_ms_p50"] > 0 and rep["mode"].startswith("lockstep")
