"""MC_RUN_HOST_ZEROED: the drop-in call writes only what the transport made
nonzero into caller arrays that hold zeros on entry.

- The results equal those of the same call with MC_RUN_ZERO_FIRST (which
  writes every entry) -- the same entries nonzero, the values to 1e-12 for
  FP64 arrays and to one FP32 rounding for FP32 ones (the FP64 sums are
  atomics, so two calls differ in the last bits) -- for pageable (numpy) and
  pinned (page-locked) host arrays, on gas-only grids (identity and
  non-identity march layouts) and a dusty one, in the chosen and plain forms.
- The call reports the bytes it copied, and on a gas-only grid they are
  below those of the dense copies: the Jste rows below ionEdge(1) hold no
  deposit and escapedPackets is sparse.
- On a gas-only grid the opacity rows below ionEdge(1) are neither uploaded
  nor read: filling them with NaN leaves the results unchanged.
"""
import numpy as np
import pytest

from mocassin_gb300 import nebula, transport
from tests import helpers

pytestmark = pytest.mark.gpu

CASES = nebula.small_cases()


def _arrays(neb, dtype, pinned):
    js, _, es = helpers.zeros_like_estimators(neb)
    js, es = js.astype(dtype), es.astype(dtype)
    if not pinned:
        return js, es, None
    import torch
    tj = torch.from_numpy(js).pin_memory()
    te = torch.from_numpy(es).pin_memory()
    return tj.numpy(), te.numpy(), (tj, te)


@pytest.mark.parametrize("form", ["graph", "plain"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
@pytest.mark.parametrize("case", [1, 2, 3], ids=lambda i: CASES[i].name)
def test_host_zeroed_equals_the_dense_call(gpu_lib, case, pinned, dtype, form):
    neb = nebula.build(CASES[case])
    rj, re_ = (a.astype(dtype) for a in helpers.zeros_like_estimators(neb)[::2])
    transport.energy_packet_driver(neb, precision="fp64", seed=61, jste=rj, escaped=re_, zero_first=True, form=form)
    js, es, keep = _arrays(neb, dtype, pinned)
    _, _, _, st = transport.energy_packet_driver(neb, precision="fp64", seed=61, jste=js, escaped=es,
                                                 host_zeroed=True, form=form)
    rtol = 1e-12 if dtype == np.float64 else 2.5e-7
    for got, ref in ((js, rj), (es, re_)):
        assert np.array_equal(got != 0, ref != 0)
        np.testing.assert_allclose(got, ref, rtol=rtol, atol=0)
    assert st["h2d_bytes"] > 0 and st["d2h_bytes"] > 0
    if not neb.flags & nebula.FLAG_DUST:
        assert st["d2h_bytes"] < (rj.nbytes + re_.nbytes) / 2
    del keep


def test_gas_grid_reads_no_opacity_row_below_the_ionisation_edge(gpu_lib):
    neb = nebula.build(CASES[1])
    ref = transport.energy_packet_driver(neb, precision="fp64", seed=62, host_zeroed=True, form="graph")
    b0 = int(np.argmax(neb.nu >= np.float32(neb.ion_edge1)))
    assert b0 > 0
    bad = helpers.with_opacity(neb, neb.opacity.copy())
    bad.opacity[:b0] = np.nan
    for form in ("graph", "plain"):
        got = transport.energy_packet_driver(bad, precision="fp64", seed=62, host_zeroed=True, form=form)
        if form == "graph":
            np.testing.assert_allclose(got[0], ref[0], rtol=1e-12, atol=0)
            np.testing.assert_allclose(got[2], ref[2], rtol=1e-12, atol=0)
        assert np.isfinite(got[0]).all() and got[3]["crossings"] == ref[3]["crossings"]


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
def test_new_opacity_reaches_the_next_calls_march(gpu_lib, pinned):
    """A second drop-in call of the same grid shape keeps the device buffers
    of the first and uploads only the opacity rows a packet can march in:
    with another opacity it gives the transport of that opacity (the FP64
    plain form is the reference: the same draws, counters and sums to
    1e-12)."""
    neb = nebula.build(CASES[1])
    js, es, keep = _arrays(neb, np.float64, pinned)
    transport.energy_packet_driver(neb, precision="fp64", seed=71, jste=js, escaped=es, host_zeroed=True,
                                   form="graph")
    op = np.ascontiguousarray(neb.opacity * 3.0)
    if pinned:
        import torch
        top = torch.from_numpy(op).pin_memory()
        op = top.numpy()
    neb.opacity = op
    js2, es2, keep2 = _arrays(neb, np.float64, pinned)
    _, _, _, st = transport.energy_packet_driver(neb, precision="fp64", seed=72, jste=js2, escaped=es2,
                                                 host_zeroed=True, form="graph")
    rj, re_ = helpers.zeros_like_estimators(neb)[::2]
    _, _, _, ref = transport.energy_packet_driver(neb, precision="fp64", seed=72, jste=rj, escaped=re_,
                                                  zero_first=True, form="plain")
    for k in ("crossings", "absorptions", "escaped"):
        assert st[k] == ref[k], (k, st[k], ref[k])
    np.testing.assert_allclose(js2, rj, rtol=1e-12, atol=0)
    np.testing.assert_allclose(es2, re_, rtol=1e-12, atol=0)
    del keep, keep2
