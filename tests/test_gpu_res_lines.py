"""Resonance-line packets (energyPacketDriver, source/photon_mod.f90:180-266):
after each star's packets, resLinePackets(cell) "diffuse" packets from the
node of every active cell, each followed through its re-emissions.

- FP64 march, Philox draws: the GPU (wave and graph forms) against the
  oracle's restatement of the same branch, on the small dusty nebula with
  0..3 packets per cell: every counter exactly, Jste and escapedPackets to
  1e-12;
- the FP32 march sends the same number of extra histories;
- the forms and inputs it does not cover are refused."""
import numpy as np
import pytest

from mocassin_gb300 import nebula, transport
from oracle import runner
from tests import helpers

pytestmark = pytest.mark.gpu

KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")


def _counts(neb, seed=1, top=4):
    rng = np.random.default_rng(seed)
    c = np.zeros(neb.ncells + 1, dtype=np.int32)
    c[1:] = rng.integers(0, top, neb.ncells)
    return c


@pytest.mark.parametrize("case", [3, 4], ids=["full11_dust_iso", "full9_dust_hg"])
def test_fp64_resonance_packets_match_oracle(gpu_lib, case):
    neb = nebula.build(nebula.small_cases()[case])
    counts = _counts(neb)
    o = runner.run(neb, precision="fp64", seed=7, res_counts=counts)
    base = runner.run(neb, precision="fp64", seed=7)
    assert o[3]["lines"] > base[3]["lines"]
    for form in ("wave", "graph"):
        ctx = transport.TransportContext(neb)
        ctx.set_res_lines(counts)
        st = ctx.run(seed=7, precision="fp64", zero_first=True, form=form)
        js, _, es = ctx.download()
        ctx.close()
        for k in KEYS:
            assert st[k] == o[3][k], (form, k, st[k], o[3][k])
        assert helpers.rel_err(js, o[0]) < 1e-12
        assert helpers.rel_err(es, o[2]) < 1e-12


def test_fp32_resonance_packets_add_their_histories(gpu_lib):
    neb = nebula.build(nebula.small_cases()[3])
    counts = _counts(neb, seed=2)
    ctx = transport.TransportContext(neb)
    a = ctx.run(seed=3, precision="fp32", zero_first=True, form="graph")
    ctx.set_res_lines(counts)
    b = ctx.run(seed=3, precision="fp32", zero_first=True, form="graph")
    ctx.set_res_lines(None)
    c = ctx.run(seed=3, precision="fp32", zero_first=True, form="graph")
    ctx.close()
    assert c == a or all(c[k] == a[k] for k in KEYS)
    # every extra history ends as a line, an escape, a trap or a silent exit
    # (from an outer node); the round-0 histories are the same
    ends = lambda s: s["lines"] + s["escaped"] + s["trapped"] + s["silent_exits"]
    extra = ends(b) - ends(a)
    assert extra == int(counts.sum())


def test_resonance_packets_refused_where_not_built(gpu_lib):
    neb = nebula.build(nebula.small_cases()[3])
    ctx = transport.TransportContext(neb)
    bad = _counts(neb)
    bad[5] = -1
    with pytest.raises(transport.TransportError):
        ctx.set_res_lines(bad)
    ctx.set_res_lines(_counts(neb))
    with pytest.raises(transport.TransportError):
        ctx.run(seed=1, precision="fp64", form="plain")
    draws = np.random.default_rng(1).random((int(sum(neb.n_packets)), 256))
    with pytest.raises(transport.TransportError):
        ctx.run(seed=1, precision="fp64", replay=draws)
    ctx.close()
