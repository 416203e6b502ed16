"""Parity of the GPU transport (through the C-ABI) with the CPU oracle.

FP64 march: the GPU consumes the same draws as the oracle (Philox streams or
a replay buffer) and must reproduce every counter exactly and Jste /
escapedPackets to 1e-12 relative.  FP32 march: stochastic agreement with the
FP64 oracle within 4 sigma of packet noise.
"""
import os

import numpy as np
import pytest

from mocassin_gb300 import nebula, transport
from oracle import runner
from tests import helpers
from tests.golden import make_golden

pytestmark = pytest.mark.gpu

CASES = nebula.small_cases()
KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")
GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "transport_small_fp64.npz"))
RTOL = 1e-12


def _compare(g, o):
    js, _, es, st = g
    ojs, _, oes, ost = o
    for k in KEYS:
        assert st[k] == ost[k], (k, st[k], ost[k])
    assert helpers.rel_err(js, ojs) < RTOL
    assert helpers.rel_err(es, oes) < RTOL
    assert abs(st["qphot"] - ost["qphot"]) <= 1e-12 * max(abs(ost["qphot"]), 1e-300)


FORMS = ("wave", "plain")


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("spec", CASES, ids=lambda s: s.name)
def test_fp64_philox_parity(gpu_lib, spec, form):
    neb = nebula.build(spec)
    g = transport.energy_packet_driver(neb, precision="fp64", seed=17, form=form)
    o = runner.run(neb, precision="fp64", seed=17)
    _compare(g, o)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("spec", CASES[:4], ids=lambda s: s.name)
def test_fp64_replay_parity(gpu_lib, spec, form):
    neb = nebula.build(spec)
    n = 800
    draws = np.random.default_rng(99).random((n * len(neb.n_packets), 2048))
    g = transport.energy_packet_driver(neb, n_packets=n, precision="fp64", replay=draws, form=form)
    o = runner.run(neb, n_packets=n, precision="fp64", replay=draws)
    _compare(g, o)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("spec", CASES, ids=lambda s: s.name)
def test_fp64_matches_golden(gpu_lib, spec, form):
    neb = nebula.build(spec)
    js, _, es, st = transport.energy_packet_driver(neb, precision="fp64", seed=make_golden.SEED, form=form)
    counts = np.array([st[k] for k in make_golden.KEYS])
    np.testing.assert_array_equal(counts, GOLDEN[spec.name + "/counts"])
    np.testing.assert_allclose(js.sum(0), GOLDEN[spec.name + "/j_cell"], rtol=RTOL, atol=0)
    np.testing.assert_allclose(es.sum(1), GOLDEN[spec.name + "/esc_nu"], rtol=RTOL, atol=0)


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("spec", [CASES[1], CASES[2], CASES[3], CASES[4]], ids=lambda s: s.name)
def test_fp32_march_agrees_with_fp64_oracle(gpu_lib, spec, form):
    """Band-integrated J per cell: GPU FP32 vs oracle FP64 over 8 seeds each;
    the difference of the means stays within 4 sigma (batch means) for the
    grid total and for >= 97% of well-sampled cells."""
    neb = nebula.build(spec)
    g, o = [], []
    for seed in range(1, 9):
        g.append(transport.energy_packet_driver(neb, n_packets=3000, precision="fp32", seed=seed,
                                                form=form)[0].sum(0))
        o.append(runner.run(neb, n_packets=3000, precision="fp64", seed=100 + seed)[0].sum(0))
    g, o = np.array(g), np.array(o)
    sig = np.sqrt(g.var(0, ddof=1) / len(g) + o.var(0, ddof=1) / len(o))
    d = np.abs(g.mean(0) - o.mean(0))
    tot_sig = np.sqrt(g.sum(1).var(ddof=1) / len(g) + o.sum(1).var(ddof=1) / len(o))
    assert abs(g.sum(1).mean() - o.sum(1).mean()) < 4 * tot_sig
    ok = sig > 0.02 * o.mean(0).clip(1e-300)
    frac = float(np.mean(d[ok] < 4 * sig[ok]))
    assert frac >= 0.97, frac


@pytest.mark.parametrize("form", FORMS)
def test_vacuum_known_answer_on_gpu(gpu_lib, form):
    spec = nebula.NebulaSpec("vac", 9, 3.0e18, True, [nebula.Star(40000.0, 10.0, (0, 0, 0), 200000)],
                             nh_median=100.0, r_in=0.0)
    neb = helpers.vacuum(nebula.build(spec))
    for prec in ("fp64", "fp32"):
        js, _, es, st = transport.energy_packet_driver(neb, precision=prec, seed=3, form=form)
        path = (js.sum(0) * helpers.cell_volumes(neb)).sum() / (neb.delta_e[0] * neb.n_packets[0])
        mu, sd = helpers.octant_path_expectation(3.0e18)
        assert abs(path - mu) < 4 * sd / np.sqrt(neb.n_packets[0]) + 1e-3 * mu, prec
        assert st["escaped"] == neb.n_packets[0]


@pytest.mark.parametrize("form", ["wave", "graph"])
@pytest.mark.parametrize("sym", [True, False])
def test_counted_stellar_escapes_equal_one_by_one_sums(gpu_lib, form, sym):
    """The fast march counts a warp's stellar escapes of its bin and adds
    count x deltaE to escapedPackets(star cell, nu); one thread per history
    adds deltaE per escape.  In vacuum every stellar packet escapes in round
    0 and both forms draw the same bins, so the SEDs agree to rounding."""
    stars = [nebula.Star(40000.0, 10.0, (0, 0, 0), 200000)]
    if not sym:
        stars.append(nebula.Star(60000.0, 5.0, (0.34, 0.0, 0.0), 100000))
    spec = nebula.NebulaSpec("vacesc", 9 if sym else 11, 3.0e18, sym, stars, nh_median=100.0, r_in=0.0)
    neb = helpers.vacuum(nebula.build(spec))
    _, _, es_w, st_w = transport.energy_packet_driver(neb, precision="fp32", seed=5, form=form)
    _, _, es_p, st_p = transport.energy_packet_driver(neb, precision="fp32", seed=5, form="plain")
    assert st_w["escaped"] == st_p["escaped"] == int(np.sum(neb.n_packets))
    assert es_w.sum() > 0
    np.testing.assert_allclose(es_w, es_p, rtol=1e-12, atol=0)


@pytest.mark.parametrize("form,prec", [("wave", "fp32"), ("graph", "fp32"), ("wave", "fp64")])
def test_safe_limit_known_answer(gpu_lib, form, prec):
    """safeLimit (photon_mod.f90:1190) ends a packet's pathSegment after that
    many loop bodies.  In a vacuum octant of 9 cells per axis with the star in
    the corner cell a packet needs at least 9 crossings to leave, so with a
    limit of 3 every packet stops after exactly 3."""
    spec = nebula.NebulaSpec("vacsafe", 9, 3.0e18, True, [nebula.Star(40000.0, 10.0, (0, 0, 0), 20000)],
                             nh_median=100.0, r_in=0.0)
    neb = helpers.vacuum(nebula.build(spec))
    _, _, _, st = transport.energy_packet_driver(neb, precision=prec, seed=9, form=form, safe_limit=3)
    n = int(neb.n_packets[0])
    assert st["safe_limit_hits"] == n and st["crossings"] == 3 * n and st["escaped"] == 0


@pytest.mark.parametrize("form", FORMS)
def test_zero_packets_and_errors(gpu_lib, form):
    neb = nebula.build(CASES[0])
    js, _, es, st = transport.energy_packet_driver(neb, n_packets=0, precision="fp32", form=form)
    assert st["crossings"] == 0 and js.sum() == 0 and es.sum() == 0
    bad = nebula.build(CASES[0])
    bad.star_cell = [(0, 1, 1)]
    with pytest.raises(transport.TransportError) as e:
        transport.energy_packet_driver(bad, n_packets=10, form=form)
    assert e.value.status == 3  # MC_ERR_BOUNDS
    # replay stream too short: MC_ERR_REPLAY, reported by the device, no fault
    draws = np.full((10, 3), 0.5)
    with pytest.raises(transport.TransportError) as e:
        transport.energy_packet_driver(neb, n_packets=10, precision="fp64", replay=draws, form=form)
    assert e.value.status == 5
    # the library stays usable after device-side errors
    js, _, es, st = transport.energy_packet_driver(neb, n_packets=100, precision="fp64", seed=1, form=form)
    assert st["escaped"] + st["lines"] == 100


@pytest.mark.parametrize("form", FORMS)
def test_watchdog_returns_timeout_status(gpu_lib, monkeypatch, form):
    """A kernel budget of ~0 makes every thread give up after its first
    check: the call returns MC_ERR_TIMEOUT and the context stays usable."""
    neb = nebula.build(nebula.octant21(20000))
    monkeypatch.setenv("MC_KERNEL_BUDGET_S", "1e-9")
    with pytest.raises(transport.TransportError) as e:
        transport.energy_packet_driver(neb, precision="fp32", form=form)
    assert e.value.status == 6
    monkeypatch.delenv("MC_KERNEL_BUDGET_S")
    js, _, es, st = transport.energy_packet_driver(neb, precision="fp32", form=form)
    assert st["escaped"] + st["lines"] == 20000


def test_resident_context_accumulates(gpu_lib):
    neb = nebula.build(CASES[1])
    ctx = transport.TransportContext(neb)
    s1 = ctx.run(seed=5, precision="fp64")
    s2 = ctx.run(seed=6, precision="fp64")
    js, _, es = ctx.download()
    a = runner.run(neb, precision="fp64", seed=5)
    b = runner.run(neb, precision="fp64", seed=6)
    assert helpers.rel_err(js, a[0] + b[0]) < RTOL
    ctx.zero()
    js0, _, _ = ctx.download()
    assert js0.sum() == 0
    ctx.close()
    assert s1["crossings"] == a[3]["crossings"] and s2["crossings"] == b[3]["crossings"]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("symmetric", [True, False])
def test_grey_absorber_known_answer_on_gpu(gpu_lib, form, prec, symmetric):
    """First-flight path length with a grey absorber: E[(1 - exp(-kappa s)) / kappa]
    over isotropic directions, s the distance to the march boundary."""
    spec = nebula.NebulaSpec("grey", 11, 3.0e18, symmetric, [nebula.Star(40000.0, 10.0, (0, 0, 0), 200000)],
                             nh_median=100.0, r_in=0.0)
    neb = helpers.vacuum(nebula.build(spec), kappa=6.0e-19, debug=True)
    js, jd, es, st = transport.energy_packet_driver(neb, precision=prec, seed=21, form=form)
    path = (js.sum(0) * helpers.cell_volumes(neb)).sum() / (neb.delta_e[0] * neb.n_packets[0])
    mu, sd = helpers.octant_path_expectation(3.0e18, kappa=6.0e-19)
    assert abs(path - mu) < 4 * sd / np.sqrt(neb.n_packets[0]) + 2e-4 * mu
    assert st["escaped"] + st["lines"] + st["trapped"] == neb.n_packets[0]


def test_drop_in_call_accumulates_and_reuses_its_buffers(gpu_lib):
    """Two drop-in calls into the same arrays add up (the Fortran zeroes Jste
    once per iteration and calls once per star); a call on another grid shape
    in between makes the library rebuild its cached buffers."""
    neb = nebula.build(CASES[1])
    other = nebula.build(CASES[0])
    js, jd, es = helpers.zeros_like_estimators(neb)
    transport.energy_packet_driver(neb, precision="fp64", seed=41, jste=js, escaped=es)
    transport.energy_packet_driver(other, precision="fp64", seed=1)
    transport.energy_packet_driver(neb, precision="fp64", seed=42, jste=js, escaped=es)
    a = runner.run(neb, precision="fp64", seed=41)
    b = runner.run(neb, precision="fp64", seed=42)
    assert helpers.rel_err(js, a[0] + b[0]) < RTOL
    assert helpers.rel_err(es, a[2] + b[2]) < RTOL
    assert gpu_lib.mc_transport_release() == 0


def test_drop_in_zero_first_overwrites(gpu_lib):
    neb = nebula.build(CASES[2])
    ref = transport.energy_packet_driver(neb, precision="fp64", seed=41)
    js, jd, es = helpers.zeros_like_estimators(neb)
    js[:] = 1.0
    es[:] = 2.0
    got = transport.energy_packet_driver(neb, precision="fp64", seed=41, jste=js, escaped=es, zero_first=True)
    assert helpers.rel_err(got[0], ref[0]) < 1e-12 and helpers.rel_err(got[2], ref[2]) < 1e-12


@pytest.mark.gpu
def test_drop_in_fp32_estimators_are_the_fp64_sums_rounded(gpu_lib):
    """mc_transport_run_f32 writes the grid's own 4-byte arrays: the FP64
    device sums rounded once (so within one FP32 rounding of the FP64 call's
    results), and it accumulates into their current values."""
    neb = nebula.build(CASES[2])
    ref = transport.energy_packet_driver(neb, precision="fp64", seed=41)
    js = np.zeros_like(ref[0], dtype=np.float32)
    es = np.zeros_like(ref[2], dtype=np.float32)
    got = transport.energy_packet_driver(neb, precision="fp64", seed=41, jste=js, escaped=es, zero_first=True)
    for a, b in ((got[0], ref[0]), (got[2], ref[2])):
        assert a.dtype == np.float32
        np.testing.assert_allclose(a, b.astype(np.float32), rtol=2.5e-7, atol=0)
    js2 = np.full_like(js, 0.5)
    es2 = np.full_like(es, 0.25)
    acc = transport.energy_packet_driver(neb, precision="fp64", seed=41, jste=js2, escaped=es2)
    np.testing.assert_allclose(acc[0], (ref[0] + 0.5).astype(np.float32), rtol=2.5e-7, atol=0)
    np.testing.assert_allclose(acc[2], (ref[2] + 0.25).astype(np.float32), rtol=2.5e-7, atol=0)
