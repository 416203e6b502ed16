"""Pins the CPU oracle before it is trusted as the checker.

The reference (Fortran 90 + MPI) ships no tests, fixtures or golden vectors
and cannot be compiled here, so the oracle is pinned by:
  * the published Philox4x32-10 known-answer vectors (Salmon et al. 2011,
    Random123 kat_vectors) for the draw streams;
  * analytic known answers of the transport itself: total path length of an
    isotropic point source in vacuum and the first-flight path length with a
    grey absorber, (1 - exp(-kappa s)) / kappa averaged over directions;
  * conservation of packets and of escaped energy.
"""
import numpy as np
import pytest

from mocassin_gb300 import nebula
from oracle import runner
from tests import helpers


def test_philox_known_answers():
    assert runner.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert runner.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert runner.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_draw_streams_are_uniform_and_in_range():
    d64 = runner.draws(1, 1, 1, 12345, 1, 20000)
    d32 = runner.draws(1, 1, 1, 12345, 0, 20000)
    for d in (d64, d32):
        assert d.min() >= 0.0 and d.max() < 1.0
        assert abs(d.mean() - 0.5) < 0.01 and abs(d.var() - 1 / 12) < 0.005
    # FP32 draw k is the top 24 bits of word k; FP64 draw k spans words 2k, 2k+1
    assert np.all(d32 * 2 ** 24 == np.floor(d32 * 2 ** 24))
    assert not np.array_equal(runner.draws(1, 1, 1, 0, 1, 8), runner.draws(1, 1, 2, 0, 1, 8))
    assert not np.array_equal(runner.draws(1, 1, 1, 0, 1, 8), runner.draws(1, 2, 1, 0, 1, 8))


@pytest.mark.parametrize("symmetric", [True, False])
def test_vacuum_total_path_length(symmetric):
    n = 9
    spec = nebula.NebulaSpec("vac", n, 3.0e18, symmetric, [nebula.Star(40000.0, 10.0, (0, 0, 0), 40000)],
                             nh_median=100.0, r_in=0.0)
    neb = helpers.vacuum(nebula.build(spec))
    js, _, es, st = runner.run(neb, precision="fp64", seed=3)
    vol = helpers.cell_volumes(neb)
    path = (js.sum(0) * vol).sum() / (neb.delta_e[0] * neb.n_packets[0])
    # symmetric: cube [0, R]^3 from its corner; full grid: the march region is
    # [x1, xn]^3 = [-R, R]^3 from the centre (the packet escapes at the node)
    mu, sd = helpers.octant_path_expectation(3.0e18)
    assert abs(path - mu) < 4 * sd / np.sqrt(neb.n_packets[0]) + 1e-3 * mu
    assert st["escaped"] == neb.n_packets[0]
    assert st["absorptions"] == 0 and st["lines"] == 0
    assert abs(es.sum() - 10.0) < 1e-6 * 10


@pytest.mark.parametrize("kappa", [1.0e-19, 6.0e-19])
def test_grey_first_flight_path_length(kappa):
    spec = nebula.NebulaSpec("grey", 11, 3.0e18, True, [nebula.Star(40000.0, 10.0, (0, 0, 0), 40000)],
                             nh_median=100.0, r_in=0.0)
    neb = helpers.vacuum(nebula.build(spec), kappa=kappa, debug=True)
    js, jd, es, st = runner.run(neb, precision="fp64", seed=5)
    vol = helpers.cell_volumes(neb)
    # debug routes diffuse (re-emitted) packets to Jdif: Jste is first flight only
    path = (js.sum(0) * vol).sum() / (neb.delta_e[0] * neb.n_packets[0])
    mu, sd = helpers.octant_path_expectation(3.0e18, kappa=kappa)
    assert abs(path - mu) < 4 * sd / np.sqrt(neb.n_packets[0]) + 1e-3 * mu
    # first-flight absorption probability E[1 - exp(-kappa s)]
    rng = np.random.default_rng(1)
    w = 2 * rng.random(2_000_000) - 1
    t = np.sqrt(1 - w * w)
    a = np.pi * (2 * rng.random(2_000_000) - 1)
    u = np.abs(np.stack([t * np.cos(a), t * np.sin(a), w]))
    p_abs = float((-np.expm1(-kappa * 3.0e18 / u.max(0))).mean())
    # absorptions count first flights plus re-emitted continuum packets
    assert st["absorptions"] >= p_abs * neb.n_packets[0] - 4 * np.sqrt(neb.n_packets[0])
    assert jd.sum() > 0


def test_packet_and_energy_conservation():
    for spec in nebula.small_cases():
        neb = nebula.build(spec)
        js, jd, es, st = runner.run(neb, precision="fp64", seed=11)
        n = sum(neb.n_packets)
        ended = st["escaped"] + st["lines"] + st["trapped"] + st["silent_exits"] + st["safe_limit_hits"]
        assert ended == n, (spec.name, st)
        lum = sum(float(d) * k for d, k in zip(neb.delta_e, neb.n_packets))
        e_lines = 0.0
        # every packet carries deltaE of its star: escaped energy + line energy = L
        if len(neb.n_packets) == 1:
            e_lines = st["lines"] * float(neb.delta_e[0])
            assert abs(es.sum() + e_lines - lum) < 1e-9 * lum, spec.name
        assert np.all(js >= 0) and np.all(es >= 0)
        assert st["crossings"] > 0


def test_resonance_packets_in_the_oracle():
    """No resonance-line packets is the plain transport (to the rounding of
    the threads' sums); each extra packet is one more history that ends as
    a line, an escape or a trap."""
    import numpy as np
    from mocassin_gb300 import nebula
    from oracle import runner
    from tests import helpers
    neb = nebula.build(nebula.small_cases()[3])
    a = runner.run(neb, precision="fp64", seed=4)
    b = runner.run(neb, precision="fp64", seed=4, res_counts=np.zeros(neb.ncells + 1, np.int32))
    for k in ("crossings", "absorptions", "lines", "escaped", "trapped"):
        assert a[3][k] == b[3][k]
    assert helpers.rel_err(a[0], b[0]) < 1e-13
    cnt = np.zeros(neb.ncells + 1, np.int32)
    cnt[1:] = np.random.default_rng(1).integers(0, 3, neb.ncells)
    c = runner.run(neb, precision="fp64", seed=4, res_counts=cnt)
    ends = lambda s: s["lines"] + s["escaped"] + s["trapped"] + s["silent_exits"]
    assert ends(c[3]) - ends(a[3]) == int(cnt.sum())
