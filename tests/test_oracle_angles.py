"""Viewing-angle planes of the escape SED in the oracle (photon_mod.f90:372-462,
grid_mod.f90:416-468), pinned by known answers: in a vacuum every packet
escapes on its first flight with an isotropic direction, so the share of a
viewing-angle plane is the solid-angle share of its theta (and phi) bin."""
import dataclasses

import numpy as np
import pytest

from mocassin_gb300 import nebula
from oracle import runner
from tests import helpers

PI = float(np.float32(3.141592654))
N = 60000


def vac(symmetric, views, n_theta=0, n_phi=0):
    spec = nebula.NebulaSpec("vac_views", 9, 3.0e18, symmetric, [nebula.Star(40000.0, 10.0, (0, 0, 0), N)],
                             nh_median=100.0, r_in=0.0, views=tuple(views), n_theta_bins=n_theta, n_phi_bins=n_phi)
    return helpers.vacuum(nebula.build(spec))


def share(es):
    return es[1:].sum(axis=(1, 2)) / es[0].sum()


def within(got, p, n=N):
    return abs(got - p) < 4 * np.sqrt(p * (1 - p) / n) + 1e-9


def test_theta_only_view_full_grid():
    # phi < 0 switches the phi dependence off (grid_mod.f90:419-427)
    neb = vac(False, [(1.0, -1.0)])
    _, _, es, st = runner.run(neb, precision="fp64", seed=11)
    assert es.shape == (2, neb.nbins + 1, neb.ncells + 1)
    assert st["escaped"] == N and abs(es[0].sum() - 10.0) < 1e-6 * 10  # deltaE is FP32
    dth = PI / 10
    k = int(1.0 / dth)  # bin [k dth, (k+1) dth)
    p = (np.cos(k * dth) - np.cos((k + 1) * dth)) / 2
    assert within(share(es)[0], p)


def test_theta_phi_view_full_grid():
    neb = vac(False, [(1.0, 0.7)])
    _, _, es, _ = runner.run(neb, precision="fp64", seed=12)
    dth, dph = PI / 10, 2 * PI / 20
    k = int(1.0 / dth)
    # atan (not atan2) of y/x is uniform on (-pi/2, pi/2): a phi bin above the
    # first holds dphi / pi of the directions
    p = (np.cos(k * dth) - np.cos((k + 1) * dth)) / 2 * (dph / PI)
    assert int(0.7 / dph) + 1 >= 2
    assert within(share(es)[0], p)


def test_symmetric_octant_view():
    neb = vac(True, [(0.5, 0.3)], n_theta=8, n_phi=16)
    _, _, es, _ = runner.run(neb, precision="fp64", seed=13)
    dth, dph = PI / 8, 2 * PI / 16
    k = int(0.5 / dth)
    # |z| is uniform on [0, 1] and atan(|y|/|x|) uniform on [0, pi/2)
    p = (np.cos(k * dth) - np.cos((k + 1) * dth)) * (dph / (PI / 2))
    assert within(share(es)[0], p)


def test_two_views_and_plane_zero_unchanged():
    views = [(1.0, 0.7), (2.2, 5.5)]
    neb0 = vac(False, [])
    neb2 = vac(False, views)
    _, _, e0, _ = runner.run(neb0, precision="fp64", seed=14)
    _, _, e2, _ = runner.run(neb2, precision="fp64", seed=14)
    # every escape still goes to plane 0, with the same draws
    np.testing.assert_array_equal(e2[0], e0)
    dth, dph = PI / 10, 2 * PI / 20
    for i, (th, ph) in enumerate(views):
        k = int(th / dth)
        pt = (np.cos(k * dth) - np.cos((k + 1) * dth)) / 2
        # 5.5 rad is reached by negative atan values, folded by totAngleBinsPhi + idirP
        assert within(share(e2)[i], pt * dph / PI)


def test_phi_bins_atan_cannot_reach_are_empty():
    # atan(y/x) lies in (-pi/2, pi/2): phi bins in (pi/2, 3pi/2) never fill
    _, _, es, _ = runner.run(vac(False, [(1.0, 0.7), (2.2, 4.0)]), precision="fp64", seed=15)
    assert share(es)[1] == 0.0 and share(es)[0] > 0.0


def test_invalid_views_are_errors():
    with pytest.raises(RuntimeError):
        runner.run(vac(True, [(2.0, 0.3)]), precision="fp64")       # theta > pi/2 in an octant
    with pytest.raises(RuntimeError):
        runner.run(vac(False, [(0.5, 0.1)] * 3), precision="fp64")  # at most two viewing angles
