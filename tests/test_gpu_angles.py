"""Viewing-angle planes of the escape SED on the GPU vs the oracle.

FP64: the same draws as the oracle, every counter exact and every plane of
escapedPackets to 1e-12 relative (wave and plain forms).  FP32: plane shares
against the solid-angle known answer of a vacuum within 4 sigma.
"""
import dataclasses

import numpy as np
import pytest

from mocassin_gb300 import nebula, transport
from oracle import runner
from tests import helpers

pytestmark = pytest.mark.gpu

RTOL = 1e-12
KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")
BASE = nebula.small_cases()
CASES = [
    dataclasses.replace(BASE[0], name="sym9_view", views=((0.5, 0.3),)),
    dataclasses.replace(BASE[1], name="sym11_two_views", views=((0.2, 1.2), (1.3, -1.0)), n_theta_bins=12),
    dataclasses.replace(BASE[2], name="full9_rout_views", views=((1.0, 0.7), (2.2, 5.5))),
    dataclasses.replace(BASE[3], name="full11_dust_iso_view", views=((1.2, -1.0),)),
    dataclasses.replace(BASE[4], name="full9_dust_hg_views", views=((0.9, 0.2), (2.6, 6.0)), n_phi_bins=24),
    dataclasses.replace(BASE[5], name="full9_twostar_view", views=((1.7, 0.1),)),
]


def _compare_planes(g, o):
    js, _, es, st = g
    ojs, _, oes, ost = o
    for k in KEYS:
        assert st[k] == ost[k], (k, st[k], ost[k])
    assert helpers.rel_err(js, ojs) < RTOL
    assert es.shape == oes.shape and es.ndim == 3
    for p in range(es.shape[0]):
        assert helpers.rel_err(es[p], oes[p]) < RTOL, p


@pytest.mark.parametrize("form", ("wave", "plain"))
@pytest.mark.parametrize("spec", CASES, ids=lambda s: s.name)
def test_fp64_parity_with_views(gpu_lib, spec, form):
    neb = nebula.build(spec)
    g = transport.energy_packet_driver(neb, precision="fp64", seed=23, form=form)
    o = runner.run(neb, precision="fp64", seed=23)
    _compare_planes(g, o)
    assert o[2][1:].sum() > 0.0


def test_fp32_vacuum_plane_share(gpu_lib):
    pi = float(np.float32(3.141592654))
    n = 400000
    spec = nebula.NebulaSpec("vac_views", 9, 3.0e18, False, [nebula.Star(40000.0, 10.0, (0, 0, 0), n)],
                             nh_median=100.0, r_in=0.0, views=((1.0, 0.7), (2.2, -1.0)))
    neb = helpers.vacuum(nebula.build(spec))
    _, _, es, st = transport.energy_packet_driver(neb, precision="fp32", seed=5)
    assert st["escaped"] == n
    # phi < 0 on any viewpoint switches phi off for all (grid_mod.f90:419-427)
    dth = pi / 10
    sh = es[1:].sum(axis=(1, 2)) / es[0].sum()
    for i, th in enumerate((1.0, 2.2)):
        k = int(th / dth)
        p = (np.cos(k * dth) - np.cos((k + 1) * dth)) / 2
        assert abs(sh[i] - p) < 4 * np.sqrt(p * (1 - p) / n)


def test_views_in_resident_context(gpu_lib):
    neb = nebula.build(CASES[2])
    ctx = transport.TransportContext(neb)
    ctx.run(seed=29, precision="fp64")
    js, _, es = ctx.download()
    ctx.close()
    o = runner.run(neb, precision="fp64", seed=29)
    assert es.shape == o[2].shape
    for p in range(es.shape[0]):
        assert helpers.rel_err(es[p], o[2][p]) < RTOL


def test_bad_views_rejected(gpu_lib):
    neb = nebula.build(dataclasses.replace(BASE[0], views=((2.0, 0.3),)))  # theta > pi/2 in an octant
    with pytest.raises(transport.TransportError):
        transport.energy_packet_driver(neb, precision="fp64")
