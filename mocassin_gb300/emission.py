"""Tables of the diffuse-emission CDF built on the GPU
(TransportContext.build_emission, mc_ctx_build_emission).

The reference computes each cell's recPDF row and totalLines on the host
before every transport (emissionDriver and setDiffusePDF,
source/emission_mod.f90:32-1311).  The data it reads -- the f-b + f-f gamma
tables, the two-photon distribution, the recombination-line ratios and fits,
the Gaunt-factor coefficients, the heavy ions' outer shells -- are in
data/emission_tables.npz (written from the reference's data files by
data/make_emission_tables.py).  This module adds the grid's own arrays
(nuArray, widFlx) and the ground-state cross-sections of H0, He0 and He+
from the cross-section matrix, and hands everything to the C-ABI, which
derives the per-bin tables and runs the kernels.
"""
import os

import numpy as np

from . import dust, nebula

T_SUBLIME = 1400.0  # sublimation temperature of the synthetic silicate-like grains [K]

_T = None


def _data():
    global _T
    if _T is None:
        d = np.load(os.path.join(os.path.dirname(__file__), "data", "emission_tables.npz"))
        _T = {k: d[k] for k in d.files}
    return _T


def tables(neb):
    """The emission tables for the frequency grid and cross-sections of a
    nebula built by mocassin_gb300.nebula."""
    t = dict(_data())
    if not np.array_equal(t["nu"], neb.nu):
        raise ValueError("the emission tables were made for another frequency grid")
    ions = [tuple(int(v) for v in r) for r in nebula.atomic_table()["ions"]]
    ix = {ion: k for k, ion in enumerate(ions)}
    t["wid_flx"] = nebula.wid_flx(neb.nu)
    t["xs_h"], t["xs_hei"], t["xs_heii"] = neb.xs[ix[(1, 1)]], neb.xs[ix[(2, 1)]], neb.xs[ix[(2, 2)]]
    if neb.flags & nebula.FLAG_DUST:
        # the grains of nebula._dust_kappa: one species, grainAbun 1
        xs_abs, w, _ = dust.grains(neb.nu)
        t["xs_abs"], t["grain_weight"], t["t_sublime"] = xs_abs, w, T_SUBLIME
        t["ndust"] = neb.ndust
    return t
