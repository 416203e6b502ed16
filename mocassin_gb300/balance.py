"""Host side of the cell update (ionisation and thermal balance).

The cell update of updateCell (source/update_mod.f90:15-525) needs, per cell,
two sums over frequency of the normalised Jste for each of the 33 ions with
bound electrons up to nstages - 1 (H0; He0, He+; C, N, O, Ne, S stages 1..6):
    nPhotoSte = sum_j Jste(j) phXSec(j) / (hcRyd nu(j))            (:210-267)
    heatIon   = sum_{j >= IP} Jste(j) phXSec(j) (nu(j) - nu(IP)) / nu(j)
                (stopping at the first zero cross-section, :1170-1217)
and whether any Jste(j) > 0 (lgHit, :103-123).  All three are moments of
Jste with a fixed weight table, computed on the GPU by
TransportContext.jste_moments; this module builds the table, the initial
state and the per-cell abundances of the ion-density layout
[cell][element][stage 1..7].
"""
import os

import numpy as np

from . import nebula

HCRYD = 2.1799153e-11           # continuum_mod.f90:11
ELEMENTS = (1, 2, 6, 7, 8, 10, 16)
NSTAGES = 7
XSTRIDE = NSTAGES + 1           # stage index 1..7 (0 unused)
BALANCE_IONS = tuple((z, i) for z in ELEMENTS for i in range(1, min(z, NSTAGES - 1) + 1))
NBAL = len(BALANCE_IONS)        # 33
_TABLES = None


def tables():
    """The atomic data of the update (make_update_tables.py)."""
    global _TABLES
    if _TABLES is None:
        p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "update_tables.npz")
        _TABLES = {k: v for k, v in np.load(p).items()}
    return _TABLES


def abundances():
    return np.array([nebula.ABUNDANCES[z] for z in ELEMENTS], dtype=np.float64)


def moment_weights(xs, nu, ions):
    """(nbins, 1 + 2*NBAL) float32: column 0 = 1 (hit test), then the
    photoionisation weights and the heating weights of BALANCE_IONS."""
    nb = len(nu)
    nu64 = nu.astype(np.float64)
    rows = {tuple(int(v) for v in r): k for k, r in enumerate(ions)}
    w = np.zeros((nb, 1 + 2 * NBAL))
    w[:, 0] = 1.0
    for b, key in enumerate(BALANCE_IONS):
        x = xs[rows[key]].astype(np.float64)
        x = np.where(x < 1e-35, 0.0, x)
        w[:, 1 + b] = x / (HCRYD * nu64)
        nz = np.nonzero(x > 0)[0]
        if len(nz):
            ip = nz[0]
            end = ip
            while end < nb and x[end] >= 1e-35:
                end += 1
            j = np.arange(ip, end)
            w[j, 1 + NBAL + b] = x[j] * (nu64[j] - nu64[ip]) / nu64[j]
    return np.ascontiguousarray(w.astype(np.float32))


def ion_thresholds(xs, nu, ions):
    """Threshold energy [Ryd] of each of the 33 balance ions: nu at the first
    bin with a nonzero cross-section (the IP of the heating sums)."""
    rows = {tuple(int(v) for v in r): k for k, r in enumerate(ions)}
    out = np.zeros(NBAL)
    for b, key in enumerate(BALANCE_IONS):
        x = xs[rows[key]].astype(np.float64)
        nz = np.nonzero(x >= 1e-35)[0]
        out[b] = float(nu[nz[0]]) if len(nz) else 0.0
    return out


def initial_state(neb):
    """(te, ne, X) at the start of an iteration from the nebula's ion rows:
    X[cell, element, stage] fractions, the top stage the remainder."""
    nc1 = neb.ncells + 1
    tab = nebula.atomic_table()
    ions = [tuple(int(v) for v in r) for r in tab["ions"]]
    ab = {z: nebula.ABUNDANCES[z] for z in ELEMENTS}
    X = np.zeros((nc1, len(ELEMENTS), XSTRIDE))
    h = neb.hden.astype(np.float64)
    safe = np.where(h > 0, h, 1.0)
    for k, (z, st) in enumerate(ions):
        e = ELEMENTS.index(z)
        X[:, e, st] = neb.ion_den[:, k].astype(np.float64) / (ab[z] * safe)
    for e, z in enumerate(ELEMENTS):
        top = min(z + 1, NSTAGES)
        rest = 1.0 - X[:, e, 1:top].sum(1)
        X[:, e, top] = np.maximum(rest, 0.0)
    X = np.clip(X, 1e-20, None)
    X[:, :, 0] = 0.0
    for e, z in enumerate(ELEMENTS):
        X[:, e, min(z + 1, NSTAGES) + 1:] = 0.0
    te = np.full(nc1, float(neb.spec.te))
    ne = electron_density(X, h)
    return te, ne, X


def electron_density(X, hden):
    """Ne = Hden * sum (ion - 1) abund X over ions with X >= 1e-10 (ionBalance :1556-1568)."""
    ab = abundances()
    ne = np.zeros(X.shape[0])
    for e, z in enumerate(ELEMENTS):
        for ion in range(2, min(z + 1, NSTAGES) + 1):
            x = X[:, e, ion]
            ne += np.where(x >= 1e-10, (ion - 1) * ab[e] * x, 0.0)
    ne = ne * hden
    return np.where(ne == 0.0, 1.0, ne)


def opacity_species(X, hden, ions):
    """den[k, cell] = X(elem, stage) abund Hden for the opacity rows ``ions``
    (the ionDen x elemAbun x Hden of ionizationDriver, ionization_mod.f90:65-80)."""
    ab = {z: nebula.ABUNDANCES[z] for z in ELEMENTS}
    den = np.zeros((len(ions), X.shape[0]), dtype=np.float32)
    for k, (z, st) in enumerate(ions):
        den[k] = (X[:, ELEMENTS.index(z), st] * ab[z] * hden).astype(np.float32)
    den[:, 0] = 0.0
    return den
