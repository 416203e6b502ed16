"""Shared helpers of the test suite: analytic expectations and comparisons."""
import dataclasses

import numpy as np

from mocassin_gb300 import nebula


def vacuum(neb, kappa=0.0, debug=False):
    """The same grid with a grey opacity kappa [1/cm] (0 = vacuum) in every
    active cell and every packet marching (ionEdge(1) = 0)."""
    n = dataclasses.replace(neb)
    op = np.zeros_like(neb.opacity)
    op[:, 1:] = np.float32(kappa)
    n.opacity = op
    n.ion_edge1 = 0.0
    if debug:
        n.flags = neb.flags | nebula.FLAG_DEBUG
    return n


def octant_path_expectation(extent, kappa=0.0, symmetric=True, n=4_000_000, seed=12345):
    """E[first-flight path length] of an isotropic packet from the corner of a
    cube octant [0, R]^3 (symmetric grid) or the centre of [-R, R]^3: the ray
    leaves after s = R / max|u_i|; with grey absorption the path is
    min(s, Exp(kappa)) whose mean is (1 - exp(-kappa s)) / kappa."""
    rng = np.random.default_rng(seed)
    w = 2 * rng.random(n) - 1
    t = np.sqrt(1 - w * w)
    a = np.pi * (2 * rng.random(n) - 1)
    u = np.abs(np.stack([t * np.cos(a), t * np.sin(a), w]))
    s = extent / u.max(0)
    if kappa > 0:
        mean = float((-np.expm1(-kappa * s) / kappa).mean())
        # per-packet spread of the sampled path min(s, Exp(kappa))
        vals = np.minimum(s, rng.exponential(1.0 / kappa, n))
        return mean, float(vals.std())
    return float(s.mean()), float(s.std())


def cell_volumes(neb):
    """dV (in 1e45 cm^3) of every active cell, photon_mod.f90:1469-1512."""
    sym = bool(neb.flags & nebula.FLAG_SYMMETRIC_XYZ)

    def widths(ax):
        n = len(ax)
        w = np.zeros(n)
        a = ax.astype(np.float64)
        for p in range(1, n + 1):
            if 1 < p < n:
                d = abs(a[p] - a[p - 2]) / 2
            elif p == 1:
                d = abs(a[1] - a[0]) / (2 if sym else 1)
            else:
                d = abs(a[p - 1] - a[p - 2])
            w[p - 1] = d / 1e15
        return w

    wx, wy, wz = widths(neb.x_axis), widths(neb.y_axis), widths(neb.z_axis)
    vol = np.zeros(neb.ncells + 1)
    act = neb.active  # (z, y, x)
    zz, yy, xx = np.nonzero(act)
    vol[act[zz, yy, xx]] = wx[xx] * wy[yy] * wz[zz]
    return vol


def rel_err(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return float(np.abs(a - b).max() / scale)


def with_opacity(neb, opacity):
    """The same nebula with another opacity table (nbins, Nc+1)."""
    n = dataclasses.replace(neb)
    n.opacity = np.ascontiguousarray(opacity, dtype=np.float32)
    return n


def zeros_like_estimators(neb):
    nc1 = neb.ncells + 1
    from mocassin_gb300 import abi
    return np.zeros((neb.nbins, nc1)), np.zeros((neb.nbins, nc1)), np.zeros(abi.escaped_shape(neb))
