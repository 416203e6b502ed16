"""CPU oracle of the photoionisation sums of updateCell (test infrastructure).

Restates source/update_mod.f90:175-269 in FP64: for every cell and ion,
    nPhotoSte(ion) = 1e-20 + sum_{j in the ion's range} Jste(cell, j) * phXSec(j) / (hcRyd * nu(j))
with Jste normalised as iteration_mod.f90:705-724 does (x 1e-9, / 8 for a
symmetric octant); cross-sections below 1e-35 count as zero (:228-234).
The generic form used by the GPU kernel is moments(J, W, scale).
"""
import numpy as np

HCRYD = 2.1799153e-11  # continuum_mod.f90:11


def photo_weights(xs, nu):
    """W(nu, ion) = phXSec / (hcRyd nu), the phXSec < 1e-35 cut applied."""
    x = np.where(xs < 1e-35, 0.0, xs.astype(np.float64))
    return (x / (HCRYD * nu.astype(np.float64)[None, :])).T       # (nbins, nion)


def moments(jste, w, scale=1.0):
    """scale * sum_nu jste(nu, cell) w(nu, o) -> (nout, Nc+1)."""
    return scale * (w.astype(np.float64).T @ jste.astype(np.float64))


def n_photo(jste, xs, nu, symmetric):
    scale = 1e-9 / (8.0 if symmetric else 1.0)
    return 1e-20 + moments(jste, photo_weights(xs, nu), scale)
