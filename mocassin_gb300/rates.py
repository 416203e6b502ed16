"""Host side of the cell-update moments (photoionisation sums of updateCell).

updateCell (source/update_mod.f90:175-269) forms, per cell and ion,
    nPhotoSte = 1e-20 + sum_j Jste(cell, j) * phXSec(j) / (hcRyd * nu(j)),
phXSec below 1e-35 counted as zero (:228-234), on the Jste that
iteration_mod.f90:705-724 normalised (x 1e-9, / 8 for a symmetric octant).
The sum runs on the GPU (TransportContext.jste_moments); this module builds
the weight table and applies the normalisation and the 1e-20 floor.
"""
import numpy as np

HCRYD = 2.1799153e-11  # erg per Rydberg (continuum_mod.f90:11)


def photo_weights(xs, nu):
    """(nbins, nion) float32 table phXSec / (hcRyd nu) with the 1e-35 cut."""
    x = np.where(xs < 1e-35, 0.0, xs.astype(np.float64))
    return np.ascontiguousarray((x / (HCRYD * nu.astype(np.float64)[None, :])).T.astype(np.float32))


def jste_scale(symmetric):
    return 1e-9 / (8.0 if symmetric else 1.0)


def n_photo(ctx, xs, nu, symmetric):
    """nPhotoSte for every ion and cell, shape (nion, Nc+1), on the resident Jste of ``ctx``."""
    out, _ = ctx.jste_moments(photo_weights(xs, nu), jste_scale(symmetric))
    return out.astype(np.float64) + 1e-20
