"""CPU oracle of the opacity build (test infrastructure only).

Restates, in FP64, the dense form of addOpacity (source/ionization_mod.f90:
349-484: free-free in bin 1 only, then xSecArray * density summed over every
ion's shell ranges) and of the dust add of iterateMC
(source/iteration_mod.f90:166-227: grainAbun * grainWeight * Ndust *
(xs_sca + xs_abs) per grain species and size):

    opacity(cell, nu) = sum_k den(k, cell) * xs(k, nu) + ff(cell) [nu = 1]

with den [K][Nc+1] and xs [K][nbins] (cell / bin fastest) and the result
[nbins][Nc+1].  Parity unpinned, like the transport oracle: the reference
ships no golden vectors for it.
"""
import numpy as np


def opacity(den, xs, ff=None):
    out = xs.astype(np.float64).T @ den.astype(np.float64)   # (nbins, Nc+1)
    if ff is not None:
        out[0] += ff.astype(np.float64)
    return out
