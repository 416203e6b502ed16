"""CPU oracle of the grain temperatures (getDustT, source/update_mod.f90:1836-1945;
test infrastructure only): the absorbed integrals in FP64 and the reference's
`locate` (interpolation_mod.f90) followed by its linear step."""
import numpy as np


def locate(xa, x):
    """interpolation_mod locate: n above the table, 0 below, else
    max(minloc(xa - x, mask xa - x > 0) - 1, 1) (1-based)."""
    n = len(xa)
    if x > xa[n - 1]:
        return n
    if x < xa[0]:
        return 0
    d = xa - x
    pos = np.nonzero(d > 0)[0]
    first = (pos[np.argmin(d[pos])] + 1) if len(pos) else 0   # minloc, 1-based; 0 if the mask is empty
    return max(first - 1, 1)


def temperature(em, x):
    nt = len(em)
    i = locate(em, x)
    if i <= 0:
        return 1.0
    if i >= nt:
        return float(nt)
    return i + (x - em[i - 1]) * 1.0 / (em[i] - em[i - 1])


def dust_temperatures(absorbed, em_table, grain_weight, hit):
    """absorbed [nsizes, Nc+1] -> tdust [nsizes+1, Nc+1] (row 0 the weighted mean)."""
    ns, nc1 = absorbed.shape
    out = np.zeros((ns + 1, nc1))
    for c in range(1, nc1):
        if not hit[c]:
            continue
        for k in range(ns):
            out[1 + k, c] = temperature(em_table[k], absorbed[k, c])
        out[0, c] = float(np.dot(grain_weight, out[1:, c]))
    return out
