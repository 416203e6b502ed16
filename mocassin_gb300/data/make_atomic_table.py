"""Generates ``atomic_table.npz``: the frequency grid and the per-ion
photoionisation cross-section matrix XS[ion, nu] used to build synthetic
nebulae.

This script runs where the reference's data files are available and is the
only place that reads them; the table it writes is committed, so nothing at
run time needs the reference tree.  It restates (in numpy, FP32 like the
Fortran ``real``):

* ``phInit`` reading order of ``data/ph1.dat`` / ``data/ph2.dat``
  (source/ph_mod.f90:408-472),
* ``phFitEl``, the Verner et al. (1996, ApJ 465, 487) / Verner & Yakovlev
  (1995, A&AS 109, 125) partial cross-section fits (source/ph_mod.f90:477-559),
* ``getOuterShell`` (source/hydro_mod.f90:89-182),
* the ionisation-edge list and the frequency-grid builder of
  ``initCartesianGrid`` for a gas-only grid (source/grid_mod.f90:128-258,
  :331-336).

XS[ion, nu] is the shell-summed cross-section [cm^2] of each ion with bound
electrons (H0; He0, He+; C0..C5+; N, O, Ne, S 0..6+ at nstages = 7), the dense
matrix whose contraction with the per-cell ion densities gives the bound-free
opacity of addOpacity (source/ionization_mod.f90:396-482).  It is a synthetic
input: mocassin's own xSecArray additionally uses hydrogenic fits for H and
He (ph_mod.f90:204-402), which this table does not reproduce.

Usage: python make_atomic_table.py <reference data dir> [out.npz]
"""
import os
import sys

import numpy as np

f32 = np.float32
RYD_TO_EV = f32(13.6056981)  # constants_mod.f90:31
NSTAGES = 7                  # set_input_mod.f90:76
# H, He, C, N, O, Ne, S: the elements of the benchmark abundance sets
ELEMENTS = (1, 2, 6, 7, 8, 10, 16)

N_TOT = (1, 1, 2, 2, 3, 3, 3, 3, 3, 3, 4, 4, 5, 5, 5, 5, 5, 5, 6, 6, 6, 6, 6, 6, 6, 6, 6, 6, 7, 7)
N_INN = (0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 3, 3, 3, 3, 3, 3, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5, 5)
LEVEL = (0, 0, 1, 0, 1, 2, 0)
SERIES_EDGE = (0.0069, 0.0083, 0.01, 0.0123, 0.0156, 0.0204, 0.0278, 0.04, 0.0625, 0.11117,
               0.11610, 0.12248, 0.13732, 0.24763, 0.24994, 0.26630, 0.29189)
RADIO_4P9GHZ = f32(1.489434e-6)


def read_ph(data_dir):
    """ph1[nz][ne][shell] -> 6 params, ph2[nz][ne] -> 7 params (1-based keys)."""
    with open(os.path.join(data_dir, "ph1.dat")) as fh:
        rows1 = [list(map(float, ln.split())) for ln in fh if ln.strip()]
    with open(os.path.join(data_dir, "ph2.dat")) as fh:
        rows2 = [list(map(float, ln.split())) for ln in fh if ln.strip()]
    ph1, it = {}, iter(rows1)
    for j in range(1, 31):
        for k in range(1, min(j, 30) + 1):
            nt = N_TOT[k - 1]
            if j == k and k > 18:
                nt = 7
            if j == k + 1 and j in (20, 21, 22, 25, 26):
                nt = 7
            for l in range(1, nt + 1):
                ph1[(j, k, l)] = [f32(v) for v in next(it)]
    ph2, it = {}, iter(rows2)
    for k in range(1, 31):
        for j in range(1, min(k, 30) + 1):
            if k not in (15, 17, 19) and (k <= 20 or k == 26):
                ph2[(k, j)] = [f32(v) for v in next(it)]
    return ph1, ph2


def n_out_shell(nz, ne):
    n_out = N_TOT[ne - 1]
    if nz == ne and nz > 18:
        n_out = 7
    if nz == ne + 1 and nz in (20, 21, 22, 25, 26):
        n_out = 7
    return n_out


def ph_fit_el(ph1, ph2, nz, ne, shell, e_ev):
    """Partial cross-section [Mb] of shell `shell` of ion (nz, ne) at e_ev [eV]."""
    e = f32(e_ev)
    if nz < 1 or nz > 30 or ne < 1 or ne > nz:
        return f32(0)
    n_out = n_out_shell(nz, ne)
    if shell > n_out:
        return f32(0)
    p = ph1[(nz, ne, shell)]
    if e < p[0]:
        return f32(0)
    n_int = N_INN[ne - 1]
    if nz in (15, 17, 19) or (nz > 20 and nz != 26):
        e_inn = f32(0)
    else:
        e_inn = f32(1e30) if ne < 3 else ph1[(nz, ne, n_int)][0]
    if shell < n_out and shell > n_int and e < e_inn:
        return f32(0)
    if shell <= n_int or e >= e_inn:
        p1 = -p[4]
        y = e / p[1]
        q = f32(-0.5) * p1 - f32(LEVEL[shell - 1]) - f32(5.5)
        a = p[2] * ((y - f32(1)) ** 2 + p[5] ** 2)
        b = np.sqrt(y / p[3]) + f32(1)
        return f32(a * y ** q * b ** p1)
    c = ph2[(nz, ne)]
    p1 = -c[3]
    q = f32(-0.5) * p1 - f32(5.5)
    x = e / c[0] - c[5]
    z = np.sqrt(x * x + c[6] * c[6])
    a = c[1] * ((x - f32(1)) * (x - f32(1)) + c[4] * c[4])
    b = np.sqrt(z / c[2]) + f32(1)
    return f32(a * z ** q * b ** p1)


def ion_edges(ph1, nu_max):
    """ionEdge(1:nEdges), sorted (grid_mod.f90:136-176)."""
    edges = []
    for elem in ELEMENTS:
        for ion in range(1, min(elem, NSTAGES - 1) + 1):
            if elem > 2:
                ne = elem - ion + 1
                out = N_TOT[ne - 1]
                if elem == ne and elem > 18:
                    out = 7
                if elem == ne + 1 and elem in (20, 21, 22, 25, 26):
                    out = 7
                e = ph1[(elem, ne, out)][0] / RYD_TO_EV
            elif elem == 1:
                e = f32(0.999434)
            elif ion == 1:
                e = f32(1.80804)
            else:
                e = f32(4.0)
            if e <= f32(nu_max):
                edges.append(f32(e))
    return np.sort(np.array(edges, dtype=f32))


def nu_grid(edges, nbins, nu_min, nu_max):
    """Gas-only frequency grid of initCartesianGrid (grid_mod.f90:212-258)."""
    nu = np.zeros(nbins, dtype=f32)
    if f32(nu_min) < RADIO_4P9GHZ:
        nu[0] = RADIO_4P9GHZ
        cnt = 2
    else:
        cnt = 1
    nu_min_a, nu_max_a = f32(nu_min), f32(nu_max)
    for se in SERIES_EDGE:
        se = f32(se)
        nu[cnt - 1] = se
        nu[cnt] = se - f32(0.0003)
        nu[cnt + 1] = se + f32(0.0003)
        if se < nu_min_a:
            nu_min_a = se - f32(0.0006)
        if se > nu_max_a:
            nu_max_a = se
        cnt += 3
    for e in edges:
        if e < nu_max_a:
            nu[cnt - 1] = e
            nu[cnt] = e - f32(0.0003)
            nu[cnt + 1] = e + f32(0.0003)
            if e < nu_min_a:
                nu_min_a = e - f32(0.0006)
            cnt += 3
    icount = nbins - cnt + 1
    step = (np.log10(nu_max_a) - np.log10(nu_min_a)) / f32(icount - 1)
    nu[cnt - 1] = nu_min_a
    for i in range(cnt, nbins):
        nu[i] = f32(10.0) ** (np.log10(nu[i - 1]) + step)
    return np.sort(nu)


def main():
    data_dir = sys.argv[1]
    out = sys.argv[2] if len(sys.argv) > 2 else os.path.join(os.path.dirname(__file__), "atomic_table.npz")
    nbins, nu_min, nu_max = 600, 1.0e-5, 24.5
    ph1, ph2 = read_ph(data_dir)
    edges = ion_edges(ph1, nu_max)
    nu = nu_grid(edges, nbins, nu_min, nu_max)
    ions = []
    for elem in ELEMENTS:
        for stage in range(1, min(elem, NSTAGES) + 1):
            ions.append((elem, stage))
    xs = np.zeros((len(ions), nbins), dtype=f32)
    for i, (z, stage) in enumerate(ions):
        ne = z - stage + 1
        for k in range(nbins):
            e_ev = nu[k] * RYD_TO_EV
            tot = f32(0)
            for shell in range(1, n_out_shell(z, ne) + 1):
                tot += ph_fit_el(ph1, ph2, z, ne, shell, e_ev)
            xs[i, k] = tot * f32(1e-18)
    np.savez_compressed(out, nu=nu, xs=xs, ions=np.array(ions, dtype=np.int32),
                        edges=edges, nbins=nbins, nu_min=nu_min, nu_max=nu_max)
    print("wrote", out, "ions", len(ions), "edges", len(edges), "ionEdge(1)", edges[0])


if __name__ == "__main__":
    main()
