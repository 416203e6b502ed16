"""Grid snapshots in the reference's output files, for warm restarts.

writeGrid (source/grid_mod.f90:2646-2779) writes, for the mother grid,
  output/grid0.out  nGrids; nx ny nz nCells motherP R_out; the x, y, z axes
                    (one value per line); then per cell, x outer and z inner:
                    active lgConverged lgBlack
  output/grid1.out  per cell (same order, row 0 for inactive cells): Te Ne Hden
  output/grid2.out  per cell and element (H, He, C, N, O, Ne, S here): the
                    min(elem+1, nstages) ionic fractions on one line
  output/dustGrid.out  per cell: Ndust, then for sizes 0..nSizes a line of
                    Tdust(species 0..nSpeciesMax)
and resetGrid (:2967-3567) reads them back in the same order to restart a
model.  write_grid takes the state of a TransportContext (downloaded from
the GPU by get_cell_state / dust_temperatures) and writes these files with
Fortran list-directed formatting; read_grid reads them the way resetGrid
does.  Together they move a model between this code and the Fortran one.
"""
import os

import numpy as np

from . import balance

NSTAGES = 7


def _f(x):
    return "%16.8E" % float(x)


def write_grid(path, neb, te, ne, X, conv=None, black=None, tdust=None, ndust=None, r_out=None):
    """Writes grid0.out, grid1.out, grid2.out (and dustGrid.out when tdust is
    given: shape (nSizes+1, Nc+1), one species) into ``path``."""
    os.makedirs(path, exist_ok=True)
    nc1 = neb.ncells + 1
    conv = np.zeros(nc1, dtype=np.int32) if conv is None else np.asarray(conv)
    black = np.zeros(nc1, dtype=np.int32) if black is None else np.asarray(black)
    rout = neb.r_out if r_out is None else r_out
    act = neb.active  # (z, y, x)
    hden = neb.hden
    with open(os.path.join(path, "grid0.out"), "w") as g0, open(os.path.join(path, "grid1.out"), "w") as g1, \
            open(os.path.join(path, "grid2.out"), "w") as g2:
        g0.write("%12d\n" % 1)
        g0.write("%12d%12d%12d%12d%12d%s\n" % (neb.nx, neb.ny, neb.nz, neb.ncells, 0, _f(rout)))
        for ax in (neb.x_axis, neb.y_axis, neb.z_axis):
            for v in ax:
                g0.write(_f(v) + "\n")
        for i in range(neb.nx):
            for j in range(neb.ny):
                for k in range(neb.nz):
                    a = int(act[k, j, i])
                    c = max(a, 0)
                    g0.write("%12d%12d%12d\n" % (a, int(conv[c]), int(black[c])))
                    g1.write("%s%s%s\n" % (_f(te[c]), _f(ne[c]), _f(hden[c])))
                    for e, z in enumerate(balance.ELEMENTS):
                        ns = min(z + 1, NSTAGES)
                        g2.write("".join(_f(X[c, e, s]) for s in range(1, ns + 1)) + "\n")
    if tdust is not None:
        nd = np.zeros(nc1) if ndust is None else np.asarray(ndust)
        with open(os.path.join(path, "dustGrid.out"), "w") as gd:
            for i in range(neb.nx):
                for j in range(neb.ny):
                    for k in range(neb.nz):
                        c = max(int(act[k, j, i]), 0)
                        gd.write(_f(nd[c]) + "\n")
                        for ai in range(tdust.shape[0]):
                            # species 0 (the mix) and species 1 (the one species) carry the same value
                            gd.write("%s %s\n" % (_f(tdust[ai, c]), _f(tdust[ai, c])))


class _Reader:
    """Fortran list-directed input: each read takes the next record(s)."""

    def __init__(self, p):
        with open(p) as fh:
            self.lines = fh.read().splitlines()
        self.pos = 0

    def read(self, n):
        out = []
        while len(out) < n:
            out.extend(self.lines[self.pos].replace(",", " ").split())
            self.pos += 1
        return out[:n]


def read_grid(path, dust_sizes=None):
    """Reads the snapshot as resetGrid does; returns a dict with nx, ny, nz,
    ncells, r_out, the axes, active (z, y, x), conv, black, te, ne, hden,
    X (Nc+1, 7, 8) and, with dust_sizes, ndust and tdust (nSizes+1, Nc+1)."""
    r0 = _Reader(os.path.join(path, "grid0.out"))
    r1 = _Reader(os.path.join(path, "grid1.out"))
    r2 = _Reader(os.path.join(path, "grid2.out"))
    int(r0.read(1)[0])
    v = r0.read(6)
    nx, ny, nz, nc, _mother = (int(x) for x in v[:5])
    rout = float(v[5])
    ax = [np.array([float(r0.read(1)[0]) for _ in range(n)]) for n in (nx, ny, nz)]
    nc1 = nc + 1
    active = np.zeros((nz, ny, nx), dtype=np.int32)
    conv = np.zeros(nc1, dtype=np.int32)
    black = np.zeros(nc1, dtype=np.int32)
    te, ne, hden = np.zeros(nc1), np.zeros(nc1), np.zeros(nc1)
    X = np.zeros((nc1, len(balance.ELEMENTS), NSTAGES + 1))
    rd = _Reader(os.path.join(path, "dustGrid.out")) if dust_sizes else None
    ndust = np.zeros(nc1) if rd else None
    tdust = np.zeros((dust_sizes + 1, nc1)) if rd else None
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                a, p0, p00 = r0.read(3)
                c = max(int(a), 0)
                active[k, j, i] = int(a)
                conv[c] = int(round(float(p0)))
                black[c] = int(round(float(p00)))
                p1, p2, p3 = (float(x) for x in r1.read(3))
                te[c], ne[c], hden[c] = p1, p2, p3
                for e, z in enumerate(balance.ELEMENTS):
                    ns = min(z + 1, NSTAGES)
                    X[c, e, 1:ns + 1] = [float(x) for x in r2.read(ns)]
                if rd:
                    ndust[c] = float(rd.read(1)[0])
                    for ai in range(dust_sizes + 1):
                        tdust[ai, c] = float(rd.read(2)[0])
    out = {"nx": nx, "ny": ny, "nz": nz, "ncells": nc, "r_out": rout, "x_axis": ax[0], "y_axis": ax[1],
           "z_axis": ax[2], "active": active, "conv": conv, "black": black, "te": te, "ne": ne, "hden": hden, "X": X}
    if rd:
        out["ndust"], out["tdust"] = ndust, tdust
    return out
