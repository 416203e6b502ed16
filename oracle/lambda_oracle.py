"""CPU oracle of the Lambda iteration (test infrastructure only).

iterateMC (source/iteration_mod.f90:33-1140) restated from the oracle's
pieces, all in FP64 on the host:

  1. the transport of every star: mc_oracle.cpp (photon_mod.f90), from the
     current opacity, recPDF rows and totalLines;
  2. the photoionisation and heating sums of every cell from Jste x 1e-9
     (/ 8 in a symmetric octant; iteration_mod.f90:705-724,
     update_mod.f90:175-269 and :1120-1217): update_runner.sums;
  3. updateCell of every cell (update_mod.f90:15-525): update_oracle.cpp,
     with the per-cell convergence flag |dX(H0)/X(H0)| <= XHILimit;
  4. the opacity of the next transport from the new ion densities
     (ionizationDriver / addOpacity, ionization_mod.f90:26-484):
     opacity_oracle.opacity on den(k, cell) = X(e_k, s_k) abund(e_k) Hden;
  5. the re-emission CDFs and line fractions of the next transport
     (emissionDriver / setDiffusePDF, emission_mod.f90:32-1311):
     emission_oracle.diffuse_pdf with the forbidden-line totals of
     update_runner.forbidden_lines.

Line fluxes follow outputGas (source/output_mod.f90:455-520): per line ion
the volume emissivity sum over cells of forbiddenLines x Hden x dV, next to
the H-beta volume emissivity HIRecLines(4,2) x Hden x dV (the recombination
emissivity of emission_oracle is not split into lines, so the ratios here
are relative to the total H recombination-line emission of each cell).
Gas-only grids; parity unpinned like its pieces (no reference outputs).
"""
import dataclasses

import numpy as np

from mocassin_gb300 import balance, nebula
from oracle import emission_oracle, opacity_oracle, runner, update_runner


def species_density(X, abund, hden, ions):
    """den [K][Nc+1]: X(e_k, s_k) abund(e_k) Hden(cell), row 0 (the sink) zero."""
    den = np.zeros((len(ions), len(hden)))
    for k, (z, st) in enumerate(ions):
        e = balance.ELEMENTS.index(z)
        den[k] = X[:, e, st] * abund[e] * hden
    den[:, 0] = 0.0
    return den


def cell_volumes(neb):
    """dV [1e45 cm^3] of every active cell row (photon_mod.f90:1469-1512)."""
    sym = bool(neb.flags & nebula.FLAG_SYMMETRIC_XYZ)

    def widths(ax):
        a = ax.astype(np.float64)
        n = len(a)
        w = np.empty(n)
        for p in range(n):
            if 0 < p < n - 1:
                w[p] = abs(a[p + 1] - a[p - 1]) / 2
            elif p == 0:
                w[p] = abs(a[1] - a[0]) / (2 if sym else 1)
            else:
                w[p] = abs(a[p] - a[p - 1])
        return w / 1e15

    wx, wy, wz = widths(neb.x_axis), widths(neb.y_axis), widths(neb.z_axis)
    vol = np.zeros(neb.ncells + 1)
    zz, yy, xx = np.nonzero(neb.active)
    vol[neb.active[zz, yy, xx]] = wx[xx] * wy[yy] * wz[zz]
    return vol


def line_luminosities(neb, te, ne, X, tables=None):
    """Per line ion, sum over active cells of the forbidden-line emissivity
    [1e-25 erg/s per H, update_runner.forbidden_lines] x Hden x dV."""
    tab = balance.tables() if tables is None else tables
    ab = balance.abundances()
    rows = np.arange(1, neb.ncells + 1)
    forb = update_runner.forbidden_lines(tab, ab, te[rows], ne[rows], X[rows])
    w = neb.hden.astype(np.float64)[rows] * cell_volumes(neb)[rows]
    return (forb * w[:, None]).sum(0)


class OracleLambda:
    """A gas-only nebula and its cell state, iterated on the host."""

    def __init__(self, neb, xhi_limit=0.05, threads=0):
        if neb.flags & nebula.FLAG_DUST:
            raise ValueError("the oracle Lambda iteration is gas-only")
        self.neb = dataclasses.replace(neb)
        self.xhi = xhi_limit
        self.threads = threads
        self.tables = balance.tables()
        self.ab = balance.abundances()
        self.ions = [tuple(int(v) for v in r) for r in nebula.atomic_table()["ions"]]
        self.hden = neb.hden.astype(np.float64)
        self.te, self.ne, self.X = balance.initial_state(neb)
        self.scale = 1e-9 / (8.0 if neb.flags & nebula.FLAG_SYMMETRIC_XYZ else 1.0)
        self.history = []
        self._emission()

    def _emission(self):
        """recPDF rows and totalLines of the next transport from the state."""
        n = self.neb
        rows = np.arange(1, n.ncells + 1)
        forb = update_runner.forbidden_lines(self.tables, self.ab, self.te[rows], self.ne[rows], self.X[rows])
        cdf, tl = emission_oracle.diffuse_pdf(self.te[rows], self.ne[rows], self.X[rows], self.ab, forb,
                                              nu=n.nu, xs=n.xs, ions=self.ions)
        rec = np.ones((n.nbins, n.ncells + 1), dtype=np.float32)   # Fortran layout (nbins, Nc+1)
        rec[:, 1:] = cdf.T.astype(np.float32)
        tot = np.zeros(n.ncells + 1, dtype=np.float32)
        tot[1:] = tl.astype(np.float32)
        n.rec_pdf = rec
        n.total_lines = tot

    def _opacity(self):
        den = species_density(self.X, self.ab, self.hden, self.ions)
        self.neb.opacity = opacity_oracle.opacity(den, self.neb.xs).astype(np.float32)

    def step(self, seed, iteration=None):
        it = len(self.history) + 1 if iteration is None else iteration
        js, _, _, st = runner.run(self.neb, precision="fp64", seed=seed, iteration=it, threads=self.threads)
        photo, heat, hit = update_runner.sums(js, self.neb.xs, self.neb.nu, self.ions, self.scale)
        te, ne, X, conv, niter, flags = update_runner.update_cells(self.tables, self.ab, self.hden, photo, heat, hit,
                                                                   self.te, self.ne, self.X, xhi_limit=self.xhi,
                                                                   threads=self.threads)
        self.te, self.ne, self.X = te, ne, X
        nhit = int(hit[1:].sum())
        rec = {"iteration": it, "crossings": st["crossings"], "hit": nhit,
               "converged_pct": 100.0 * float(conv[1:][hit[1:] > 0].sum()) / max(nhit, 1)}
        self._opacity()
        self._emission()
        self.history.append(rec)
        return rec
