"""Generates ``emission_tables.npz``: the data of the diffuse-emission CDF
(setDiffusePDF and the routines it calls, source/emission_mod.f90:32-1311).

This script runs where the reference's data files are available and is the
only place that reads them; the table it writes is committed, so nothing at
run time needs the reference tree.  It reads, in the reference's record order
(Fortran list-directed input):

* ``data/gammaHI.dat``, ``gammaHeI.dat``, ``gammaHeII.dat``: the f-b + f-f
  emission coefficients below the series limits on a temperature grid
  (initGammaCont, source/ph_mod.f90:40-199; positive values stored as log10,
  the others as 0);
* ``data/HeI2phot.dat``: the HeI 2^1S two-photon distribution (41 records,
  readData, source/readdata_mod.f90:38-48);
* ``data/r1b0100.dat``, ``r2a0100.dat``, ``r2b0100.dat``: the HI Balmer-and-up
  line ratios, the HeII Lyman lines and the HeII line ratios of Storey &
  Hummer (1995) (readdata_mod.f90:50-92);
* ``data/HeIrecLines.dat``: the HeI recombination-line fits of Benjamin,
  Skillman & Smits (1999), 34 lines at 3 densities, the first coefficient
  scaled by 1e25 (readHeIRecLines, source/hydro_mod.f90:184-203);
* the 8 x 11 Chebyshev coefficients of Hummer's (1988, ApJ 327, 477)
  thermally averaged free-free Gaunt factor from the ``dd`` table of
  getGauntFF (source/ionization_mod.f90:193-330);
* for the heavy ions that recombine in gammaHeavies (C, N, O, Ne, S, stages
  1..6; fb_ff, emission_mod.f90:477-527): the outer shell and the
  statistical weights of getOuterShell (hydro_mod.f90:89-182), the outer
  shell's threshold and its upper limit (setShells / limitShell,
  hydro_mod.f90:208-330), and its partial cross-section on the frequency
  grid of ``atomic_table.npz`` (makeOpacity, ph_mod.f90:744-803, with the
  Verner fits of make_atomic_table).

Usage: python make_emission_tables.py <reference source dir> <reference data dir> [out.npz]
"""
import os
import re
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import make_atomic_table as mat  # noqa: E402

f32 = np.float32
HEAVY = (6, 7, 8, 10, 16)
SS = (1, 1, 2, 2, 3, 3, 3, 3, 3, 3, 4, 4, 5, 5, 5, 5, 5, 5, 6, 6, 6, 6, 6, 6, 6, 6, 6, 6, 7, 7)
GL = (2, 1, 2, 1, 6, 9, 4, 9, 6, 1, 2, 1, 6, 9, 4, 9, 6, 1, 2, 1, 10, 21, 28, 7, 6, 25, 28, 21, 2, 1)


class ListReader:
    """Fortran list-directed input: each read starts at the next record and
    takes values from as many records as it needs; the rest of its last
    record is skipped.  Commas and blanks separate values."""

    def __init__(self, path):
        with open(path) as fh:
            self.lines = fh.read().splitlines()
        self.pos = 0

    def read(self, n):
        out = []
        while len(out) < n:
            out.extend(t for t in re.split(r"[,\s]+", self.lines[self.pos].strip()) if t)
            self.pos += 1
        return [float(v) for v in out[:n]]


def read_gamma(path):
    r = ListReader(path)
    ntk, nlim = (int(v) for v in r.read(2))
    tk = np.array(r.read(ntk), dtype=f32)
    nu = np.zeros(nlim, dtype=f32)
    lg = np.zeros((ntk, nlim), dtype=f32)
    for i in range(nlim):
        v = r.read(1 + ntk)
        nu[i] = f32(v[0])
        g = np.array(v[1:], dtype=f32)
        lg[:, i] = np.where(g > 0, np.log10(np.where(g > 0, g, f32(1))), f32(0)).astype(f32)
    return tk, nu, lg


def read_gaunt_dd(src_dir):
    with open(os.path.join(src_dir, "ionization_mod.f90")) as fh:
        text = fh.read()
    start = text.index("subroutine getGauntFF")
    block = text[text.index("dd = (/", start):]
    block = block[: block.index("/)")]
    vals = re.findall(r"[-+]?\d+\.\d+e[-+]\d+", block)
    assert len(vals) == 88, len(vals)
    return np.array([float(v) for v in vals], dtype=np.float64)


def heavy_shells(nu):
    """Outer shell of every recombining heavy ion and its partial
    cross-section on the grid (zero outside [IPnuP, highNuP])."""
    data_dir = os.environ["MC_REF_DATA"]
    ph1, ph2 = mat.read_ph(data_dir)
    nb = len(nu)
    k_shell_p = mat_locate(nu, f32(7.35e4))
    rows = []
    xs = []
    for z in HEAVY:
        for ion in range(1, 7):
            if ion > z:
                break
            ne = z - ion + 1
            out = SS[ne - 1]
            g0 = GL[ne - 1]
            g1 = 1 if ne == 1 else GL[ne - 2]
            lo = np.zeros(8, dtype=np.int64)
            for shell in range(1, out + 1):
                thres = f32(ph1[(z, ne, shell)][0]) / mat.RYD_TO_EV
                lo[shell] = 2 if thres <= f32(0.1) else mat_locate(nu, thres)
            thres_out = f32(ph1[(z, ne, out)][0]) / mat.RYD_TO_EV
            if out <= 3:
                hi = k_shell_p
            elif out <= 6:
                hi = lo[1] - 1
            else:
                hi = (lo[5] if lo[6] < 3 else lo[6]) - 1
            ip = mat_locate(nu, thres_out)
            row = np.zeros(nb, dtype=f32)
            for i in range(ip, hi + 1):
                e = max(f32(nu[i - 1]) * mat.RYD_TO_EV, f32(ph1[(z, ne, out)][0]))
                row[i - 1] = f32(mat.ph_fit_el(ph1, ph2, z, ne, out, e) * f32(1e-18))
            rows.append((z, ion, ne, out, g0, g1, ip, hi))
            xs.append(row)
    return np.array(rows, dtype=np.int32), np.array(xs, dtype=f32)


def mat_locate(xa, x):
    """locate (interpolation_mod.f90:48-81), 1-based."""
    x = f32(x)
    n = len(xa)
    if x > xa[n - 1]:
        return n
    if x < xa[0]:
        return 0
    above = np.nonzero(xa - x > 0)[0]
    if len(above) == 0:
        return 1
    return max(int(above[np.argmin((xa - x)[above])]) + 1 - 1, 1)


def main():
    src_dir, data_dir = sys.argv[1], sys.argv[2]
    os.environ["MC_REF_DATA"] = data_dir
    here = os.path.dirname(os.path.abspath(__file__))
    out = sys.argv[3] if len(sys.argv) > 3 else os.path.join(here, "emission_tables.npz")
    nu = np.load(os.path.join(here, "atomic_table.npz"))["nu"]
    tk, nu_hi, lg_hi = read_gamma(os.path.join(data_dir, "gammaHI.dat"))
    tk2, nu_hei, lg_hei = read_gamma(os.path.join(data_dir, "gammaHeI.dat"))
    tk3, nu_heii, lg_heii = read_gamma(os.path.join(data_dir, "gammaHeII.dat"))
    assert np.array_equal(tk, tk2) and np.array_equal(tk, tk3)
    r = ListReader(os.path.join(data_dir, "HeI2phot.dat"))
    y_ay = np.array([r.read(2) for _ in range(41)], dtype=f32)
    r = ListReader(os.path.join(data_dir, "r1b0100.dat"))
    hi_rec = np.zeros((16, 9), dtype=f32)  # [iup][ilow]
    for iup in range(15, 2, -1):
        hi_rec[iup, 2:min(8, iup - 1) + 1] = r.read(min(8, iup - 1) - 1)
    r = ListReader(os.path.join(data_dir, "r2a0100.dat"))
    lyman = np.array([r.read(2) for _ in range(4)], dtype=f32)  # data, nu
    r = ListReader(os.path.join(data_dir, "r2b0100.dat"))
    heii_rec = np.zeros((31, 17), dtype=f32)
    for iup in range(30, 2, -1):
        heii_rec[iup, 2:min(16, iup - 1) + 1] = r.read(min(16, iup - 1) - 1)
    r = ListReader(os.path.join(data_dir, "HeIrecLines.dat"))
    hei = np.zeros((34, 3, 4), dtype=f32)
    for iden in range(3):
        for line in range(34):
            v = r.read(4)
            hei[line, iden] = v
            hei[line, iden, 0] = f32(v[0]) * f32(1e25)
    dd = read_gaunt_dd(src_dir)
    shells, xs_outer = heavy_shells(nu)
    np.savez_compressed(out, tk=tk, nu_gamma_hi=nu_hi, lg_hi=lg_hi, nu_gamma_hei=nu_hei, lg_hei=lg_hei,
                        nu_gamma_heii=nu_heii, lg_heii=lg_heii, y_ay=y_ay, hi_rec=hi_rec, heii_lyman=lyman,
                        heii_rec=heii_rec, hei_rec=hei, gaunt_dd=dd, shells=shells, xs_outer=xs_outer, nu=nu)
    print("wrote", out, "gamma limits", len(nu_hi), len(nu_hei), len(nu_heii), "heavy ions", len(shells))


if __name__ == "__main__":
    main()
