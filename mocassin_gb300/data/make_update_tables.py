"""Generates ``update_tables.npz``: the atomic data of the cell update
(ionisation and thermal balance) for the elements of the benchmark
abundance sets (H, He, C, N, O, Ne, S).

This script runs where the reference's data files are available and is the
only place that reads them; the table it writes is committed, so nothing at
run time needs the reference tree.  It follows the reference's readers:

* radiative recombination fits, ``radRecFit`` reading ``data/radrec.dat``
  (source/update_mod.f90:1674-1780): power laws ``rrec(2, z, n)`` and the
  Verner & Ferland (1996) fits ``rnew(4, z, n)``, in the file's loop order;
* dielectronic recombination, ``readData`` reading ``data/dielectronic.dat``
  (Nussbaumer & Storey fits, 25 rows) and ``data/aldrovandi.dat``
  (Aldrovandi & Pequignot 1973, 167 rows), source/readdata_mod.f90:90-118;
* collisionally excited line data, ``makeElements`` reading
  ``data/fileNames.dat`` and one file per ion (source/hydro_mod.f90:474-664):
  levels, temperatures, effective collision strengths (``iRats = 0``
  format), transition probabilities, statistical weights, level energies
  [1/cm] and the recombination-fit line ``br, z, a_r(4), a_d(5)`` (the last
  line read wins, as in the reader).

Usage: python make_update_tables.py <reference data dir> [out.npz]
"""
import os
import sys

import numpy as np

ELEMENTS = (1, 2, 6, 7, 8, 10, 16)
NSTAGES = 7         # set_input_mod.f90:76
NFORLEVELS = 17     # constants_mod.f90:48
NTMAX = 32


class ListReader:
    """Fortran list-directed input over the records of a text file."""

    def __init__(self, path):
        with open(path) as fh:
            self.lines = fh.read().splitlines()
        self.pos = 0

    def eof(self):
        return self.pos >= len(self.lines)

    def record(self):
        if self.eof():
            raise EOFError
        line = self.lines[self.pos]
        self.pos += 1
        return line

    def items(self, n):
        out = []
        while len(out) < n:
            toks = self.record().replace(",", " ").split()
            out.extend(toks)
        return out[:n]

    def floats(self, n):
        return [float(t.replace("d", "e").replace("D", "e")) for t in self.items(n)]

    def ints(self, n):
        return [int(float(t)) for t in self.items(n)]


def read_radrec(path):
    """rrec[i, z, n] (i < 2) and rnew[i, z, n] (i < 4), 1-based z and n."""
    r = ListReader(path)
    rrec = np.zeros((2, 31, 31))
    rnew = np.zeros((4, 31, 31))
    for n in range(4, 31):
        if n == 11:
            continue
        for z in range(n, 31):
            if z != 26 or n >= 14:
                rrec[:, z, n] = r.floats(2)
    for n in range(1, 4):
        for z in range(n, 31):
            rnew[:, z, n] = r.floats(4)
    for z in range(11, 31):
        rnew[:, z, 11] = r.floats(4)
    for n in range(4, 11):
        for z in range(max(6, n), 9):
            rnew[:, z, n] = r.floats(4)
        rnew[:, 10, n] = r.floats(4)
    for n in range(12, 27):
        rnew[:, 26, n] = r.floats(4)
    return rrec, rnew


def read_rows(path, nmax, ncol):
    rows = []
    r = ListReader(path)
    for _ in range(nmax):
        try:
            rows.append(r.floats(ncol))
        except EOFError:
            break
    return np.array(rows, dtype=np.float64)


def file_names(data_dir):
    """dataFile(elem, ion) for elem 3..30, ion 1..min(elem+1, 10) (hydro_mod.f90:500-505)."""
    r = ListReader(os.path.join(data_dir, "fileNames.dat"))
    names = {}
    for elem in range(3, 31):
        for ion in range(1, min(elem + 1, 10) + 1):
            names[(elem, ion)] = r.record()[:20].strip()
    return names


def read_cel(path):
    r = ListReader(path)
    ncoms = r.ints(1)[0]
    for _ in range(ncoms):
        r.record()
    nlev, ntemp = r.ints(2)
    for _ in range(nlev):
        r.record()
    logt = np.log10(np.array([r.floats(1)[0] for _ in range(ntemp)]))
    irats = r.floats(1)[0]
    if irats != 0:
        raise ValueError("%s: only the iRats = 0 format is used by these elements" % path)
    qom = np.zeros((ntemp, nlev + 1, nlev + 1))
    lo_prev = up_prev = 0
    k = 0
    while True:
        lo, up, qx = r.floats(3)
        lo, up = int(lo), int(up)
        if qx == 0.0:
            break
        if lo == 0:
            lo = lo_prev
            k += 1
        else:
            lo_prev = lo
            k = 1
        if up == 0:
            up = up_prev
        else:
            up_prev = up
        qom[k - 1, lo, up] = qx
    a = np.zeros((nlev + 1, nlev + 1))
    for kk in range(1, nlev):
        for _ in range(kk + 1, nlev + 1):
            i, j, ax = r.floats(3)
            a[int(j), int(i)] = ax
    g = np.zeros(nlev + 1)
    e = np.zeros(nlev + 1)
    for _ in range(nlev):
        i, gx, ex = r.floats(3)
        g[int(i)] = int(gx)
        e[int(i)] = ex
    br, z, a_r, a_d = 0.0, 0.0, np.zeros(4), np.zeros(5)
    for _ in range(2, nlev + 1):
        try:
            v = r.floats(11)
        except EOFError:
            break
        br, z, a_r, a_d = v[0], v[1], np.array(v[2:6]), np.array(v[6:11])
    return dict(nlev=nlev, ntemp=ntemp, logt=logt, qom=qom, a=a, g=g, e=e, br=br, z=z, a_r=a_r, a_d=a_d)


def main(data_dir, out):
    rrec, rnew = read_radrec(os.path.join(data_dir, "radrec.dat"))
    direc = read_rows(os.path.join(data_dir, "dielectronic.dat"), 25, 8)
    aldro = read_rows(os.path.join(data_dir, "aldrovandi.dat"), 167, 6)
    names = file_names(data_dir)
    keys, cels = [], []
    for elem in ELEMENTS:
        if elem < 3:
            continue
        for ion in range(1, min(elem + 1, NSTAGES) + 1):
            rel = names[(elem, ion)]
            path = os.path.join(data_dir, os.path.basename(rel))
            if not os.path.exists(path):
                continue
            c = read_cel(path)
            if c["nlev"] > NFORLEVELS:
                raise ValueError("%s has more than %d levels" % (path, NFORLEVELS))
            keys.append((elem, ion))
            cels.append(c)
    m = len(cels)
    L = NFORLEVELS + 1
    t = dict(
        rrec=rrec, rnew=rnew, direc=direc, aldro=aldro,
        cel_key=np.array(keys, dtype=np.int32), cel_nlev=np.array([c["nlev"] for c in cels], dtype=np.int32),
        cel_ntemp=np.array([c["ntemp"] for c in cels], dtype=np.int32),
        cel_logt=np.zeros((m, NTMAX)), cel_qom=np.zeros((m, NTMAX, L, L)), cel_a=np.zeros((m, L, L)),
        cel_g=np.zeros((m, L)), cel_e=np.zeros((m, L)), cel_br=np.array([c["br"] for c in cels]),
        cel_z=np.array([c["z"] for c in cels]), cel_ar=np.array([c["a_r"] for c in cels]),
        cel_ad=np.array([c["a_d"] for c in cels]))
    for i, c in enumerate(cels):
        n, nt = c["nlev"], c["ntemp"]
        t["cel_logt"][i, :nt] = c["logt"]
        t["cel_qom"][i, :nt, :n + 1, :n + 1] = c["qom"]
        t["cel_a"][i, :n + 1, :n + 1] = c["a"]
        t["cel_g"][i, :n + 1] = c["g"]
        t["cel_e"][i, :n + 1] = c["e"]
    np.savez_compressed(out, **t)
    print("wrote", out, "with", m, "line-cooling ions:", keys)


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    main(sys.argv[1], sys.argv[2] if len(sys.argv) > 2 else os.path.join(here, "update_tables.npz"))
