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
  output/grid3.out  the model parameters, one record per line (:2800-2867)
  output/photoSource.out  the ionising sources (:2780-2797)
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


def _l(b):
    return "T" if b else "F"


def model_parameters(neb, xhi_limit=0.05, max_iterate=30, min_convergence=95.0):
    """The grid3.out parameters of a nebula built by mocassin_gb300.nebula:
    its own (grid, frequencies, dust, viewing angles, stars) and the
    reference's defaults for the driver's switches it does not use."""
    from . import nebula
    spec = neb.spec
    views = list(getattr(spec, "views", ()) or ())
    dust = bool(neb.flags & nebula.FLAG_DUST)
    return {"nGrids": 1, "convWriteGrid": 0.0, "lgAutoPackets": False, "convIncPercent": 0.0, "nPhotIncrease": 0,
            "maxPhotons": 0, "lgSymmetricXYZ": bool(neb.flags & nebula.FLAG_SYMMETRIC_XYZ), "lgTalk": False,
            "lg1D": False, "nbins": int(neb.nbins), "nuStepSize": 0.075, "nuMax": float(neb.nu[-1]),
            "nuMin": float(neb.nu[0]), "R_in": float(max(spec.r_in, 0.0)), "XHIlimit": float(xhi_limit),
            "maxIterateMC": int(max_iterate), "minConvergence": float(min_convergence), "lgDebug": False,
            "lgPlaneIonization": False, "abundanceFile": ["abundances.dat"], "lgOutput": True, "dxSlit": 0.0,
            "dySlit": 0.0, "lgDust": dust, "lgDustConstant": False, "lgMultiDustChemistry": False,
            "dustSpeciesFile": ["grains.dat"] if dust else ["none"], "dustFile2": "none",
            "lgGas": bool(neb.flags & nebula.FLAG_GAS), "lgRecombination": False,
            "nSpeciesMax": 1, "nSpecies": 1, "nSizes": 10 if dust else 1, "nSpeciesPart": [1],
            "resLinesTransfer": 101.0, "lgDustScattering": dust, "nAngleBins": len(views),
            "viewPointTheta": [0.0] + [float(v[0]) for v in views],
            "viewPointPhi": [0.0] + [float(v[1]) for v in views], "contCube": (-1.0, -1.0),
            "lgPhotoelectric": False, "lgTraceHeating": False, "Ldiffuse": 0.0, "Tdiffuse": 0.0,
            "shapeDiffuse": "none", "nPhotonsDiffuse": 0, "emittingGrid": 0, "nstages": 7,
            "lgMultistars": bool(neb.flags & nebula.FLAG_MULTISTARS), "lg2D": False, "lgEcho": False,
            "echot1": 0.0, "echot2": 0.0, "echoTemp": 0.0, "lgNosource": False,
            "stars": [(float(st.t_star), float(st.lum), int(st.n_packets), tuple(float(f) for f in st.frac_pos))
                      for st in spec.stars]}


def write_parameters(path, p):
    """grid3.out and photoSource.out in writeGrid's record order
    (grid_mod.f90:2780-2867), Fortran list-directed style.  writeGrid writes
    the viewing angles 0..nAngleBins; resetGrid reads 1..nAngleBins from the
    same records, so a restart shifts them by one (kept as the reference)."""
    os.makedirs(path, exist_ok=True)
    rec = []
    rec.append("%d" % p["nGrids"])
    rec.append("%s convWriteGrid" % _f(p["convWriteGrid"]))
    rec.append("%s %s %d %d lgAutoPackets" % (_l(p["lgAutoPackets"]), _f(p["convIncPercent"]), p["nPhotIncrease"],
                                              p["maxPhotons"]))
    for k in ("lgSymmetricXYZ", "lgTalk", "lg1D"):
        rec.append("%s %s" % (_l(p[k]), k))
    rec.append("%d nbins" % p["nbins"])
    for k in ("nuStepSize", "nuMax", "nuMin", "R_in", "XHIlimit"):
        rec.append("%s %s" % (_f(p[k]), k))
    rec.append("%d %s maxIterateMC" % (p["maxIterateMC"], _f(p["minConvergence"])))
    for k in ("lgDebug", "lgPlaneIonization"):
        rec.append("%s %s" % (_l(p[k]), k))
    rec.append("%d nAbComponents" % len(p["abundanceFile"]))
    rec.extend('"%s"' % f for f in p["abundanceFile"])
    rec.append("%s lgOutput" % _l(p["lgOutput"]))
    rec.append("%s %s dxSlit,dySlit" % (_f(p["dxSlit"]), _f(p["dySlit"])))
    rec.append("%s %s lgDust, lgDustConstant" % (_l(p["lgDust"]), _l(p["lgDustConstant"])))
    rec.append("%s %d lgMultiDustChemistry, nDustComponents" % (_l(p["lgMultiDustChemistry"]),
                                                                len(p["dustSpeciesFile"])))
    rec.extend('"%s" dustFile' % f for f in p["dustSpeciesFile"])
    rec.append('"%s" dustFile' % p["dustFile2"])
    for k in ("lgGas", "lgRecombination"):
        rec.append("%s %s" % (_l(p[k]), k))
    rec.append("%d %d %d nSpeciesMax, nSpecies, nSizes" % (p["nSpeciesMax"], p["nSpecies"], p["nSizes"]))
    rec.append(" ".join("%d" % v for v in p["nSpeciesPart"]) + " Partial nspecies")
    rec.append("%s resLinesTransfer" % _f(p["resLinesTransfer"]))
    rec.append("%s lgDustScattering" % _l(p["lgDustScattering"]))
    rec.append("%d nAngleBins" % p["nAngleBins"])
    if p["nAngleBins"] > 0:
        rec.append(" ".join(_f(v) for v in p["viewPointTheta"]) + " inclination theta")
        rec.append(" ".join(_f(v) for v in p["viewPointPhi"]) + " inclination theta")
    rec.append("%s %s continuumCube" % (_f(p["contCube"][0]), _f(p["contCube"][1])))
    for k in ("lgPhotoelectric", "lgTraceHeating"):
        rec.append("%s %s" % (_l(p[k]), k))
    rec.append("%s Ldiffuse" % _f(p["Ldiffuse"]))
    rec.append("%s Tdiffuse" % _f(p["Tdiffuse"]))
    rec.append("%s shapeDiffuse" % p["shapeDiffuse"])
    rec.append("%d nPhotonsDiffuse" % p["nPhotonsDiffuse"])
    rec.append("%d emittingGrid" % p["emittingGrid"])
    rec.append("%d emittingGrid" % p["nstages"])
    rec.append("%s lgMultiStars" % _l(p["lgMultistars"]))
    rec.append("%s 2D geometry?" % _l(p["lg2D"]))
    rec.append("%s %s %s %s Echo on/off" % (_l(p["lgEcho"]), _f(p["echot1"]), _f(p["echot2"]), _f(p["echoTemp"])))
    rec.append("%s NoSourceSED" % _l(p["lgNosource"]))
    with open(os.path.join(path, "grid3.out"), "w") as fh:
        fh.write("\n".join(" " + r for r in rec) + "\n")
    with open(os.path.join(path, "photoSource.out"), "w") as fh:
        fh.write(" %d number of photon sources\n" % len(p["stars"]))
        for t, lum, n, pos in p["stars"]:
            fh.write(" 'blackbody' %s %s %d %s %s %s star 0.0\n" % (_f(t), _f(lum), n, _f(pos[0]), _f(pos[1]),
                                                                     _f(pos[2])))
        fh.write(" (contShape, T_eff[K], L_* [E36 erg/s], nPackets, (x,y,z) position, spID, tstep)\n")


def read_parameters(path):
    """grid3.out as resetGrid reads it (grid_mod.f90:3028-3110): each read
    starts a new record and takes the values it lists."""
    r = _Reader(os.path.join(path, "grid3.out"))
    lg = lambda tok: tok.strip().upper().startswith("T") or tok.strip().upper().startswith(".T")
    p = {}
    p["nGrids"] = int(r.read(1)[0])
    p["convWriteGrid"] = float(r.read(1)[0])
    v = r.read(4)
    p["lgAutoPackets"], p["convIncPercent"], p["nPhotIncrease"], p["maxPhotons"] = lg(v[0]), float(v[1]), int(v[2]), \
        int(v[3])
    for k in ("lgSymmetricXYZ", "lgTalk", "lg1D"):
        p[k] = lg(r.read(1)[0])
    p["nbins"] = int(r.read(1)[0])
    for k in ("nuStepSize", "nuMax", "nuMin", "R_in", "XHIlimit"):
        p[k] = float(r.read(1)[0])
    v = r.read(2)
    p["maxIterateMC"], p["minConvergence"] = int(v[0]), float(v[1])
    for k in ("lgDebug", "lgPlaneIonization"):
        p[k] = lg(r.read(1)[0])
    nab = int(r.read(1)[0])
    p["abundanceFile"] = [r.read(1)[0].strip('"') for _ in range(nab)]
    p["lgOutput"] = lg(r.read(1)[0])
    v = r.read(2)
    p["dxSlit"], p["dySlit"] = float(v[0]), float(v[1])
    v = r.read(2)
    p["lgDust"], p["lgDustConstant"] = lg(v[0]), lg(v[1])
    v = r.read(2)
    p["lgMultiDustChemistry"], ndc = lg(v[0]), int(v[1])
    p["dustSpeciesFile"] = [r.read(1)[0].strip('"') for _ in range(ndc)]
    p["dustFile2"] = r.read(1)[0].strip('"')
    for k in ("lgGas", "lgRecombination"):
        p[k] = lg(r.read(1)[0])
    v = r.read(3)
    p["nSpeciesMax"], p["nSpecies"], p["nSizes"] = (int(x) for x in v)
    p["nSpeciesPart"] = [int(x) for x in r.read(ndc)]
    p["resLinesTransfer"] = float(r.read(1)[0])
    p["lgDustScattering"] = lg(r.read(1)[0])
    p["nAngleBins"] = int(r.read(1)[0])
    if p["nAngleBins"] > 0:
        na = p["nAngleBins"]
        p["viewPointTheta"] = [0.0] + [float(x) for x in r.read(na)]
        p["viewPointPhi"] = [0.0] + [float(x) for x in r.read(na)]
    v = r.read(2)
    p["contCube"] = (float(v[0]), float(v[1]))
    for k in ("lgPhotoelectric", "lgTraceHeating"):
        p[k] = lg(r.read(1)[0])
    p["Ldiffuse"] = float(r.read(1)[0])
    p["Tdiffuse"] = float(r.read(1)[0])
    p["shapeDiffuse"] = r.read(1)[0]
    p["nPhotonsDiffuse"] = int(r.read(1)[0])
    p["emittingGrid"] = int(r.read(1)[0])
    p["nstages"] = int(r.read(1)[0])
    p["lgMultistars"] = lg(r.read(1)[0])
    p["lg2D"] = lg(r.read(1)[0])
    v = r.read(4)
    p["lgEcho"], p["echot1"], p["echot2"], p["echoTemp"] = lg(v[0]), float(v[1]), float(v[2]), float(v[3])
    p["lgNosource"] = lg(r.read(1)[0])
    return p

