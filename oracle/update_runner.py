"""ctypes runner of the cell-update oracle (update_oracle.cpp): test
infrastructure only."""
import ctypes as C

import numpy as np

from oracle import build_oracle

_LIB = None
_dp, _ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
ELEMENTS = (1, 2, 6, 7, 8, 10, 16)
NSTAGES = 7
HCRYD = 2.1799153e-11


class UpdTables(C.Structure):
    _fields_ = [("rrec", _dp), ("rnew", _dp), ("direc", _dp), ("ndirec", C.c_int32), ("aldro", _dp),
                ("naldro", C.c_int32), ("ncel", C.c_int32), ("cel_key", _ip), ("cel_nlev", _ip),
                ("cel_ntemp", _ip), ("cel_logt", _dp), ("cel_qom", _dp), ("cel_a", _dp), ("cel_g", _dp),
                ("cel_e", _dp), ("cel_br", _dp), ("cel_z", _dp), ("cel_ar", _dp), ("cel_ad", _dp)]


class UpdGrains(C.Structure):
    _fields_ = [("nsizes", C.c_int32), ("nbins", C.c_int32), ("nu", _dp), ("xs_abs", _dp), ("radius_um", _dp),
                ("weight", _dp), ("abundance", C.c_double), ("vn", C.c_double), ("msurf", C.c_double),
                ("ion_nu", _dp)]


def library():
    global _LIB
    if _LIB is None:
        _LIB = C.CDLL(build_oracle.build())
        _LIB.oracle_update_cells.restype = C.c_int
        _LIB.oracle_update_pieces.restype = C.c_int
        _LIB.oracle_update_cells_grains.restype = C.c_int
        _LIB.oracle_grain_pieces.restype = C.c_int
    return _LIB


def marshal_grains(gp):
    """UpdGrains from the grain description of mocassin_gb300.dust.grain_physics
    (xs_abs [nsizes][nbins], radius_um, weight, abundance, vn, msurf, nu,
    ion_nu), every array widened to FP64."""
    keep = {}

    def d(name):
        a = np.ascontiguousarray(gp[name], dtype=np.float64)
        keep[name] = a
        return a.ctypes.data_as(_dp)

    xs = np.asarray(gp["xs_abs"])
    s = UpdGrains(nsizes=xs.shape[0], nbins=xs.shape[1], nu=d("nu"), xs_abs=d("xs_abs"), radius_um=d("radius_um"),
                  weight=d("weight"), abundance=float(gp["abundance"]), vn=float(gp["vn"]),
                  msurf=float(gp["msurf"]), ion_nu=d("ion_nu"))
    s._keep = keep
    return s


def marshal(t):
    keep = {}

    def d(name):
        a = np.ascontiguousarray(t[name], dtype=np.float64)
        keep[name] = a
        return a.ctypes.data_as(_dp)

    def i(name):
        a = np.ascontiguousarray(t[name], dtype=np.int32)
        keep[name] = a
        return a.ctypes.data_as(_ip)

    s = UpdTables(rrec=d("rrec"), rnew=d("rnew"), direc=d("direc"), ndirec=len(t["direc"]), aldro=d("aldro"),
                  naldro=len(t["aldro"]), ncel=len(t["cel_key"]), cel_key=i("cel_key"), cel_nlev=i("cel_nlev"),
                  cel_ntemp=i("cel_ntemp"), cel_logt=d("cel_logt"), cel_qom=d("cel_qom"), cel_a=d("cel_a"),
                  cel_g=d("cel_g"), cel_e=d("cel_e"), cel_br=d("cel_br"), cel_z=d("cel_z"), cel_ar=d("cel_ar"),
                  cel_ad=d("cel_ad"))
    s._keep = keep
    return s


def balance_ions():
    return [(z, i) for z in ELEMENTS for i in range(1, min(z, NSTAGES - 1) + 1)]


def sums(jste, xs, nu, ions, scale):
    """Photoionisation and heating sums per cell and balance ion, FP64, and
    the hit flags, from the normalised Jste (updateCell :175-269,
    thermBalance :1120-1217)."""
    J = jste.astype(np.float64) * scale              # (nbins, Nc+1)
    nu64 = nu.astype(np.float64)
    rows = {tuple(int(v) for v in r): k for k, r in enumerate(ions)}
    bal = balance_ions()
    photo = np.zeros((J.shape[1], len(bal)))
    heat = np.zeros((J.shape[1], len(bal)))
    for b, key in enumerate(bal):
        x = xs[rows[key]].astype(np.float64)
        x = np.where(x < 1e-35, 0.0, x)
        photo[:, b] = (x / (HCRYD * nu64)) @ J
        ip = int(np.argmax(x > 0))
        end = ip
        while end < len(x) and x[end] >= 1e-35:
            end += 1
        j = np.arange(ip, end)
        heat[:, b] = (x[j] * (nu64[j] - nu64[ip]) / nu64[j]) @ J[j]
    hit = (J > 0).any(0).astype(np.int32)
    return photo, heat, hit


def update_cells(tables, abund, hden, photo, heat, hit, te, ne, X, xhi_limit=0.05, threads=0, grains=None):
    """Runs the oracle update on copies of (te, ne, X); returns
    (te, ne, X, conv, niter, flags), and with grains = (grain_physics dict,
    jste_scaled [nbins][Nc+1], ndust [Nc+1], tdust [nsizes][Nc+1] or None)
    also the grain state [3][nsizes][Nc+1] (potential, photoelHeat_d,
    gasDustColl_d of each cell's last T step)."""
    lib = library()
    t = marshal(tables)
    nc1 = len(te)
    te = np.ascontiguousarray(te, dtype=np.float64).copy()
    ne = np.ascontiguousarray(ne, dtype=np.float64).copy()
    X = np.ascontiguousarray(X, dtype=np.float64).copy()
    photo = np.ascontiguousarray(photo, dtype=np.float64)
    heat = np.ascontiguousarray(heat, dtype=np.float64)
    hit = np.ascontiguousarray(hit, dtype=np.int32)
    hden = np.ascontiguousarray(hden, dtype=np.float64)
    ab = np.ascontiguousarray(abund, dtype=np.float64)
    conv = np.zeros(nc1, dtype=np.int32)
    niter = np.zeros(nc1, dtype=np.int32)
    flags = np.zeros(nc1, dtype=np.int32)
    p = lambda a: a.ctypes.data_as(_dp)
    q = lambda a: a.ctypes.data_as(_ip)
    if grains is None:
        rc = lib.oracle_update_cells(C.byref(t), C.c_int32(nc1 - 1), p(ab), p(hden), p(photo), p(heat), q(hit),
                                     C.c_double(xhi_limit), p(te), p(ne), p(X), q(conv), q(niter), q(flags),
                                     C.c_int32(threads))
        if rc != 0:
            raise RuntimeError("update oracle failed: %d" % rc)
        return te, ne, X, conv, niter, flags
    gp, js, nd, td = grains
    g = marshal_grains(gp)
    js = np.ascontiguousarray(js, dtype=np.float64)
    nd = np.ascontiguousarray(nd, dtype=np.float64)
    tdp = None
    if td is not None:
        td = np.ascontiguousarray(td, dtype=np.float64)
        tdp = p(td)
    gout = np.zeros((3, g.nsizes, nc1))
    rc = lib.oracle_update_cells_grains(C.byref(t), C.c_int32(nc1 - 1), p(ab), p(hden), p(photo), p(heat), q(hit),
                                        C.c_double(xhi_limit), p(te), p(ne), p(X), q(conv), q(niter), q(flags),
                                        C.c_int32(threads), C.byref(g), p(js), p(nd), tdp, p(gout))
    if rc != 0:
        raise RuntimeError("update oracle failed: %d" % rc)
    return te, ne, X, conv, niter, flags, gout


def grain_pieces(gp, abund, hden, te, ne, X, jrow, ndust, tdust=None):
    """The grain block of one cell at a fixed state: (out [3][nsizes] =
    potential, photoelHeat_d, gasDustColl_d; (photoelHeat_g, gasDustColl_g,
    all converged); emi_rec [nsizes][2] at the final potentials)."""
    lib = library()
    g = marshal_grains(gp)
    ns = g.nsizes
    ab = np.ascontiguousarray(abund, dtype=np.float64)
    Xc = np.ascontiguousarray(X, dtype=np.float64)
    jr = np.ascontiguousarray(jrow, dtype=np.float64)
    td = np.ascontiguousarray(np.zeros(ns) if tdust is None else tdust, dtype=np.float64)
    out = np.zeros((3, ns))
    gas = np.zeros(3)
    er = np.zeros((ns, 2))
    p = lambda a: a.ctypes.data_as(_dp)
    rc = lib.oracle_grain_pieces(C.byref(g), p(ab), C.c_double(hden), C.c_double(te), C.c_double(ne), p(Xc), p(jr),
                                 C.c_double(ndust), p(td), p(out), p(gas), p(er))
    if rc != 0:
        raise RuntimeError("grain oracle failed: %d" % rc)
    return out, (gas[0], gas[1], bool(gas[2])), er


def pieces(tables, abund, hden, photo, heat, te, ne, X):
    """alphaTot [33], per-ion line cooling [ncel] and (heat, cool) at a fixed state."""
    lib = library()
    t = marshal(tables)
    alpha = np.zeros(33)
    cel = np.zeros(len(tables["cel_key"]))
    hc = np.zeros(2)
    p = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)
    Xc = np.ascontiguousarray(X, dtype=np.float64)
    ab = np.ascontiguousarray(abund, dtype=np.float64)
    ph = np.ascontiguousarray(photo, dtype=np.float64)
    he = np.ascontiguousarray(heat, dtype=np.float64)
    lib.oracle_update_pieces(C.byref(t), ab.ctypes.data_as(_dp), C.c_double(hden), ph.ctypes.data_as(_dp),
                             he.ctypes.data_as(_dp), C.c_double(te), C.c_double(ne), Xc.ctypes.data_as(_dp),
                             alpha.ctypes.data_as(_dp), cel.ctypes.data_as(_dp), hc.ctypes.data_as(_dp))
    return alpha, cel, hc


def forbidden_lines(tables, abund, te, ne, X):
    """Per cell and line ion, the summed forbidden-line emissivity
    [1e-25 erg/s per H] of setDiffusePDF's normFor (lines above 1e-35), at the
    cells' Te [n], Ne [n] and ionic fractions X [n][7][8]; returns [n][ncel]."""
    lib = library()
    lib.oracle_forbidden_lines.restype = C.c_int
    t = marshal(tables)
    ab = np.ascontiguousarray(abund, dtype=np.float64)
    te = np.asarray(te, dtype=np.float64)
    ne = np.asarray(ne, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    n = len(te)
    out = np.zeros((n, len(tables["cel_key"])))
    for c in range(n):
        lib.oracle_forbidden_lines(C.byref(t), ab.ctypes.data_as(_dp), C.c_double(te[c]), C.c_double(ne[c]),
                                   X[c].ctypes.data_as(_dp), out[c].ctypes.data_as(_dp))
    return out
