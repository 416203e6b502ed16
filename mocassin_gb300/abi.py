"""ctypes mirror of include/mocassin_gpu.h and marshalling from a Nebula.

The structs here are byte-for-byte the C-ABI structs; a Fortran caller would
declare the same layout with ``bind(C)`` derived types.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

MC_OK = 0
MC_PREC_FP32 = 0
MC_PREC_FP64 = 1
MC_RNG_PHILOX = 0
MC_RNG_REPLAY = 1
MC_RUN_ZERO_FIRST = 1
MC_RUN_FORM_PLAIN = 2
MC_RUN_GRAPH = 4
MC_RUN_HOST_ZEROED = 8

STATUS_NAMES = {0: "MC_OK", 1: "MC_ERR_ARG", 2: "MC_ERR_CUDA", 3: "MC_ERR_BOUNDS", 4: "MC_ERR_NAN",
                5: "MC_ERR_REPLAY", 6: "MC_ERR_TIMEOUT", 7: "MC_ERR_UNSUPPORTED", 8: "MC_ERR_NOMEM",
                9: "MC_ERR_NO_DEVICE"}

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_dp = C.POINTER(C.c_double)


class McGrid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("ncells", C.c_int32),
                ("nbins", C.c_int32), ("n_angle", C.c_int32),
                ("x_axis", _fp), ("y_axis", _fp), ("z_axis", _fp), ("active", _ip),
                ("opacity", _fp), ("sca_opac", _fp), ("rec_pdf", _fp), ("total_lines", _fp),
                ("dust_pdf", _fp), ("nu_array", _fp), ("g_sca", _fp),
                ("geo_corr", C.c_float * 3), ("r_out", C.c_float), ("ion_edge1", C.c_float),
                ("flags", C.c_uint32), ("n_theta_bins", C.c_int32), ("n_phi_bins", C.c_int32),
                ("view_theta", _fp), ("view_phi", _fp)]


class McSource(C.Structure):
    _fields_ = [("istar", C.c_int32), ("cell", C.c_int32 * 3), ("n_packets", C.c_int64),
                ("delta_e", C.c_double), ("pos", C.c_float * 3), ("spec_cdf", _fp)]


class McRunOpts(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("iteration", C.c_uint32), ("precision", C.c_int32),
                ("rng", C.c_int32), ("recursion_limit", C.c_int32), ("safe_limit", C.c_int32),
                ("run_flags", C.c_int32), ("replay", _dp), ("replay_stride", C.c_int64)]


class McStats(C.Structure):
    _fields_ = [("crossings", C.c_int64), ("absorptions", C.c_int64), ("scatterings", C.c_int64),
                ("escaped", C.c_int64), ("lines", C.c_int64), ("trapped", C.c_int64),
                ("silent_exits", C.c_int64), ("safe_limit_hits", C.c_int64), ("qphot", C.c_double),
                ("kernel_ms", C.c_double), ("error_code", C.c_int32), ("error_packet", C.c_int32),
                ("march_ms", C.c_double), ("rounds", C.c_int64), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class McUpdateTables(C.Structure):
    _fields_ = [("rrec", _dp), ("rnew", _dp), ("direc", _dp), ("ndirec", C.c_int32), ("aldro", _dp),
                ("naldro", C.c_int32), ("ncel", C.c_int32), ("cel_key", _ip), ("cel_nlev", _ip),
                ("cel_ntemp", _ip), ("cel_logt", _dp), ("cel_qom", _dp), ("cel_a", _dp), ("cel_g", _dp),
                ("cel_e", _dp), ("cel_br", _dp), ("cel_z", _dp), ("cel_ar", _dp), ("cel_ad", _dp)]


_fp = C.POINTER(C.c_float)


class McEmissionTables(C.Structure):
    _fields_ = [("nbins", C.c_int32), ("nu", _fp), ("wid_flx", _fp), ("xs_h", _fp), ("xs_hei", _fp),
                ("xs_heii", _fp), ("ntk", C.c_int32), ("tk", _fp), ("nlim_hi", C.c_int32), ("nlim_hei", C.c_int32),
                ("nlim_heii", C.c_int32), ("nu_gamma_hi", _fp), ("nu_gamma_hei", _fp), ("nu_gamma_heii", _fp),
                ("lg_hi", _fp), ("lg_hei", _fp), ("lg_heii", _fp), ("y_ay", _fp), ("hi_rec", _fp),
                ("heii_rec", _fp), ("heii_lyman", _fp), ("hei_rec", _fp), ("gaunt_dd", _dp), ("n_heavy", C.c_int32),
                ("heavy", _ip), ("xs_outer", _fp), ("n_sizes", C.c_int32), ("xs_abs", _fp), ("grain_weight", _fp),
                ("t_sublime", C.c_float), ("ndust", _fp)]


def emission_tables_struct(t):
    """McEmissionTables over the arrays of mocassin_gb300.emission.tables()."""
    keep = {}

    def f(name):
        a = np.ascontiguousarray(t[name], dtype=np.float32)
        keep[name] = a
        return a.ctypes.data_as(_fp)

    dd = np.ascontiguousarray(t["gaunt_dd"], dtype=np.float64)
    hv = np.ascontiguousarray(t["shells"], dtype=np.int32)
    keep["dd"], keep["hv"] = dd, hv
    s = McEmissionTables(nbins=len(t["nu"]), nu=f("nu"), wid_flx=f("wid_flx"), xs_h=f("xs_h"), xs_hei=f("xs_hei"),
                         xs_heii=f("xs_heii"), ntk=len(t["tk"]), tk=f("tk"), nlim_hi=len(t["nu_gamma_hi"]),
                         nlim_hei=len(t["nu_gamma_hei"]), nlim_heii=len(t["nu_gamma_heii"]),
                         nu_gamma_hi=f("nu_gamma_hi"), nu_gamma_hei=f("nu_gamma_hei"),
                         nu_gamma_heii=f("nu_gamma_heii"), lg_hi=f("lg_hi"), lg_hei=f("lg_hei"),
                         lg_heii=f("lg_heii"), y_ay=f("y_ay"), hi_rec=f("hi_rec"), heii_rec=f("heii_rec"),
                         heii_lyman=f("heii_lyman"), hei_rec=f("hei_rec"), gaunt_dd=dd.ctypes.data_as(_dp),
                         n_heavy=len(hv), heavy=hv.ctypes.data_as(_ip), xs_outer=f("xs_outer"))
    if t.get("xs_abs") is not None:
        s.n_sizes = len(t["grain_weight"])
        s.xs_abs, s.grain_weight, s.ndust = f("xs_abs"), f("grain_weight"), f("ndust")
        s.t_sublime = float(t["t_sublime"])
    s._keep = keep
    return s


class McGrainPhysics(C.Structure):
    _fields_ = [("nsizes", C.c_int32), ("xs_abs", _fp), ("radius_um", _dp), ("weight", _dp),
                ("abundance", C.c_double), ("vn", C.c_double), ("msurf", C.c_double), ("ion_nu", _dp),
                ("ndust", _fp)]


def grain_physics_struct(gp):
    """McGrainPhysics over the arrays of mocassin_gb300.dust.grain_physics()."""
    keep = {}

    def arr(name, dt):
        a = np.ascontiguousarray(gp[name], dtype=dt)
        keep[name] = a
        return a.ctypes.data_as(_fp if dt == np.float32 else _dp)

    xs = np.asarray(gp["xs_abs"])
    s = McGrainPhysics(nsizes=xs.shape[0], xs_abs=arr("xs_abs", np.float32), radius_um=arr("radius_um", np.float64),
                       weight=arr("weight", np.float64), abundance=float(gp["abundance"]), vn=float(gp["vn"]),
                       msurf=float(gp["msurf"]), ion_nu=arr("ion_nu", np.float64), ndust=arr("ndust", np.float32))
    s._keep = keep
    return s


class McUpdateStats(C.Structure):
    _fields_ = [("hit", C.c_int64), ("converged", C.c_int64), ("no_te_balance", C.c_int64),
                ("no_ion_balance", C.c_int64), ("t_iterations", C.c_int64), ("dte_max", C.c_double),
                ("frac_dte_1pc", C.c_double), ("moments_ms", C.c_double), ("update_ms", C.c_double),
                ("warm_fallback", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def update_tables_struct(t):
    """McUpdateTables over the arrays of mocassin_gb300.balance.tables()."""
    keep = {}

    def d(name):
        a = np.ascontiguousarray(t[name], dtype=np.float64)
        keep[name] = a
        return a.ctypes.data_as(_dp)

    def i(name):
        a = np.ascontiguousarray(t[name], dtype=np.int32)
        keep[name] = a
        return a.ctypes.data_as(_ip)

    s = McUpdateTables(rrec=d("rrec"), rnew=d("rnew"), direc=d("direc"), ndirec=len(t["direc"]),
                       aldro=d("aldro"), naldro=len(t["aldro"]), ncel=len(t["cel_key"]), cel_key=i("cel_key"),
                       cel_nlev=i("cel_nlev"), cel_ntemp=i("cel_ntemp"), cel_logt=d("cel_logt"),
                       cel_qom=d("cel_qom"), cel_a=d("cel_a"), cel_g=d("cel_g"), cel_e=d("cel_e"),
                       cel_br=d("cel_br"), cel_z=d("cel_z"), cel_ar=d("cel_ar"), cel_ad=d("cel_ad"))
    s._keep = keep
    return s


def _ptr(a, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


class Marshalled:
    """Keeps the numpy buffers alive while the structs point at them."""

    def __init__(self, neb, n_packets=None, delta_e=None):
        self.keep = []

        def f(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float32)
            self.keep.append(a)
            return a

        act = np.ascontiguousarray(neb.active, dtype=np.int32)
        self.keep.append(act)
        g = McGrid()
        g.nx, g.ny, g.nz = neb.nx, neb.ny, neb.nz
        views = list(getattr(neb.spec, "views", ()) or ())
        g.ncells, g.nbins, g.n_angle = neb.ncells, neb.nbins, len(views)
        g.x_axis = _ptr(f(neb.x_axis), C.c_float)
        g.y_axis = _ptr(f(neb.y_axis), C.c_float)
        g.z_axis = _ptr(f(neb.z_axis), C.c_float)
        g.active = _ptr(act, C.c_int32)
        g.opacity = _ptr(f(neb.opacity), C.c_float)
        g.sca_opac = _ptr(f(neb.sca_opac), C.c_float)
        g.rec_pdf = _ptr(f(neb.rec_pdf), C.c_float)
        g.total_lines = _ptr(f(neb.total_lines), C.c_float)
        # a dust-only grid (no lgGas) re-emits from its dustPDF rows, which the
        # nebula carries in rec_pdf
        dust_only = not (neb.flags & (1 << 1))
        g.dust_pdf = _ptr(f(neb.rec_pdf) if dust_only else None, C.c_float)
        g.nu_array = _ptr(f(neb.nu), C.c_float)
        g.g_sca = _ptr(f(neb.g_sca), C.c_float)
        for i in range(3):
            g.geo_corr[i] = float(neb.geo_corr[i])
        g.r_out = float(neb.r_out)
        g.ion_edge1 = float(neb.ion_edge1)
        g.flags = int(neb.flags)
        g.n_theta_bins = int(getattr(neb.spec, "n_theta_bins", 0))
        g.n_phi_bins = int(getattr(neb.spec, "n_phi_bins", 0))
        if views:
            # viewPointTheta / viewPointPhi (0:nAngleBins), element 0 unused (0)
            g.view_theta = _ptr(f([0.0] + [v[0] for v in views]), C.c_float)
            g.view_phi = _ptr(f([0.0] + [v[1] for v in views]), C.c_float)
        else:
            g.view_theta = _ptr(None, C.c_float)
            g.view_phi = _ptr(None, C.c_float)
        self.grid = g
        ns = len(neb.star_pos)
        self.sources = (McSource * ns)()
        for s in range(ns):
            src = self.sources[s]
            src.istar = s + 1
            for i in range(3):
                src.cell[i] = int(neb.star_cell[s][i])
                src.pos[i] = float(neb.star_pos[s][i])
            npk = neb.n_packets[s] if n_packets is None else (n_packets[s] if hasattr(n_packets, "__len__") else n_packets)
            src.n_packets = int(npk)
            de = neb.delta_e[s] if delta_e is None else delta_e[s]
            src.delta_e = float(de)
            src.spec_cdf = _ptr(f(neb.spec_cdf[s]), C.c_float)
        self.nsrc = ns
        self.total_packets = sum(int(self.sources[s].n_packets) for s in range(ns))


def make_opts(seed=1, iteration=1, precision=MC_PREC_FP64, replay=None, recursion_limit=0, safe_limit=0,
              run_flags=0):
    o = McRunOpts()
    o.run_flags = run_flags
    o.seed = seed
    o.iteration = iteration
    o.precision = precision
    o.recursion_limit = recursion_limit
    o.safe_limit = safe_limit
    if replay is not None:
        replay = np.ascontiguousarray(replay, dtype=np.float64)
        o.rng = MC_RNG_REPLAY
        o.replay = replay.ctypes.data_as(_dp)
        o.replay_stride = replay.shape[1]
        o._keep = replay
    else:
        o.rng = MC_RNG_PHILOX
        o.replay = C.cast(None, _dp)
        o.replay_stride = 0
    return o


def n_angle(neb):
    return len(getattr(neb.spec, "views", ()) or ())


def escaped_shape(neb):
    """escapedPackets(0:Nc, 0:nbins, 0:nAngleBins) in C order: (nbins+1, Nc+1), or
    (nAngleBins+1, nbins+1, Nc+1) with viewing angles."""
    nc1 = neb.ncells + 1
    na = n_angle(neb)
    return (neb.nbins + 1, nc1) if na == 0 else (na + 1, neb.nbins + 1, nc1)


def estimator_arrays(neb):
    """Zeroed host accumulators: Jste, Jdif (nbins, Nc+1), escaped (escaped_shape)."""
    nc1 = neb.ncells + 1
    return (np.zeros((neb.nbins, nc1)), np.zeros((neb.nbins, nc1)), np.zeros(escaped_shape(neb)))
