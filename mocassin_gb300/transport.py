"""Host-side mirror of mocassin's transport interface over libmcgpu.so.

``energy_packet_driver`` is the call the Fortran ``iterateMC`` makes
(``call energyPacketDriver(iStar, load, grid(1:nGrids))``,
source/iteration_mod.f90:488-493): it runs all packets of the given stars and
adds the path-length estimators into Jste (and escapedPackets).  Errors are
raised as ``TransportError`` carrying the C-ABI status and message, the
counterpart of the reference's fatal ``print*; stop`` insanity checks.

There is no CPU fallback: if the CUDA library is missing or no GPU is
visible, the call fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_LIB = None
LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libmcgpu.so")


class TransportError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), message))
        self.status = status


def library():
    """Loads libmcgpu.so (built by mocassin_gb300.build); raises if absent."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise TransportError(2, "libmcgpu.so is not built (%s); run mocassin_gb300.build.build()" % LIB_PATH)
        lib = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        fp = C.POINTER(C.c_float)
        lib.mc_abi_version.restype = C.c_int
        lib.mc_last_error.restype = C.c_char_p
        lib.mc_transport_run.restype = C.c_int
        lib.mc_transport_run.argtypes = [C.POINTER(abi.McGrid), C.POINTER(abi.McSource), C.c_int32,
                                         C.POINTER(abi.McRunOpts), dp, dp, dp, C.POINTER(abi.McStats)]
        lib.mc_transport_run_f32.restype = C.c_int
        lib.mc_transport_run_f32.argtypes = [C.POINTER(abi.McGrid), C.POINTER(abi.McSource), C.c_int32,
                                             C.POINTER(abi.McRunOpts), fp, fp, fp, C.POINTER(abi.McStats)]
        lib.mc_ctx_create.restype = C.c_int
        lib.mc_ctx_create.argtypes = [C.POINTER(abi.McGrid), C.POINTER(C.c_void_p)]
        lib.mc_ctx_update.restype = C.c_int
        lib.mc_ctx_update.argtypes = [C.c_void_p, C.POINTER(abi.McGrid)]
        lib.mc_ctx_zero.restype = C.c_int
        lib.mc_ctx_zero.argtypes = [C.c_void_p]
        lib.mc_ctx_run.restype = C.c_int
        lib.mc_batch_run.restype = C.c_int
        lib.mc_batch_run.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.POINTER(abi.McSource)),
                                     C.POINTER(C.c_int32), C.POINTER(abi.McRunOpts), C.POINTER(abi.McStats)]
        lib.mc_ctx_run.argtypes = [C.c_void_p, C.POINTER(abi.McSource), C.c_int32, C.POINTER(abi.McRunOpts),
                                   C.POINTER(abi.McStats)]
        lib.mc_ctx_download.restype = C.c_int
        lib.mc_ctx_download.argtypes = [C.c_void_p, dp, dp, dp, C.c_int32]
        lib.mc_ctx_device_estimators.restype = C.c_int
        lib.mc_ctx_device_estimators.argtypes = [C.c_void_p, C.POINTER(dp), C.POINTER(dp), C.POINTER(dp)]
        lib.mc_transport_release.restype = C.c_int
        lib.mc_ctx_jste_moments.restype = C.c_int
        lib.mc_ctx_jste_moments.argtypes = [C.c_void_p, C.c_int32, fp, C.c_double, fp, dp]
        ip = C.POINTER(C.c_int32)
        lib.mc_ctx_set_update_tables.restype = C.c_int
        lib.mc_ctx_set_update_tables.argtypes = [C.c_void_p, C.POINTER(abi.McUpdateTables), dp, dp]
        lib.mc_ctx_set_emission_tables.restype = C.c_int
        lib.mc_ctx_set_emission_tables.argtypes = [C.c_void_p, C.POINTER(abi.McEmissionTables)]
        lib.mc_ctx_build_emission.restype = C.c_int
        lib.mc_ctx_build_emission.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        lib.mc_ctx_get_emission.restype = C.c_int
        lib.mc_ctx_get_emission.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.mc_ctx_get_dust_emission.restype = C.c_int
        lib.mc_ctx_get_dust_emission.argtypes = [C.c_void_p, C.c_void_p]
        lib.mc_ctx_set_cell_state.restype = C.c_int
        lib.mc_ctx_set_cell_state.argtypes = [C.c_void_p, dp, dp, dp]
        lib.mc_ctx_get_cell_state.restype = C.c_int
        lib.mc_ctx_get_cell_state.argtypes = [C.c_void_p, dp, dp, dp, ip, ip, ip]
        lib.mc_ctx_update_cells.restype = C.c_int
        lib.mc_ctx_update_cells.argtypes = [C.c_void_p, fp, C.c_double, C.c_double, C.c_int32,
                                            C.POINTER(abi.McUpdateStats)]
        lib.mc_ctx_opacity_from_state.restype = C.c_int
        lib.mc_ctx_opacity_from_state.argtypes = [C.c_void_p, C.c_int32, ip, fp, C.c_int32, dp]
        lib.mc_ctx_set_fixed_opacity.restype = C.c_int
        lib.mc_ctx_set_fixed_opacity.argtypes = [C.c_void_p, C.c_int32, fp, fp]
        u64 = C.c_uint64
        lib.mc_ctx_surrogate_init.restype = C.c_int
        lib.mc_ctx_surrogate_rows.restype = C.c_int
        lib.mc_ctx_surrogate_rows.argtypes = [C.c_void_p, C.POINTER(C.c_int64), fp, fp]
        lib.mc_ctx_surrogate_load.restype = C.c_int
        lib.mc_ctx_surrogate_load.argtypes = [C.c_void_p, C.c_int64, fp, fp]
        lib.mc_ctx_surrogate_rule.restype = C.c_int
        lib.mc_ctx_surrogate_rule.argtypes = [C.c_void_p, C.c_double, C.c_double]
        lib.mc_ctx_surrogate_init.argtypes = [C.c_void_p, u64, C.c_int64]
        lib.mc_ctx_surrogate_collect.restype = C.c_int
        lib.mc_ctx_surrogate_collect.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        lib.mc_ctx_surrogate_train.restype = C.c_int
        lib.mc_ctx_surrogate_train.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_float, u64, dp, dp]
        lib.mc_ctx_update_cells_warm.restype = C.c_int
        lib.mc_ctx_update_cells_warm.argtypes = [C.c_void_p, fp, C.c_double, C.c_double, C.c_int32,
                                                 C.POINTER(abi.McUpdateStats)]
        lib.mc_ctx_surrogate_params.restype = C.c_int
        lib.mc_ctx_surrogate_params.argtypes = [C.c_void_p, fp, fp]
        lib.mc_ctx_surrogate_grads.restype = C.c_int
        lib.mc_ctx_surrogate_grads.argtypes = [C.c_void_p, C.c_int32, fp, fp, dp, fp, fp]
        lib.mc_ctx_set_tuning.restype = C.c_int
        lib.mc_ctx_set_tuning.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
        lib.mc_ctx_get_tuning.restype = C.c_int
        lib.mc_ctx_get_tuning.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        lib.mc_ctx_set_res_lines.restype = C.c_int
        lib.mc_ctx_set_res_lines.argtypes = [C.c_void_p, C.POINTER(C.c_int32)]
        lib.mc_ctx_set_grain_opacity.restype = C.c_int
        lib.mc_ctx_set_grain_opacity.argtypes = [C.c_void_p, C.c_int32, fp, fp, fp, fp, C.c_float]
        lib.mc_ctx_set_grain_physics.restype = C.c_int
        lib.mc_ctx_set_grain_physics.argtypes = [C.c_void_p, C.POINTER(abi.McGrainPhysics)]
        lib.mc_ctx_grain_state.restype = C.c_int
        lib.mc_ctx_grain_state.argtypes = [C.c_void_p, dp, dp, dp]
        lib.mc_ctx_dust_temperatures.restype = C.c_int
        lib.mc_ctx_dust_temperatures.argtypes = [C.c_void_p, C.c_int32, fp, fp, C.c_int32, fp, C.c_double, fp, dp]
        lib.mc_ctx_get_opacity.restype = C.c_int
        lib.mc_ctx_get_opacity.argtypes = [C.c_void_p, fp]
        lib.mc_ctx_get_scattering.restype = C.c_int
        lib.mc_ctx_get_scattering.argtypes = [C.c_void_p, fp]
        lib.mc_ctx_destroy.restype = None
        lib.mc_ctx_destroy.argtypes = [C.c_void_p]
        lib.mc_opacity_build.restype = C.c_int
        lib.mc_opacity_build.argtypes = [C.c_int32, C.c_int32, C.c_int32, fp, fp, fp, C.c_int32, fp, dp]
        lib.mc_ctx_build_opacity.restype = C.c_int
        lib.mc_ctx_build_opacity.argtypes = [C.c_void_p, C.c_int32, fp, fp, fp, C.c_int32, C.c_int32, dp]
        if lib.mc_abi_version() != 2:
            raise TransportError(1, "ABI version mismatch")
        _LIB = lib
    return _LIB


def _check(status):
    if status != 0:
        raise TransportError(status, library().mc_last_error().decode())


def _dptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _check_shapes(neb, jste, jdif, escaped):
    """The estimators are all float64 (mc_transport_run) or all float32
    (mc_transport_run_f32, the grid's own arrays)."""
    nj = (neb.nbins, neb.ncells + 1)
    dt = jste.dtype if jste is not None else np.dtype(np.float64)
    if dt not in (np.float64, np.float32):
        raise ValueError("the estimators must be float64 or float32")
    for name, a, shape in (("jste", jste, nj), ("jdif", jdif, nj), ("escaped", escaped, abi.escaped_shape(neb))):
        if a is None:
            continue
        if a.shape != shape or a.dtype != dt or not a.flags.c_contiguous:
            raise ValueError("%s must be a C-contiguous %s array of shape %s" % (name, dt, shape))


def _flags(form, zero_first=False, host_zeroed=False):
    """form: "wave" (rounds driven by the host), "graph" (the same rounds
    inside one CUDA graph) or "plain" (one thread per history)."""
    if form not in ("wave", "plain", "graph"):
        raise ValueError("form must be 'wave', 'graph' or 'plain'")
    f = {"wave": 0, "graph": abi.MC_RUN_GRAPH, "plain": abi.MC_RUN_FORM_PLAIN}[form]
    return f | (abi.MC_RUN_ZERO_FIRST if zero_first else 0) | (abi.MC_RUN_HOST_ZEROED if host_zeroed else 0)


def energy_packet_driver(neb, n_packets=None, seed=1, iteration=1, precision="fp32", replay=None,
                         jste=None, jdif=None, escaped=None, recursion_limit=0, safe_limit=0, form="wave",
                         zero_first=False, host_zeroed=False):
    """Runs every packet of every star of ``neb`` through the GPU transport.

    Accumulates into ``jste`` / ``jdif`` / ``escaped`` (created zeroed when not
    given; shapes ``(nbins, Nc+1)`` and ``(nbins+1, Nc+1)``, i.e. Fortran
    ``(0:Nc, 1:nbins)`` cell fastest) and returns ``(jste, jdif, escaped,
    stats)``.  ``form`` selects the frequency-sorted persistent march
    ("wave", the default; "graph" with its rounds in one CUDA graph) or one
    thread per history ("plain").  zero_first: the arrays are overwritten
    with this transport's sums instead of accumulated into (they are not
    uploaded).  host_zeroed: the arrays hold zeros on entry and only the
    entries this transport made nonzero are written (MC_RUN_HOST_ZEROED);
    stats then report the bytes the call copied (h2d_bytes, d2h_bytes).
    """
    lib = library()
    m = abi.Marshalled(neb, n_packets=n_packets)
    prec = abi.MC_PREC_FP64 if precision == "fp64" else abi.MC_PREC_FP32
    opts = abi.make_opts(seed=seed, iteration=iteration, precision=prec, replay=replay,
                         recursion_limit=recursion_limit, safe_limit=safe_limit,
                         run_flags=_flags(form, zero_first, host_zeroed))
    js0, jd0, es0 = abi.estimator_arrays(neb)
    jste = js0 if jste is None else jste
    escaped = es0 if escaped is None else escaped
    _check_shapes(neb, jste, jdif, escaped)
    if jdif is None and (neb.flags & abi_flag_debug()):
        jdif = jd0
    st = abi.McStats()
    if jste.dtype == np.float32:
        # the grid's own 4-byte arrays (mc_transport_run_f32)
        _check(lib.mc_transport_run_f32(C.byref(m.grid), m.sources, m.nsrc, C.byref(opts), _fptr(jste), _fptr(jdif),
                                        _fptr(escaped), C.byref(st)))
    else:
        _check(lib.mc_transport_run(C.byref(m.grid), m.sources, m.nsrc, C.byref(opts), _dptr(jste), _dptr(jdif),
                                    _dptr(escaped), C.byref(st)))
    return jste, jdif, escaped, st.as_dict()


OPACITY_METHODS = {"fp32": 0, "bf16x3": 1}


def _fptr(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def opacity_build(den, xs, ff=None, method="bf16x3"):
    """opacity(cell, nu) = sum_k den(k, cell) xs(k, nu) + ff(cell) [nu = 1] on the GPU.

    den: (K, Nc+1), xs: (K, nbins), ff: (Nc+1,) or None; returns (opacity
    (nbins, Nc+1) float32, kernel ms).  The dense form of addOpacity
    (ionization_mod.f90:349-484) with the dust add (iteration_mod.f90:166-227).
    """
    lib = library()
    den = np.ascontiguousarray(den, dtype=np.float32)
    xs = np.ascontiguousarray(xs, dtype=np.float32)
    ff = None if ff is None else np.ascontiguousarray(ff, dtype=np.float32)
    k, nc1 = den.shape
    nb = xs.shape[1]
    out = np.empty((nb, nc1), dtype=np.float32)
    ms = C.c_double()
    _check(lib.mc_opacity_build(nc1 - 1, k, nb, _fptr(den), _fptr(xs), _fptr(ff), OPACITY_METHODS[method],
                                _fptr(out), C.byref(ms)))
    return out, ms.value


def abi_flag_debug():
    return 1 << 4


class TransportContext:
    """A grid resident in HBM across iterations (mc_ctx_* entry points)."""

    def __init__(self, neb):
        self.lib = library()
        self.neb = neb
        self._m = abi.Marshalled(neb)
        h = C.c_void_p()
        _check(self.lib.mc_ctx_create(C.byref(self._m.grid), C.byref(h)))
        self.handle = h

    def update(self, neb):
        m = abi.Marshalled(neb)
        _check(self.lib.mc_ctx_update(self.handle, C.byref(m.grid)))
        self.neb, self._m = neb, m

    def zero(self):
        _check(self.lib.mc_ctx_zero(self.handle))

    def run(self, n_packets=None, seed=1, iteration=1, precision="fp32", replay=None, recursion_limit=0,
            safe_limit=0, zero_first=False, form="wave"):
        m = abi.Marshalled(self.neb, n_packets=n_packets)
        prec = abi.MC_PREC_FP64 if precision == "fp64" else abi.MC_PREC_FP32
        opts = abi.make_opts(seed=seed, iteration=iteration, precision=prec, replay=replay,
                             recursion_limit=recursion_limit, safe_limit=safe_limit,
                             run_flags=_flags(form, zero_first))
        st = abi.McStats()
        _check(self.lib.mc_ctx_run(self.handle, m.sources, m.nsrc, C.byref(opts), C.byref(st)))
        return st.as_dict()

    def download(self, jste=None, jdif=None, escaped=None, accumulate=False):
        js0, jd0, es0 = abi.estimator_arrays(self.neb)
        jste = js0 if jste is None else jste
        escaped = es0 if escaped is None else escaped
        _check_shapes(self.neb, jste, jdif, escaped)
        _check(self.lib.mc_ctx_download(self.handle, _dptr(jste), _dptr(jdif), _dptr(escaped), int(accumulate)))
        return jste, jdif, escaped

    def build_opacity(self, den, xs, ff=None, method="bf16x3", sca=False):
        """Rebuilds the resident opacity (or scaOpac) from den / xs on the GPU."""
        den = np.ascontiguousarray(den, dtype=np.float32)
        xs = np.ascontiguousarray(xs, dtype=np.float32)
        ff = None if ff is None else np.ascontiguousarray(ff, dtype=np.float32)
        ms = C.c_double()
        _check(self.lib.mc_ctx_build_opacity(self.handle, den.shape[0], _fptr(den), _fptr(xs), _fptr(ff),
                                             OPACITY_METHODS[method], int(sca), C.byref(ms)))
        return ms.value

    def jste_moments(self, w, scale=1.0):
        """out(o, cell) = scale * sum_nu Jste(nu, cell) w(nu, o) on the resident Jste
        (the photoionisation and heating sums of updateCell, update_mod.f90:175-269)."""
        w = np.ascontiguousarray(w, dtype=np.float32)
        nout = w.shape[1]
        out = np.empty((nout, self.neb.ncells + 1), dtype=np.float32)
        ms = C.c_double()
        _check(self.lib.mc_ctx_jste_moments(self.handle, nout, _fptr(w), float(scale), _fptr(out), C.byref(ms)))
        return out, ms.value

    # ---- the cell update (ionisation and thermal balance) ----
    def set_update_tables(self, tables, hden, abund):
        self._ut = abi.update_tables_struct(tables)
        h = np.ascontiguousarray(hden, dtype=np.float64)
        a = np.ascontiguousarray(abund, dtype=np.float64)
        _check(self.lib.mc_ctx_set_update_tables(self.handle, C.byref(self._ut), _dptr(h), _dptr(a)))

    def set_emission_tables(self, tables=None):
        """Uploads the diffuse-emission tables (mocassin_gb300.emission.tables()
        by default) for build_emission."""
        from . import emission
        t = emission.tables(self.neb) if tables is None else tables
        self._et = abi.emission_tables_struct(t)
        _check(self.lib.mc_ctx_set_emission_tables(self.handle, C.byref(self._et)))

    def build_emission(self):
        """Rebuilds every cell's recPDF row and totalLines on the GPU from the
        resident cell state; returns the device time [ms]."""
        ms = C.c_float()
        _check(self.lib.mc_ctx_build_emission(self.handle, C.byref(ms)))
        return ms.value

    def get_emission(self):
        """The CDF rows (Nc+1, nbins) and totalLines (Nc+1,) on the device."""
        nc1, nb = self.neb.ncells + 1, self.neb.nbins
        rows = np.empty((nc1, nb), dtype=np.float32)
        tl = np.empty(nc1, dtype=np.float32)
        _check(self.lib.mc_ctx_get_emission(self.handle, rows.ctypes.data, tl.ctypes.data))
        return rows, tl

    def get_dust_emission(self):
        """The dustPDF rows (Nc+1, nbins) of a dust-only grid on the device."""
        rows = np.empty((self.neb.ncells + 1, self.neb.nbins), dtype=np.float32)
        _check(self.lib.mc_ctx_get_dust_emission(self.handle, rows.ctypes.data))
        return rows

    def set_cell_state(self, te, ne, X):
        te = np.ascontiguousarray(te, dtype=np.float64)
        ne = np.ascontiguousarray(ne, dtype=np.float64)
        X = np.ascontiguousarray(X, dtype=np.float64)
        if te.shape != (self.neb.ncells + 1,) or X.shape != (self.neb.ncells + 1, 7, 8):
            raise ValueError("te (Nc+1,), ne (Nc+1,), X (Nc+1, 7, 8)")
        _check(self.lib.mc_ctx_set_cell_state(self.handle, _dptr(te), _dptr(ne), _dptr(X)))

    def get_cell_state(self):
        nc1 = self.neb.ncells + 1
        te, ne, X = np.empty(nc1), np.empty(nc1), np.empty((nc1, 7, 8))
        conv, niter, flags = (np.empty(nc1, dtype=np.int32) for _ in range(3))
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        _check(self.lib.mc_ctx_get_cell_state(self.handle, _dptr(te), _dptr(ne), _dptr(X), ip(conv), ip(niter),
                                              ip(flags)))
        return te, ne, X, conv, niter, flags

    def update_cells(self, w, scale, xhi_limit=0.05, precision="fp64", warm=False):
        """One cell update from the resident Jste; warm=True starts it from the
        trained surrogate's prediction (mc_ctx_update_cells_warm)."""
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.shape != (self.neb.nbins, 67):
            raise ValueError("w must be (nbins, 67)")
        prec = abi.MC_PREC_FP64 if precision == "fp64" else abi.MC_PREC_FP32
        st = abi.McUpdateStats()
        fn = self.lib.mc_ctx_update_cells_warm if warm else self.lib.mc_ctx_update_cells
        _check(fn(self.handle, _fptr(w), float(scale), float(xhi_limit), prec, C.byref(st)))
        return st.as_dict()

    # ---- the learned warm start ----
    N_PARAMS = 164656

    def surrogate_init(self, seed=1, capacity=2_000_000):
        _check(self.lib.mc_ctx_surrogate_init(self.handle, int(seed), int(capacity)))

    def surrogate_rows(self):
        """The collected training rows: features (n, 80), targets (n, 48)."""
        n = C.c_int64()
        _check(self.lib.mc_ctx_surrogate_rows(self.handle, C.byref(n), None, None))
        x = np.empty((n.value, 80), dtype=np.float32)
        t = np.empty((n.value, 48), dtype=np.float32)
        _check(self.lib.mc_ctx_surrogate_rows(self.handle, C.byref(n), _fptr(x), _fptr(t)))
        return x, t

    def surrogate_load(self, x, t):
        """Appends training rows (e.g. other models' cell states)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        if x.shape[1:] != (80,) or t.shape != (len(x), 48):
            raise ValueError("x (n, 80) and t (n, 48)")
        _check(self.lib.mc_ctx_surrogate_load(self.handle, len(x), _fptr(x), _fptr(t)))

    def surrogate_rule(self, accept_res=0.01, near_res=0.3):
        """The warm start's rule (mc_ctx_surrogate_rule): accept a prediction
        whose residual / heating is below accept_res, bracket it below
        near_res, else fall back to the plain solve."""
        _check(self.lib.mc_ctx_surrogate_rule(self.handle, float(accept_res), float(near_res)))

    def surrogate_collect(self):
        n = C.c_int64()
        _check(self.lib.mc_ctx_surrogate_collect(self.handle, C.byref(n)))
        return n.value

    def surrogate_train(self, steps=300, batch=8192, lr=2e-3, seed=1):
        loss, ms = C.c_double(), C.c_double()
        _check(self.lib.mc_ctx_surrogate_train(self.handle, int(steps), int(batch), float(lr), int(seed),
                                               C.byref(loss), C.byref(ms)))
        return loss.value, ms.value

    def surrogate_params(self, set=None):
        out = np.empty(self.N_PARAMS, dtype=np.float32)
        s = None if set is None else np.ascontiguousarray(set, dtype=np.float32)
        _check(self.lib.mc_ctx_surrogate_params(self.handle, _fptr(out), _fptr(s)))
        return out

    def surrogate_forward(self, x):
        """Outputs [m, 48] of the network for feature rows x [m, 80] on the
        tensor cores (the arithmetic of the warm start's prediction)."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty((len(x), 48), dtype=np.float32)
        self.lib.mc_ctx_surrogate_forward.restype = C.c_int
        self.lib.mc_ctx_surrogate_forward.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_float),
                                                      C.POINTER(C.c_float)]
        _check(self.lib.mc_ctx_surrogate_forward(self.handle, len(x), _fptr(x), _fptr(y)))
        return y

    def surrogate_grads(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        m = x.shape[0]
        g = np.empty(self.N_PARAMS, dtype=np.float32)
        y = np.empty((m, 48), dtype=np.float32)
        loss = C.c_double()
        _check(self.lib.mc_ctx_surrogate_grads(self.handle, m, _fptr(x), _fptr(t), C.byref(loss), _fptr(g), _fptr(y)))
        return loss.value, g, y

    def set_tuning(self, refill_min, inner_steps):
        _check(self.lib.mc_ctx_set_tuning(self.handle, int(refill_min), int(inner_steps)))

    def get_tuning(self):
        r, i = C.c_int32(), C.c_int32()
        _check(self.lib.mc_ctx_get_tuning(self.handle, C.byref(r), C.byref(i)))
        return r.value, i.value

    def dust_temperatures(self, w_abs, em_table, grain_weight, scale):
        """Grain temperatures (getDustT) on the resident Jste: (nsizes+1, Nc+1),
        row 0 the weighted mean over sizes; and the kernel time."""
        w_abs = np.ascontiguousarray(w_abs, dtype=np.float32)
        em = np.ascontiguousarray(em_table, dtype=np.float32)
        gw = np.ascontiguousarray(grain_weight, dtype=np.float32)
        nsizes = w_abs.shape[1]
        out = np.empty((nsizes + 1, self.neb.ncells + 1), dtype=np.float32)
        ms = C.c_double()
        _check(self.lib.mc_ctx_dust_temperatures(self.handle, nsizes, _fptr(w_abs), _fptr(em), em.shape[1], _fptr(gw),
                                                 float(scale), _fptr(out), C.byref(ms)))
        return out, ms.value

    def set_res_lines(self, counts):
        """Resonance-line packets per active cell [Nc+1] for every later run
        (None: off); see mc_ctx_set_res_lines."""
        if counts is None:
            _check(self.lib.mc_ctx_set_res_lines(self.handle, None))
            return
        c = np.ascontiguousarray(counts, dtype=np.int32)
        if c.shape != (self.neb.ncells + 1,):
            raise ValueError("counts must have Nc+1 entries")
        _check(self.lib.mc_ctx_set_res_lines(self.handle, c.ctypes.data_as(C.POINTER(C.c_int32))))

    def set_grain_opacity(self, xs_ext, xs_sca, weight, ndust, t_sublime):
        """The grains' rows of every opacity_from_state: per size, weight x
        Ndust x xs_ext into the opacity and x xs_sca into the scattering
        table, for the sizes below t_sublime (the last dust_temperatures)."""
        if xs_ext is None:
            _check(self.lib.mc_ctx_set_grain_opacity(self.handle, 0, None, None, None, None, 0.0))
            return
        ext = np.ascontiguousarray(xs_ext, dtype=np.float32)
        sca = np.ascontiguousarray(xs_sca, dtype=np.float32)
        w = np.ascontiguousarray(weight, dtype=np.float32)
        nd = np.ascontiguousarray(ndust, dtype=np.float32)
        _check(self.lib.mc_ctx_set_grain_opacity(self.handle, ext.shape[0], _fptr(ext), _fptr(sca), _fptr(w),
                                                 _fptr(nd), float(t_sublime)))

    def set_grain_physics(self, grains):
        """Grains in the gas update (photoelectric heating and gas-grain
        collisions, update_mod.f90:527-930) from the description of
        dust.grain_physics; None: a gas-only update again."""
        if grains is None:
            _check(self.lib.mc_ctx_set_grain_physics(self.handle, None))
            self._grains = None
            return
        s = abi.grain_physics_struct(grains)
        _check(self.lib.mc_ctx_set_grain_physics(self.handle, C.byref(s)))
        self._grains = int(s.nsizes)

    def grain_state(self):
        """(potential [Ryd], photoelHeat_d, gasDustColl_d), each [nsizes][Nc+1],
        of every cell's last T step in the last update with grains."""
        ns = getattr(self, "_grains", None)
        if not ns:
            raise TransportError(1, "no grain physics set")
        out = [np.empty((ns, self.neb.ncells + 1)) for _ in range(3)]
        _check(self.lib.mc_ctx_grain_state(self.handle, *[o.ctypes.data_as(C.POINTER(C.c_double)) for o in out]))
        return tuple(out)

    def get_opacity(self):
        out = np.empty((self.neb.nbins, self.neb.ncells + 1), dtype=np.float32)
        _check(self.lib.mc_ctx_get_opacity(self.handle, _fptr(out)))
        return out

    def get_scattering(self):
        out = np.empty((self.neb.nbins, self.neb.ncells + 1), dtype=np.float32)
        _check(self.lib.mc_ctx_get_scattering(self.handle, _fptr(out)))
        return out

    def set_fixed_opacity(self, den, xs):
        """Opacity rows that do not follow the cell state (den [rows][Nc+1],
        xs [rows][nbins]), appended to every opacity_from_state."""
        d = np.ascontiguousarray(np.atleast_2d(den), dtype=np.float32)
        x = np.ascontiguousarray(np.atleast_2d(xs), dtype=np.float32)
        _check(self.lib.mc_ctx_set_fixed_opacity(self.handle, len(d), _fptr(d), _fptr(x)))

    def opacity_from_state(self, species, xs, method="bf16x3"):
        sp = np.ascontiguousarray(species, dtype=np.int32)
        x = np.ascontiguousarray(xs, dtype=np.float32)
        ms = C.c_double()
        _check(self.lib.mc_ctx_opacity_from_state(self.handle, len(sp), sp.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  _fptr(x), OPACITY_METHODS[method], C.byref(ms)))
        return ms.value

    def device_estimators(self):
        j, d, e = C.POINTER(C.c_double)(), C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
        _check(self.lib.mc_ctx_device_estimators(self.handle, C.byref(j), C.byref(d), C.byref(e)))
        addr = lambda p: C.cast(p, C.c_void_p).value or 0
        return addr(j), addr(d), addr(e)

    def close(self):
        if self.handle:
            self.lib.mc_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_run(contexts, n_packets=None, seeds=None, iteration=1, precision="fp32", recursion_limit=0,
              safe_limit=0, zero_first=False):
    """One transport iteration of many resident models, their rounds in step and
    every round's march one persistent launch over all of them (mc_batch_run).
    Model i draws as ``contexts[i].run(seed=seeds[i], ...)`` would, so its
    estimators and counters are those of that call.  Returns the per-model stats."""
    contexts = list(contexts)
    n = len(contexts)
    if n == 0:
        return []
    lib = library()
    seeds = list(range(1, n + 1)) if seeds is None else list(seeds)
    npk = [n_packets] * n if n_packets is None or np.isscalar(n_packets) else list(n_packets)
    marsh = [abi.Marshalled(ctx.neb, n_packets=npk[i]) for i, ctx in enumerate(contexts)]
    prec = abi.MC_PREC_FP64 if precision == "fp64" else abi.MC_PREC_FP32
    opts = (abi.McRunOpts * n)(*[abi.make_opts(seed=seeds[i], iteration=iteration, precision=prec,
                                               recursion_limit=recursion_limit, safe_limit=safe_limit,
                                               run_flags=_flags("wave", zero_first)) for i in range(n)])
    handles = (C.c_void_p * n)(*[ctx.handle for ctx in contexts])
    srcs = (C.POINTER(abi.McSource) * n)(*[C.cast(m.sources, C.POINTER(abi.McSource)) for m in marsh])
    nsrcs = (C.c_int32 * n)(*[m.nsrc for m in marsh])
    stats = (abi.McStats * n)()
    _check(lib.mc_batch_run(handles, n, srcs, nsrcs, opts, stats))
    return [st.as_dict() for st in stats]
