"""ctypes driver of the CPU oracle (test infrastructure only).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg as
the checker / baseline; the shipped library never calls it.
"""
import ctypes as C
import os

import numpy as np

from mocassin_gb300 import abi

from . import build_oracle

_LIB = None


def library():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        lib = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        lib.oracle_transport_run.restype = C.c_int
        lib.oracle_transport_run.argtypes = [C.POINTER(abi.McGrid), C.POINTER(abi.McSource), C.c_int32,
                                             C.POINTER(abi.McRunOpts), dp, dp, dp, C.POINTER(abi.McStats),
                                             C.c_int32, C.c_int32]
        lib.oracle_philox4x32_10.restype = None
        lib.oracle_draws.restype = None
        lib.oracle_draws.argtypes = [C.c_uint64, C.c_uint32, C.c_int32, C.c_uint64, C.c_int32, C.c_int32, dp]
        _LIB = lib
    return _LIB


def run(neb, n_packets=None, seed=1, iteration=1, precision="fp64", replay=None, threads=0, acc32=False,
        recursion_limit=0, safe_limit=0, out=None, marshalled=None, res_counts=None):
    """Oracle transport of all stars of ``neb``; returns (jste, jdif, escaped, stats).

    out: (jste, jdif, escaped) arrays of abi.estimator_arrays(neb) to zero
    and fill instead of new ones; marshalled: an abi.Marshalled(neb,
    n_packets) to reuse (a timing loop keeps both out of its timed region);
    res_counts: resonance-line packets per active cell [Nc+1] (a block after
    each star's packets, Philox draws)."""
    lib = library()
    m = marshalled if marshalled is not None else abi.Marshalled(neb, n_packets=n_packets)
    prec = abi.MC_PREC_FP64 if precision == "fp64" else abi.MC_PREC_FP32
    opts = abi.make_opts(seed=seed, iteration=iteration, precision=prec, replay=replay,
                         recursion_limit=recursion_limit, safe_limit=safe_limit)
    if out is None:
        js, jd, es = abi.estimator_arrays(neb)
    else:
        js, jd, es = out
        js.fill(0.0)
        es.fill(0.0)
        if neb.flags & (1 << 4):  # MC_FLAG_DEBUG: Jdif is written only in debug mode
            jd.fill(0.0)
    st = abi.McStats()
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    if res_counts is None:
        rc = lib.oracle_transport_run(C.byref(m.grid), m.sources, m.nsrc, C.byref(opts), dp(js), dp(jd), dp(es),
                                      C.byref(st), int(threads), int(acc32))
    else:
        rcnt = np.ascontiguousarray(res_counts, dtype=np.int32)
        if rcnt.shape != (neb.ncells + 1,):
            raise ValueError("res_counts must have Nc+1 entries")
        rc = lib.oracle_transport_run_res(C.byref(m.grid), m.sources, m.nsrc, C.byref(opts), dp(js), dp(jd),
                                          dp(es), C.byref(st), int(threads),
                                          rcnt.ctypes.data_as(C.POINTER(C.c_int32)))
    if rc != 0:
        raise RuntimeError("oracle failed with status %d (packet %d)" % (rc, st.error_packet))
    return js, jd, es, st.as_dict()


def philox(ctr, key):
    lib = library()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.oracle_philox4x32_10(c, k, o)
    return list(o)


def draws(seed, iteration, istar, packet, precision, n):
    out = np.zeros(n)
    library().oracle_draws(seed, iteration, istar, packet, precision, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out
