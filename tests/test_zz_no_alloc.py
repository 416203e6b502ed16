"""mc_transport_run_noalloc: the transport for callers that cannot allocate.

Some callers cannot call cudaMalloc (a code that only hands over device
memory it already manages, a loop where an allocation could block or fail).
This entry point takes every array as a device pointer the caller owns and
allocates nothing itself.  Here the test plays such a caller: it owns the
device arrays (torch tensors) and checks, on two calls in a row, that the
results equal those of the existing entry point mc_transport_run in its
plain form on the same draws -- counters exactly, Jste / escapedPackets to
1e-12 relative (FP64 march) -- so state kept in the shared scratch between
calls cannot leak into a result.
"""
import ctypes as C

import numpy as np
import pytest

from mocassin_gb300 import abi, nebula, transport

pytestmark = pytest.mark.gpu

RTOL = 1e-12
KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")


def _lib():
    lib = transport.library()
    dp = C.POINTER(C.c_double)
    f = lib.mc_transport_run_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.McGrid), C.POINTER(abi.McSource), C.c_int32, C.POINTER(abi.McRunOpts), dp, dp, dp,
                  C.POINTER(abi.McStats), C.c_void_p]
    return lib


class DeviceNebula:
    """The caller's own device copies of a nebula's arrays."""

    def __init__(self, neb):
        import torch
        self.keep = []

        def dev(a, dtype=np.float32):
            if a is None:
                return None
            t = torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()
            self.keep.append(t)
            return t

        def fp(t):
            return C.cast(t.data_ptr() if t is not None else None, C.POINTER(C.c_float))

        g = abi.McGrid()
        g.nx, g.ny, g.nz = neb.nx, neb.ny, neb.nz
        g.ncells, g.nbins, g.n_angle = neb.ncells, neb.nbins, 0
        g.x_axis, g.y_axis, g.z_axis = fp(dev(neb.x_axis)), fp(dev(neb.y_axis)), fp(dev(neb.z_axis))
        g.active = C.cast(dev(neb.active, np.int32).data_ptr(), C.POINTER(C.c_int32))
        g.opacity = fp(dev(neb.opacity))
        g.sca_opac = fp(dev(neb.sca_opac))
        g.rec_pdf = fp(dev(neb.rec_pdf))
        g.total_lines = fp(dev(neb.total_lines))
        g.dust_pdf = fp(None)
        g.nu_array = fp(dev(neb.nu))
        g.g_sca = fp(dev(neb.g_sca))
        for i in range(3):
            g.geo_corr[i] = float(neb.geo_corr[i])
        g.r_out, g.ion_edge1, g.flags = float(neb.r_out), float(neb.ion_edge1), int(neb.flags)
        self.grid = g
        ns = len(neb.star_pos)
        self.sources = (abi.McSource * ns)()
        for s in range(ns):
            src = self.sources[s]
            src.istar = s + 1
            for i in range(3):
                src.cell[i] = int(neb.star_cell[s][i])
                src.pos[i] = float(neb.star_pos[s][i])
            src.n_packets = int(neb.n_packets[s])
            src.delta_e = float(neb.delta_e[s])
            src.spec_cdf = fp(dev(neb.spec_cdf[s]))
        self.nsrc = ns
        self.jste = torch.zeros((neb.nbins, neb.ncells + 1), dtype=torch.float64, device="cuda")
        self.esc = torch.zeros((neb.nbins + 1, neb.ncells + 1), dtype=torch.float64, device="cuda")


def _run_noalloc(lib, dn, seed):
    opts = abi.make_opts(seed=seed, precision=abi.MC_PREC_FP64, run_flags=abi.MC_RUN_ZERO_FIRST)
    st = abi.McStats()
    dp = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_double))
    rc = lib.mc_transport_run_noalloc(C.byref(dn.grid), dn.sources, dn.nsrc, C.byref(opts), dp(dn.jste), None,
                                      dp(dn.esc), C.byref(st), None)
    assert rc == 0, lib.mc_last_error().decode()
    return dn.jste.cpu().numpy(), dn.esc.cpu().numpy(), st.as_dict()


@pytest.mark.parametrize("case", [1, 2, 4], ids=lambda i: nebula.small_cases()[i].name)
def test_noalloc_matches_the_allocating_entry_point_twice(case):
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[case])
    dn = DeviceNebula(neb)
    for seed in (31, 32):
        js, es, st = _run_noalloc(lib, dn, seed)
        rjs, _, res, rst = transport.energy_packet_driver(neb, precision="fp64", seed=seed, form="plain")
        for k in KEYS:
            assert st[k] == rst[k], (k, st[k], rst[k])
        assert np.abs(js - rjs).max() <= RTOL * np.abs(rjs).max()
        assert np.abs(es - res).max() <= RTOL * np.abs(res).max()


def test_noalloc_rejects_grids_beyond_its_scratch():
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[0])
    dn = DeviceNebula(neb)
    dn.grid.nx = 1025
    opts = abi.make_opts(seed=1, precision=abi.MC_PREC_FP64)
    st = abi.McStats()
    dp = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_double))
    rc = lib.mc_transport_run_noalloc(C.byref(dn.grid), dn.sources, dn.nsrc, C.byref(opts), dp(dn.jste), None,
                                      dp(dn.esc), C.byref(st), None)
    assert rc == 7  # MC_ERR_UNSUPPORTED
    assert b"1024" in lib.mc_last_error()
