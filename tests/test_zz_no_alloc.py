"""mc_transport_run_noalloc: the transport for callers that cannot allocate.

Some callers cannot call cudaMalloc (a code that only hands over device
memory it already manages, a loop where an allocation could block or fail).
This entry point takes every array as a device pointer the caller owns and
allocates nothing itself.  Here the test plays such a caller: it owns the
device arrays (torch tensors) and checks, on two calls in a row, that the
results equal those of the existing entry point mc_transport_run in its
plain form on the same draws -- counters exactly, Jste / escapedPackets to
1e-12 relative (FP64 march) -- so state kept in the shared scratch between
calls cannot leak into a result.  It also checks the FP64 results against
the CPU oracle directly, the FP32 march against the FP64 oracle within 3
sigma of packet noise, and that every rejected call (negative or too large
`active` entries, a source outside the grid, too many sources, a missing
array) returns before it writes the caller's estimators and leaves the
shared scratch fit for the next valid call.
"""
import ctypes as C

import numpy as np
import pytest

from mocassin_gb300 import abi, nebula, transport
from oracle import runner

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
        self.active = dev(neb.active, np.int32)
        g.active = C.cast(self.active.data_ptr(), C.POINTER(C.c_int32))
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


def _call(lib, dn, seed, precision=abi.MC_PREC_FP64, n_packets=None, nsrc=None):
    if n_packets is not None:
        for s in range(dn.nsrc):
            dn.sources[s].n_packets = int(n_packets)
    opts = abi.make_opts(seed=seed, precision=precision, run_flags=abi.MC_RUN_ZERO_FIRST)
    st = abi.McStats()
    dp = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_double))
    rc = lib.mc_transport_run_noalloc(C.byref(dn.grid), dn.sources, dn.nsrc if nsrc is None else nsrc,
                                      C.byref(opts), dp(dn.jste), None, dp(dn.esc), C.byref(st), None)
    return rc, st


def _run_noalloc(lib, dn, seed, precision=abi.MC_PREC_FP64, n_packets=None):
    rc, st = _call(lib, dn, seed, precision, n_packets)
    assert rc == 0, lib.mc_last_error().decode()
    return dn.jste.cpu().numpy(), dn.esc.cpu().numpy(), st.as_dict()


def _matches_allocating_call(lib, dn, neb, seed):
    js, es, st = _run_noalloc(lib, dn, seed)
    rjs, _, res, rst = transport.energy_packet_driver(neb, precision="fp64", seed=seed, form="plain")
    for k in KEYS:
        assert st[k] == rst[k], (k, st[k], rst[k])
    assert np.abs(js - rjs).max() <= RTOL * np.abs(rjs).max()
    assert np.abs(es - res).max() <= RTOL * np.abs(res).max()


@pytest.mark.parametrize("case", [1, 2, 4], ids=lambda i: nebula.small_cases()[i].name)
def test_noalloc_matches_the_allocating_entry_point_twice(case):
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[case])
    dn = DeviceNebula(neb)
    for seed in (31, 32):
        _matches_allocating_call(lib, dn, neb, seed)


def test_noalloc_fp64_equals_the_oracle():
    """FP64 march on the oracle's draws: counters exactly, Jste and
    escapedPackets to 1e-12 relative, without the allocating entry point in
    between."""
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[3])
    dn = DeviceNebula(neb)
    js, es, st = _run_noalloc(lib, dn, 23)
    ojs, _, oes, ost = runner.run(neb, precision="fp64", seed=23)
    for k in KEYS:
        assert st[k] == ost[k], (k, st[k], ost[k])
    assert np.abs(js - ojs).max() <= RTOL * np.abs(ojs).max()
    assert np.abs(es - oes).max() <= RTOL * np.abs(oes).max()


def test_noalloc_fp32_march_agrees_with_the_fp64_oracle():
    """FP32 instantiation: band-integrated J per cell over 8 seeds against the
    FP64 oracle on other seeds; the difference of the means stays within 3
    sigma (batch means) for the grid total and for >= 97 % of well-sampled
    cells, and every packet is accounted for."""
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[1])
    dn = DeviceNebula(neb)
    g, o = [], []
    for seed in range(1, 9):
        js, _, st = _run_noalloc(lib, dn, seed, precision=abi.MC_PREC_FP32, n_packets=3000)
        assert st["escaped"] + st["lines"] + st["trapped"] == 3000 * dn.nsrc
        g.append(js.sum(0))
        o.append(runner.run(neb, n_packets=3000, precision="fp64", seed=100 + seed)[0].sum(0))
    g, o = np.array(g), np.array(o)
    sig = np.sqrt(g.var(0, ddof=1) / len(g) + o.var(0, ddof=1) / len(o))
    d = np.abs(g.mean(0) - o.mean(0))
    tot_sig = np.sqrt(g.sum(1).var(ddof=1) / len(g) + o.sum(1).var(ddof=1) / len(o))
    assert abs(g.sum(1).mean() - o.sum(1).mean()) < 3 * tot_sig
    ok = sig > 0.02 * o.mean(0).clip(1e-300)
    assert float(np.mean(d[ok] < 3 * sig[ok])) >= 0.97


SENTINEL = 7.0


def _rejected_without_writing(lib, dn, expect, **kw):
    dn.jste.fill_(SENTINEL)
    dn.esc.fill_(SENTINEL)
    rc, _ = _call(lib, dn, 5, **kw)
    assert rc == expect, (rc, lib.mc_last_error())
    import torch
    torch.cuda.synchronize()
    assert bool((dn.jste == SENTINEL).all()) and bool((dn.esc == SENTINEL).all())


def test_noalloc_rejects_subgrid_and_out_of_range_active_before_any_write():
    """A negative `active` entry (a sub-grid pointer) is MC_ERR_UNSUPPORTED
    and one above ncells MC_ERR_ARG, as mc_transport_run reports them; the
    call returns before the march or the ZERO_FIRST clear touches the
    caller's arrays, and the next valid call still matches the allocating
    entry point."""
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[1])
    dn = DeviceNebula(neb)
    good = dn.active.clone()
    flat = dn.active.view(-1)
    flat[flat.numel() // 2] = -3
    _rejected_without_writing(lib, dn, 7)
    assert b"sub-grid" in lib.mc_last_error()
    dn.active.copy_(good)
    flat[5] = neb.ncells + 1
    _rejected_without_writing(lib, dn, 1)
    assert b"exceeds ncells" in lib.mc_last_error()
    dn.active.copy_(good)
    _matches_allocating_call(lib, dn, neb, 44)


def test_noalloc_argument_errors_leave_the_estimators_and_scratch_intact():
    """A source outside the grid (MC_ERR_BOUNDS), 17 sources and a missing
    opacity array are rejected before the ZERO_FIRST clear; after each, a
    valid call matches the allocating entry point."""
    lib = _lib()
    neb = nebula.build(nebula.small_cases()[2])
    dn = DeviceNebula(neb)
    cell0 = tuple(dn.sources[0].cell)
    dn.sources[0].cell[0] = neb.nx + 1
    _rejected_without_writing(lib, dn, 3)
    for i in range(3):
        dn.sources[0].cell[i] = cell0[i]
    _matches_allocating_call(lib, dn, neb, 45)
    _rejected_without_writing(lib, dn, 7, nsrc=17)
    _matches_allocating_call(lib, dn, neb, 46)
    op = C.cast(dn.grid.opacity, C.c_void_p).value  # the address (a field read shares the struct's memory)
    dn.grid.opacity = C.cast(None, C.POINTER(C.c_float))
    _rejected_without_writing(lib, dn, 1)
    dn.grid.opacity = C.cast(op, C.POINTER(C.c_float))
    _matches_allocating_call(lib, dn, neb, 47)


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
