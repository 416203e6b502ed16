"""CPU-side checks of the C-ABI: struct layout and exported symbols.

No compute call is made (no GPU here): the library is loaded and every
function declared in include/mocassin_gpu.h must be exported.
"""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from mocassin_gb300 import abi, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mocassin_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(mc_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_the_boundary():
    fns = declared_functions()
    for f in ("mc_transport_run", "mc_ctx_create", "mc_ctx_run", "mc_ctx_download", "mc_last_error"):
        assert f in fns


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(build.build())
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing
    lib.mc_abi_version.restype = C.c_int
    assert lib.mc_abi_version() == 2


def test_struct_layout_matches_ctypes():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "mocassin_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu\n", sizeof(mc_grid_t), sizeof(mc_source_t), sizeof(mc_run_opts_t), sizeof(mc_stats_t));
  printf("%zu %zu %zu %zu\n", offsetof(mc_grid_t, geo_corr), offsetof(mc_grid_t, flags),
         offsetof(mc_source_t, spec_cdf), offsetof(mc_run_opts_t, replay_stride));
  printf("%zu %zu %zu\n", offsetof(mc_stats_t, qphot), offsetof(mc_stats_t, error_packet),
         offsetof(mc_stats_t, d2h_bytes));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    vals = list(map(int, out))
    assert vals[:4] == [C.sizeof(abi.McGrid), C.sizeof(abi.McSource), C.sizeof(abi.McRunOpts),
                        C.sizeof(abi.McStats)]
    assert vals[4] == abi.McGrid.geo_corr.offset and vals[5] == abi.McGrid.flags.offset
    assert vals[6] == abi.McSource.spec_cdf.offset and vals[7] == abi.McRunOpts.replay_stride.offset
    assert vals[8] == abi.McStats.qphot.offset and vals[9] == abi.McStats.error_packet.offset
    assert vals[10] == abi.McStats.d2h_bytes.offset


def test_product_path_has_no_cpu_fallback(monkeypatch):
    """Without the built library the transport raises; it never falls back."""
    from mocassin_gb300 import transport
    monkeypatch.setattr(transport, "LIB_PATH", "/nonexistent/libmcgpu.so")
    monkeypatch.setattr(transport, "_LIB", None)
    with pytest.raises(transport.TransportError):
        transport.library()
