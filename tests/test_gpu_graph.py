"""The chosen form with its rounds inside one CUDA graph (MC_RUN_GRAPH) gives
the same transport as the host-driven rounds: the same draws, counters and
rounds; Jste to 1e-12 in FP64 (only the order of the FP64 sums may differ)
and to 1e-5 in FP32, where the warp-private FP32 accumulators flush in an
order that depends on scheduling."""
import numpy as np
import pytest

from mocassin_gb300 import nebula, transport
from oracle import runner
from tests import helpers

pytestmark = pytest.mark.gpu

KEYS = ("crossings", "absorptions", "scatterings", "escaped", "lines", "trapped", "silent_exits")


@pytest.mark.parametrize("spec", nebula.small_cases(), ids=lambda s: s.name)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_graph_rounds_match_host_rounds(gpu_lib, spec, precision):
    neb = nebula.build(spec)
    a = transport.energy_packet_driver(neb, precision=precision, seed=31, form="wave")
    b = transport.energy_packet_driver(neb, precision=precision, seed=31, form="graph")
    for k in KEYS:
        assert a[3][k] == b[3][k], k
    assert a[3]["rounds"] == b[3]["rounds"]
    tol = 1e-12 if precision == "fp64" else 1e-5
    assert helpers.rel_err(b[0], a[0]) < tol
    assert helpers.rel_err(b[2], a[2]) < tol
    if precision == "fp64":
        o = runner.run(neb, precision="fp64", seed=31)
        assert all(b[3][k] == o[3][k] for k in KEYS)
        assert helpers.rel_err(b[0], o[0]) < 1e-12


def test_graph_form_in_a_resident_context(gpu_lib):
    neb = nebula.build(nebula.small_cases()[2])
    ctx = transport.TransportContext(neb)
    r = [ctx.run(seed=5 + k, precision="fp32", zero_first=True, form="graph") for k in range(3)]
    ctx.close()
    assert all(x["rounds"] >= 2 and x["crossings"] > 0 for x in r)
