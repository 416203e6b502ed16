"""GPU opacity build (dense addOpacity + dust add) against the FP64 oracle.

FP32 CUDA-core path: 2e-6 relative per element.  Tensor-core path (tcgen05,
two-term split BF16, FP32 accumulate): 3e-5 relative per element (all terms
are non-negative, so the missing lo*lo term bounds the error by ~1.5e-5).
The 70001-cell shape gives each CTA of the pipelined kernel several cell
tiles (its double-buffered accumulators and overlapped stores).
"""
import numpy as np
import pytest

from mocassin_gb300 import nebula, transport
from oracle import opacity_oracle, runner
from tests import helpers

pytestmark = pytest.mark.gpu

TOL = {"fp32": 2e-6, "bf16x3": 3e-5}


def _case(k, nc1, nb, seed):
    rng = np.random.default_rng(seed)
    den = (rng.lognormal(0.0, 3.0, (k, nc1)) * (rng.random((k, nc1)) > 0.1)).astype(np.float32)
    den[:, 0] = 0.0
    xs = (rng.lognormal(-40.0, 2.0, (k, nb)) * (rng.random((k, nb)) > 0.3)).astype(np.float32)
    ff = rng.lognormal(-45.0, 1.0, nc1).astype(np.float32)
    return den, xs, ff


def _check(got, ref, tol):
    err = np.abs(got.astype(np.float64) - ref)
    bound = tol * np.abs(ref) + 1e-30
    assert np.all(err <= bound), float((err / (np.abs(ref) + 1e-300)).max())


@pytest.mark.parametrize("method", ["fp32", "bf16x3"])
@pytest.mark.parametrize("shape", [(16, 128, 128), (37, 1, 600), (37, 1000, 600), (47, 4097, 257), (64, 300, 33),
                                   (48, 70001, 600)])
def test_opacity_matches_oracle(gpu_lib, method, shape):
    k, nc1, nb = shape
    den, xs, ff = _case(k, nc1, nb, seed=nc1 + nb)
    got, ms = transport.opacity_build(den, xs, ff, method=method)
    _check(got, opacity_oracle.opacity(den, xs, ff), TOL[method])


@pytest.mark.parametrize("method", ["fp32", "bf16x3"])
def test_opacity_of_a_nebula(gpu_lib, method):
    neb = nebula.build(nebula.small_cases()[2])
    den = np.ascontiguousarray(neb.ion_den.T)
    got, _ = transport.opacity_build(den, neb.xs, None, method=method)
    ref = opacity_oracle.opacity(den, neb.xs)
    _check(got, ref, TOL[method])
    np.testing.assert_allclose(got[:, 1:], neb.opacity[:, 1:], rtol=TOL[method], atol=0)


def test_resident_opacity_build_feeds_the_transport(gpu_lib):
    """The context's opacity rebuilt on the GPU gives the same transport as
    the same table built by mc_opacity_build and uploaded."""
    neb = nebula.build(nebula.small_cases()[1])
    den = np.ascontiguousarray(neb.ion_den.T)
    op, _ = transport.opacity_build(den, neb.xs, None, method="bf16x3")
    up = helpers.with_opacity(neb, op)
    a = transport.energy_packet_driver(up, precision="fp64", seed=4)
    ctx = transport.TransportContext(neb)
    ctx.build_opacity(den, neb.xs, None, method="bf16x3")
    ctx.run(seed=4, precision="fp64")
    js, _, es = ctx.download()
    ctx.close()
    assert helpers.rel_err(js, a[0]) < 1e-12 and helpers.rel_err(es, a[2]) < 1e-12
    # and it agrees with the FP64 oracle transport on the FP64 oracle opacity
    b = runner.run(up, precision="fp64", seed=4)
    assert helpers.rel_err(js, b[0]) < 1e-12


def test_opacity_rejects_bad_arguments(gpu_lib):
    den, xs, ff = _case(65, 10, 10, 1)
    with pytest.raises(transport.TransportError):
        transport.opacity_build(den, xs, ff)
