"""Jste moments on the GPU (photoionisation sums of updateCell) vs the FP64 oracle.

Tensor-core path (split BF16, FP32 accumulate): 3e-5 relative per element
(all terms non-negative).
"""
import numpy as np
import pytest

from mocassin_gb300 import nebula, rates, transport
from oracle import rates_oracle, runner

TOL = 3e-5


@pytest.mark.gpu
@pytest.mark.parametrize("spec", [nebula.small_cases()[1], nebula.small_cases()[2], nebula.small_cases()[3]],
                         ids=lambda s: s.name)
def test_photoionisation_sums_match_the_oracle(gpu_lib, spec):
    neb = nebula.build(spec)
    sym = bool(neb.flags & nebula.FLAG_SYMMETRIC_XYZ)
    ctx = transport.TransportContext(neb)
    ctx.run(seed=8, precision="fp64")
    js, _, _ = ctx.download()
    w = rates_oracle.photo_weights(neb.xs, neb.nu).astype(np.float32)
    scale = 1e-9 / (8.0 if sym else 1.0)
    got, ms = ctx.jste_moments(w, scale)
    nps = rates.n_photo(ctx, neb.xs, neb.nu, sym)
    ctx.close()
    onps = rates_oracle.n_photo(js, neb.xs, neb.nu, sym)
    assert np.all(np.abs(nps - onps) <= TOL * onps)
    ref = rates_oracle.moments(js, w, scale)
    err = np.abs(got.astype(np.float64) - ref)
    assert np.all(err <= TOL * np.abs(ref) + 1e-300), float((err / (np.abs(ref) + 1e-300)).max())
    # the FP64 oracle transport gives the same Jste, hence the same sums
    ojs = runner.run(neb, precision="fp64", seed=8)[0]
    np.testing.assert_allclose(rates_oracle.moments(ojs, w, scale), ref, rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("nout", [1, 16, 33, 64, 67, 128])
def test_moments_of_random_weights(gpu_lib, nout):
    neb = nebula.build(nebula.small_cases()[0])
    ctx = transport.TransportContext(neb)
    ctx.run(seed=3, precision="fp64")
    js, _, _ = ctx.download()
    w = np.random.default_rng(nout).lognormal(0, 2, (neb.nbins, nout)).astype(np.float32)
    got, _ = ctx.jste_moments(w, 0.5)
    ctx.close()
    ref = rates_oracle.moments(js, w, 0.5)
    err = np.abs(got.astype(np.float64) - ref)
    assert np.all(err <= TOL * np.abs(ref) + 1e-300)


def test_host_weight_table_matches_the_oracle_formula():
    neb = nebula.build(nebula.small_cases()[0])
    np.testing.assert_allclose(rates.photo_weights(neb.xs, neb.nu),
                               rates_oracle.photo_weights(neb.xs, neb.nu), rtol=1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("nout", [16, 67])
def test_moments_of_a_grid_of_many_tiles(gpu_lib, nout):
    """A 41^3 grid (539 tiles of 128 cells): the persistent CTAs take
    several tiles each (the accumulator reused from tile to tile), and two
    calls give the same sums."""
    import dataclasses
    neb = nebula.build(dataclasses.replace(nebula.clumpy61(300_000), name="clumpy41", n=41))
    ctx = transport.TransportContext(neb)
    ctx.run(seed=5, precision="fp32")
    js, _, _ = ctx.download()
    w = np.random.default_rng(100 + nout).lognormal(0, 2, (neb.nbins, nout)).astype(np.float32)
    got, _ = ctx.jste_moments(w, 0.25)
    again, _ = ctx.jste_moments(w, 0.25)
    ctx.close()
    ref = rates_oracle.moments(js, w, 0.25)
    err = np.abs(got.astype(np.float64) - ref)
    assert np.all(err <= TOL * np.abs(ref) + 1e-300), float((err / (np.abs(ref) + 1e-300)).max())
    np.testing.assert_array_equal(got, again)
