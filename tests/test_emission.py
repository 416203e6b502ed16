"""The diffuse-emission CDF (recPDF rows and totalLines, setDiffusePDF):
the CPU oracle's known answers and properties, the C-ABI struct, and the
GPU kernels against the oracle on the same cell states."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

from mocassin_gb300 import abi, balance, emission, nebula
from oracle import emission_oracle as EO
from oracle import update_runner

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_two_photon_distribution_is_normalised():
    # two photons per decay: the integral of A(y) over y is twice A(2s -> 1s) = 8.2249 / s
    y = np.linspace(0.0, 1.0, 400001)
    a = EO.two_photon_ay(y)
    assert abs(np.trapezoid(a, y) / (2 * 8.2249) - 1) < 5e-4
    np.testing.assert_allclose(a, a[::-1], rtol=1e-12, atol=1e-12)


def test_gaunt_factor_known_values():
    dd = EO.tables()["gaunt_dd"]
    # hnu << kT: the classical (Coulomb-logarithm) regime grows as nu falls
    lnu = np.log10(np.array([1e-5, 1e-3, 1e-1, 1.0, 10.0]))
    g = EO.gaunt(0.0, 4.0, lnu, dd)
    assert np.all(np.diff(g) < 0), g
    assert 1.0 < g[3] < 1.6 and g[0] > 4.0, g
    # He++ (Z = 2) has larger gamma^2, hence a different value at the same u
    g2 = EO.gaunt(0.30103, 4.0, lnu, dd)
    assert not np.allclose(g, g2)


def test_edge_pointers_pair_distinct_bins():
    t = EO.tables()
    nu = nebula.atomic_table()["nu"]
    for k in ("nu_gamma_hi", "nu_gamma_hei", "nu_gamma_heii"):
        ep = EO.edge_pointers(nu, t[k])
        assert ep[0] == 1 and np.all(np.diff(ep) >= 0)
        assert np.all(ep[1::2] > ep[0::2]), k  # fb_ff stops on a pair in one bin


def _state(n=21, seed=3):
    neb = nebula.build(nebula.small_cases()[0]) if n == 21 else None
    te, ne, X = balance.initial_state(neb)
    rng = np.random.default_rng(seed)
    # spread the state so every branch is visited: Te 3e3..3e4 K, Ne across the HeI-line density brackets
    nc1 = neb.ncells + 1
    te = 10 ** rng.uniform(3.5, 4.5, nc1)
    ne = 10 ** rng.uniform(0.0, 6.5, nc1)
    Xr = X.copy()
    for e, z in enumerate(balance.ELEMENTS):
        ns = min(z + 1, 7)
        f = rng.dirichlet(np.ones(ns), nc1)
        Xr[:, e, 1:ns + 1] = np.clip(f, 1e-20, 0.99999)
    return neb, te, ne, Xr


def test_oracle_rows_are_cdfs():
    neb, te, ne, X = _state()
    c = np.arange(1, 60)
    cdf, tl = EO.for_cells(te[c], ne[c], X[c], balance.abundances())
    assert np.all(np.diff(cdf, axis=1) >= 0)
    assert np.all(cdf[:, -1] == 1.0) and np.all(cdf >= 0) and np.all(cdf <= 1)
    assert np.all((tl > 0) & (tl < 1))


def test_emission_tables_struct_layout():
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "mocassin_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(mc_emission_tables_t), offsetof(mc_emission_tables_t, ntk),
         offsetof(mc_emission_tables_t, gaunt_dd), offsetof(mc_emission_tables_t, n_heavy),
         offsetof(mc_emission_tables_t, xs_outer));
  printf("%zu\n", sizeof(mc_update_stats_t));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        cf = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(cf, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), cf, "-o", exe])
        v = list(map(int, subprocess.check_output([exe]).decode().split()))
    T = abi.McEmissionTables
    assert v == [C.sizeof(T), T.ntk.offset, T.gaunt_dd.offset, T.n_heavy.offset, T.xs_outer.offset,
                 C.sizeof(abi.McUpdateStats)]


def _gpu_emission(neb, te, ne, X):
    from mocassin_gb300 import transport
    ctx = transport.TransportContext(neb)
    ctx.set_update_tables(balance.tables(), neb.hden, balance.abundances())
    ctx.set_cell_state(te, ne, X)
    ctx.set_emission_tables()
    ms = ctx.build_emission()
    rows, tl = ctx.get_emission()
    return ctx, rows, tl, ms


@pytest.mark.gpu
def test_gpu_emission_matches_oracle(gpu_lib):
    neb, te, ne, X = _state()
    ctx, rows, tl, ms = _gpu_emission(neb, te, ne, X)
    ctx.close()
    rng = np.random.default_rng(1)
    c = np.sort(rng.choice(np.arange(1, neb.ncells + 1), 400, replace=False))
    cdf, otl = EO.for_cells(te[c], ne[c], X[c], balance.abundances())
    # FP32 kernels against the FP64 oracle: CDF entries to 2e-5, the line fraction to 1e-4 relative
    d = np.abs(rows[c] - cdf)
    assert d.max() <= 2e-5, (d.max(), np.unravel_index(d.argmax(), d.shape))
    np.testing.assert_allclose(tl[c], otl, rtol=1e-4, atol=1e-7)
    assert np.all(rows[0] == 1.0)


@pytest.mark.gpu
def test_gpu_forbidden_line_totals_match_oracle(gpu_lib):
    # the line fraction is where the forbidden lines enter: pin it on cells where they dominate
    neb, te, ne, X = _state(seed=5)
    X[:, 0, 2] = 1e-4  # almost neutral H: little continuum, lines matter
    ctx, rows, tl, _ = _gpu_emission(neb, te, ne, X)
    ctx.close()
    c = np.arange(1, 200)
    forb = update_runner.forbidden_lines(balance.tables(), balance.abundances(), te[c], ne[c], X[c])
    _, otl = EO.diffuse_pdf(te[c], ne[c], X[c], balance.abundances(), forb)
    np.testing.assert_allclose(tl[c], otl, rtol=1e-4, atol=1e-7)


@pytest.mark.gpu
def test_gpu_emission_full_size_rows_are_cdfs(gpu_lib):
    import dataclasses
    neb = nebula.build(dataclasses.replace(nebula.clumpy61(1000), name="clumpy61"))
    te, ne, X = balance.initial_state(neb)
    ctx, rows, tl, ms = _gpu_emission(neb, te, ne, X)
    ctx.close()
    r = rows[1:]
    assert np.all(np.diff(r, axis=1) >= 0) and np.all(r[:, -1] == 1.0) and np.all(r >= 0)
    assert np.all((tl[1:] > 0) & (tl[1:] < 1))
    print("emission build 61^3: %.3f ms" % ms)


@pytest.mark.gpu
def test_lambda_iteration_rebuilds_the_emission_cdfs(gpu_lib):
    """The Lambda iteration builds the CDFs from the initial state before the
    first transport and again after every update: the resident rows are the
    oracle's for the state the update left."""
    import dataclasses
    from mocassin_gb300 import iterate
    neb = nebula.build(dataclasses.replace(nebula.clumpy61(300_000), name="clumpy21", n=21))
    li = iterate.LambdaIteration(neb, form="graph", update="fp32")
    assert li.emission
    rows0, tl0 = li.ctx.get_emission()
    _, hist = li.run(seed=3, max_iterations=2, min_convergence=101.0)
    rows, tl = li.ctx.get_emission()
    te, ne, X = li.ctx.get_cell_state()[:3]
    li.close()
    assert all(h["emission_ms"] > 0 for h in hist)
    c = np.arange(1, neb.ncells + 1, 37)
    cdf, otl = EO.for_cells(te[c], ne[c], X[c], balance.abundances())
    assert np.abs(rows[c] - cdf).max() <= 2e-5
    np.testing.assert_allclose(tl[c], otl, rtol=1e-4, atol=1e-7)
    assert not np.array_equal(tl, tl0)


def _dusty(n=21, packets=300_000, gas=True):
    import dataclasses
    neb = nebula.build(dataclasses.replace(nebula.dusty81(packets), name="dusty%d" % n, n=n))
    if not gas:
        neb = dataclasses.replace(neb, flags=neb.flags & ~nebula.FLAG_GAS)
    return neb


def _grain_temperatures(ctx, neb):
    from mocassin_gb300 import dust
    xs_abs, w, _ = dust.grains(neb.nu)
    td, _ = ctx.dust_temperatures(dust.absorption_weights(xs_abs), dust.emission_table(xs_abs, neb.nu), w, 1e-9)
    return td


@pytest.mark.gpu
def test_gpu_emission_with_grains_matches_oracle(gpu_lib):
    """A gas grid with grains: the thermal grain emission at the grain
    temperatures the GPU left joins the recPDF rows (sumDiffuseDust)."""
    from mocassin_gb300 import dust, transport
    neb = _dusty()
    ctx = transport.TransportContext(neb)
    ctx.run(seed=4, precision="fp32", zero_first=True)
    td = _grain_temperatures(ctx, neb)
    ctx.set_update_tables(balance.tables(), neb.hden, balance.abundances())
    te, ne, X = balance.initial_state(neb)
    ctx.set_cell_state(te, ne, X)
    ctx.set_emission_tables()
    ctx.build_emission()
    rows, tl = ctx.get_emission()
    ctx.close()
    hit = np.nonzero(td[1] > 0)[0]
    assert len(hit) > 100
    c = np.sort(np.random.default_rng(2).choice(hit[hit > 0], 200, replace=False))
    xs_abs, w, _ = dust.grains(neb.nu)
    d = {"tdust": td[1:, c].T.astype(np.float64), "xs_abs": xs_abs, "gw": w, "t_sub": emission.T_SUBLIME,
         "ndust_over_hden": neb.ndust[c].astype(np.float64) / neb.hden[c].astype(np.float64)}
    forb = update_runner.forbidden_lines(balance.tables(), balance.abundances(), te[c], ne[c], X[c])
    cdf, otl = EO.diffuse_pdf(te[c], ne[c], X[c], balance.abundances(), forb, dust=d)
    cdf0, _ = EO.diffuse_pdf(te[c], ne[c], X[c], balance.abundances(), forb)
    assert np.abs(cdf - cdf0).max() > 1e-3  # the grains change the rows
    assert np.abs(rows[c] - cdf).max() <= 2e-5
    np.testing.assert_allclose(tl[c], otl, rtol=1e-4, atol=1e-7)


@pytest.mark.gpu
def test_gpu_dust_only_grid_builds_dust_pdf(gpu_lib):
    """A dust-only grid: the dustPDF rows of setDustPDF from the grain
    temperatures alone (no cell state, no update tables)."""
    from mocassin_gb300 import dust, transport
    neb = _dusty(gas=False)
    ctx = transport.TransportContext(neb)
    ctx.run(seed=4, precision="fp32", zero_first=True)
    td = _grain_temperatures(ctx, neb)
    ctx.set_emission_tables()
    ctx.build_emission()
    rows = ctx.get_dust_emission()
    ctx.close()
    xs_abs, w, _ = dust.grains(neb.nu)
    c = np.arange(1, neb.ncells + 1, 23)
    cdf = EO.dust_pdf(td[1:, c].T.astype(np.float64), xs_abs, w, emission.T_SUBLIME)
    assert np.abs(rows[c] - cdf).max() <= 2e-5
    assert np.all(np.diff(rows[1:], axis=1) >= 0) and np.all(rows[1:, -1] == 1.0)


@pytest.mark.gpu
def test_lambda_iteration_on_a_dusty_grid(gpu_lib):
    """The Lambda iteration of a gas grid with grains keeps the grain opacity
    in every rebuild, follows the grain temperatures and builds the CDFs with
    their thermal emission."""
    from mocassin_gb300 import iterate, transport
    neb = _dusty(n=21, packets=300_000)
    li = iterate.LambdaIteration(neb, form="graph", update="fp32")
    _, hist = li.run(seed=5, max_iterations=2, min_convergence=101.0)
    op = li.ctx.get_opacity()
    rows, tl = li.ctx.get_emission()
    li.close()
    # opacity = gas contraction + Ndust x kappa_d: at the lowest frequencies the grains dominate
    kd = neb.ndust[1:].astype(np.float64) * neb.dust_kappa[0]
    np.testing.assert_allclose(op[0, 1:], kd, rtol=2e-3)
    assert np.all(np.diff(rows[1:], axis=1) >= 0) and np.all(rows[1:, -1] == 1.0)
    assert len(hist) == 2 and all(h["emission_ms"] > 0 for h in hist)


@pytest.mark.gpu
def test_line_totals_kept_by_the_update_are_the_recomputed_ones(gpu_lib):
    """After an FP32 update the emission build takes the forbidden-line totals
    of each cell's last T step instead of solving the level populations again;
    the rows and line fractions are bit-identical to a build that recomputes
    every cell (after the same state is set again)."""
    import dataclasses
    from mocassin_gb300 import transport
    neb = nebula.build(dataclasses.replace(nebula.clumpy61(400_000), name="clumpy21", n=21))
    ctx = transport.TransportContext(neb)
    ctx.set_update_tables(balance.tables(), neb.hden, balance.abundances())
    te, ne, X = balance.initial_state(neb)
    ctx.set_cell_state(te, ne, X)
    ctx.set_emission_tables()
    ions = [tuple(int(v) for v in r) for r in nebula.atomic_table()["ions"]]
    w = balance.moment_weights(neb.xs, neb.nu, ions)
    ctx.build_emission()
    ctx.run(seed=8, precision="fp32", zero_first=True)
    ctx.update_cells(w, 1e-9, precision="fp32")
    ctx.build_emission()
    rows1, tl1 = ctx.get_emission()
    s = ctx.get_cell_state()
    ctx.set_cell_state(s[0], s[1], s[2])
    ctx.build_emission()
    rows2, tl2 = ctx.get_emission()
    ctx.close()
    np.testing.assert_array_equal(tl1, tl2)
    np.testing.assert_array_equal(rows1, rows2)
