"""The cell update with grains (photoelectric heating and gas-grain
collisions, source/update_mod.f90:527-930) on the GPU against the FP64
oracle on the GPU's own Jste and moments, on the two small dusty nebulae:

- FP64 form: Te, Ne and the ion fractions to 1e-9, the T-step counts and
  the balance flags exactly, each size's grain potential, photoelHeat_d and
  gasDustColl_d to 1e-9 (the potential where the secant converged;
  photon-free cells stop where their capture currents cancel, a decision
  the last bit of the sum makes, so there the flag may differ and the
  potential agrees to 1e-6 Ryd);
- a second update with the grain temperatures the first one led to (the
  collision terms use them), and getDustT with gasDustColl_d - photoelHeat_d
  added to the absorbed integrals;
- FP32 form: Te within the reference's 1 % thermal tolerance of the FP64
  oracle for most cells;
- switching the grains off gives the gas-only update back, bit for bit."""
import numpy as np
import pytest

from mocassin_gb300 import balance, dust, nebula, transport
from oracle import dust_oracle
from oracle import update_runner as U

pytestmark = pytest.mark.gpu

CASES = [nebula.small_cases()[i] for i in (3, 4)]
RTOL = 1e-9


def _ions():
    return [tuple(int(v) for v in r) for r in nebula.atomic_table()["ions"]]


def _setup(spec, seed=4):
    neb = nebula.build(spec)
    ctx = transport.TransportContext(neb)
    ctx.run(seed=seed, precision="fp64")
    ctx.set_update_tables(balance.tables(), neb.hden, balance.abundances())
    te, ne, X = balance.initial_state(neb)
    ctx.set_cell_state(te, ne, X)
    w = balance.moment_weights(neb.xs, neb.nu, _ions())
    gp = dust.grain_physics(neb)
    ctx.set_grain_physics(gp)
    return neb, ctx, (te, ne, X), w, gp


def _oracle(neb, ctx, state, w, gp, tdust=None):
    mom, _ = ctx.jste_moments(w, 1e-9)
    js, _, _ = ctx.download()
    photo = mom[1:34].T.astype(np.float64)
    heat = mom[34:67].T.astype(np.float64)
    hit = (mom[0] > 0).astype(np.int32)
    te, ne, X = state
    o = U.update_cells(balance.tables(), balance.abundances(), neb.hden, photo, heat, hit, te, ne, X,
                       grains=(gp, js * 1e-9, gp["ndust"], tdust))
    return o, hit, js


def _compare(neb, g, o, gstate, hit, js):
    gte, gne, gX, gconv, gniter, gflags = g
    ote, one, oX, oconv, oniter, oflags, gout = o
    cells = np.nonzero(hit[1:])[0] + 1
    lit = cells[(js[neb.nu > dust.GRAIN_VN][:, cells] > 0).any(0)]
    np.testing.assert_array_equal(gniter[cells], oniter[cells])
    np.testing.assert_array_equal(gflags[cells] & 7, oflags[cells] & 7)
    np.testing.assert_array_equal(gflags[lit] & 8, oflags[lit] & 8)
    np.testing.assert_array_equal(gconv[cells], oconv[cells])
    np.testing.assert_allclose(gte[cells], ote[cells], rtol=RTOL)
    np.testing.assert_allclose(gne[cells], one[cells], rtol=RTOL)
    np.testing.assert_allclose(gX[cells], oX[cells], rtol=RTOL, atol=1e-30)
    pot, pd, cd = gstate
    np.testing.assert_allclose(pot[:, lit], gout[0][:, lit], rtol=RTOL, atol=1e-12)
    np.testing.assert_allclose(pot[:, cells], gout[0][:, cells], rtol=0, atol=1e-6)
    np.testing.assert_allclose(pd[:, cells], gout[1][:, cells], rtol=RTOL, atol=1e-300)
    np.testing.assert_allclose(cd[:, cells], gout[2][:, cells], rtol=1e-7)
    np.testing.assert_allclose(cd[:, lit], gout[2][:, lit], rtol=RTOL)
    return cells, lit


@pytest.mark.parametrize("spec", CASES, ids=lambda s: s.name)
def test_fp64_update_with_grains_matches_oracle(gpu_lib, spec):
    neb, ctx, state, w, gp = _setup(spec)
    o, hit, js = _oracle(neb, ctx, state, w, gp)
    st = ctx.update_cells(w, 1e-9)
    g = ctx.get_cell_state()
    gs = ctx.grain_state()
    cells, lit = _compare(neb, g, o, gs, hit, js)
    assert st["hit"] == len(cells) and len(lit) > 10
    # the grain temperatures of this iteration (getDustT with the grain terms)
    xs, gw, _ = dust.grains(neb.nu)
    em = dust.emission_table(xs, neb.nu)
    wab = dust.absorption_weights(xs)
    td, _ = ctx.dust_temperatures(wab, em, gw, 1e-9)
    absorbed = wab.T.astype(np.float64) @ (js * 1e-9) + gs[2] - gs[1]
    ref = dust_oracle.dust_temperatures(absorbed, em.astype(np.float32).astype(np.float64), gw, hit > 0)
    np.testing.assert_allclose(td[:, cells], ref[:, cells], rtol=2e-4)
    # a second update from the new state with these grain temperatures
    state2 = ctx.get_cell_state()[:3]
    o2, hit2, js2 = _oracle(neb, ctx, state2, w, gp, tdust=td[1:].astype(np.float64))
    ctx.update_cells(w, 1e-9)
    _compare(neb, ctx.get_cell_state(), o2, ctx.grain_state(), hit2, js2)
    ctx.close()


def test_fp32_update_with_grains(gpu_lib):
    neb, ctx, state, w, gp = _setup(CASES[0])
    o, hit, _ = _oracle(neb, ctx, state, w, gp)
    ctx.update_cells(w, 1e-9, precision="fp32")
    gte = ctx.get_cell_state()[0]
    pot = ctx.grain_state()[0]
    ctx.close()
    c = np.nonzero(hit[1:])[0] + 1
    d = np.abs(gte[c] / o[0][c] - 1)
    assert np.median(d) < 2e-3 and np.percentile(d, 95) < 3e-2, (np.median(d), np.percentile(d, 95))
    dp = np.abs(pot[:, c] - o[6][0][:, c])
    assert np.percentile(dp, 90) < 5e-3, np.percentile(dp, 90)


def test_grains_off_restores_the_gas_update(gpu_lib):
    neb, ctx, state, w, gp = _setup(CASES[0])
    ctx.set_grain_physics(None)
    ctx.update_cells(w, 1e-9)
    a = ctx.get_cell_state()
    ctx.close()
    neb2 = nebula.build(CASES[0])
    ctx2 = transport.TransportContext(neb2)
    ctx2.run(seed=4, precision="fp64")
    ctx2.set_update_tables(balance.tables(), neb2.hden, balance.abundances())
    ctx2.set_cell_state(*state)
    ctx2.update_cells(w, 1e-9)
    b = ctx2.get_cell_state()
    ctx2.close()
    for k in range(6):
        np.testing.assert_array_equal(a[k], b[k])


def test_grain_physics_argument_checks(gpu_lib):
    neb = nebula.build(CASES[0])
    ctx = transport.TransportContext(neb)
    gp = dust.grain_physics(neb)
    bad = dict(gp, radius_um=np.zeros_like(gp["radius_um"]))
    with pytest.raises(transport.TransportError):
        ctx.set_grain_physics(bad)
    with pytest.raises(transport.TransportError):
        ctx.grain_state()
    ctx.set_grain_physics(gp)
    with pytest.raises(transport.TransportError):
        ctx.grain_state()  # no update has run yet
    ctx.close()


def test_sublimated_grains_leave_the_opacity_and_scattering(gpu_lib):
    """The opacity rebuild adds each size bin's grains (weight x Ndust x
    (abs + sca)) and rebuilds the scattering table from the same sizes, for
    the sizes whose grain temperature is below the sublimation temperature
    (iteration_mod.f90:193-210): against a float64 restatement, with a
    threshold that half of the (size, cell) temperatures pass."""
    neb, ctx, state, w, gp = _setup(CASES[0])
    ctx.update_cells(w, 1e-9)
    xs_abs, gw, _ = dust.grains(neb.nu)
    td, _ = ctx.dust_temperatures(dust.absorption_weights(xs_abs), dust.emission_table(xs_abs, neb.nu), gw, 1e-9)
    ext, sca, wgt = dust.grain_opacity(neb.nu)
    lit = td[1:, 1:][td[1:, 1:] > 0]
    tsub = float(np.median(lit))
    ctx.set_grain_opacity(ext, sca, wgt, neb.ndust, tsub)
    ions = _ions()
    ctx.opacity_from_state(np.array(ions, dtype=np.int32), neb.xs, method="fp32")
    op, sc = ctx.get_opacity().astype(np.float64), ctx.get_scattering().astype(np.float64)
    X = ctx.get_cell_state()[2]
    ctx.close()
    den = balance.opacity_species(X, neb.hden.astype(np.float64), ions).astype(np.float64)
    keep = td[1:] < tsub                                   # (sizes, cells)
    assert 0.2 < keep[:, 1:].mean() < 0.8
    dd = keep * wgt[:, None].astype(np.float64) * neb.ndust[None, :].astype(np.float64)
    dd[:, 0] = 0.0
    ref_op = (den.T @ neb.xs.astype(np.float64)).T + (dd.T @ ext.astype(np.float64)).T
    ref_sc = (dd.T @ sca.astype(np.float64)).T
    c = np.arange(1, neb.ncells + 1)
    np.testing.assert_allclose(op[:, c], ref_op[:, c], rtol=2e-6, atol=1e-30)
    np.testing.assert_allclose(sc[:, c], ref_sc[:, c], rtol=2e-6, atol=1e-30)
    # with every size kept, the grains' rows add up to the grid's own dust opacity
    assert np.allclose((wgt[:, None] * ext).sum(0), neb.dust_kappa, rtol=1e-5)
