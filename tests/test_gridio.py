"""Grid snapshots in the reference's files (writeGrid / resetGrid)."""
import numpy as np
import pytest

from mocassin_gb300 import balance, gridio, nebula


def _state(neb, seed=1):
    rng = np.random.default_rng(seed)
    te, ne, X = balance.initial_state(neb)
    te = te * rng.uniform(0.5, 1.5, te.shape)
    X = X * rng.uniform(0.5, 1.0, X.shape)
    conv = rng.integers(0, 2, te.shape).astype(np.int32)
    black = rng.integers(0, 2, te.shape).astype(np.int32)
    return te, ne, X, conv, black


def test_round_trip(tmp_path):
    neb = nebula.build(nebula.small_cases()[2])
    te, ne, X, conv, black = _state(neb)
    gridio.write_grid(tmp_path, neb, te, ne, X, conv=conv, black=black)
    g = gridio.read_grid(tmp_path)
    assert (g["nx"], g["ny"], g["nz"], g["ncells"]) == (neb.nx, neb.ny, neb.nz, neb.ncells)
    np.testing.assert_array_equal(g["active"], neb.active)
    np.testing.assert_allclose(g["x_axis"], neb.x_axis, rtol=1e-8)
    c = np.arange(1, neb.ncells + 1)
    np.testing.assert_allclose(g["te"][c], te[c], rtol=1e-8)
    np.testing.assert_allclose(g["ne"][c], ne[c], rtol=1e-8)
    np.testing.assert_allclose(g["hden"][c], neb.hden[c], rtol=1e-7)
    np.testing.assert_array_equal(g["conv"][c], conv[c])
    np.testing.assert_array_equal(g["black"][c], black[c])
    for e, z in enumerate(balance.ELEMENTS):
        ns = min(z + 1, 7)
        np.testing.assert_allclose(g["X"][c, e, 1:ns + 1], X[c, e, 1:ns + 1], rtol=1e-8)


def test_record_layout_follows_write_grid(tmp_path):
    neb = nebula.build(nebula.small_cases()[0])
    te, ne, X, conv, black = _state(neb)
    td = np.tile(np.linspace(20, 80, 11)[:, None], (1, neb.ncells + 1))
    gridio.write_grid(tmp_path, neb, te, ne, X, conv=conv, black=black, tdust=td)
    n3 = neb.nx * neb.ny * neb.nz
    g0 = (tmp_path / "grid0.out").read_text().splitlines()
    assert len(g0) == 2 + neb.nx + neb.ny + neb.nz + n3
    assert [len(l.split()) for l in g0[:2]] == [1, 6]
    assert all(len(l.split()) == 3 for l in g0[-n3:])
    g1 = (tmp_path / "grid1.out").read_text().splitlines()
    assert len(g1) == n3 and all(len(l.split()) == 3 for l in g1)
    g2 = (tmp_path / "grid2.out").read_text().splitlines()
    assert len(g2) == n3 * 7
    assert [len(l.split()) for l in g2[:7]] == [2, 3, 7, 7, 7, 7, 7]
    gd = (tmp_path / "dustGrid.out").read_text().splitlines()
    assert len(gd) == n3 * (1 + 11)
    g = gridio.read_grid(tmp_path, dust_sizes=10)
    np.testing.assert_allclose(g["tdust"][:, 1:], td[:, 1:], rtol=1e-8)


@pytest.mark.gpu
def test_gpu_warm_restart_from_snapshot(gpu_lib, tmp_path):
    # the restored state and the opacity rebuilt from it match the model that
    # wrote the snapshot (to the 8 digits of the files)
    from mocassin_gb300 import iterate
    neb = nebula.build(nebula.small_cases()[2])
    a = iterate.LambdaIteration(neb, form="graph", update="fp64")
    a.step(seed=3, n_packets=20000)
    a.step(seed=4, n_packets=20000)
    a.write_grid(tmp_path)
    b = iterate.LambdaIteration(neb, form="graph", update="fp64")
    b.restart_from(tmp_path)
    sa, sb = a.state(), b.state()
    oa, ob = a.ctx.get_opacity(), b.ctx.get_opacity()
    a.close()
    b.close()
    c = np.arange(1, neb.ncells + 1)
    np.testing.assert_allclose(sb[0][c], sa[0][c], rtol=1e-7)
    np.testing.assert_allclose(sb[2][c], sa[2][c], rtol=1e-7, atol=1e-30)
    np.testing.assert_allclose(ob, oa, rtol=1e-5, atol=1e-30)


def test_model_parameters_round_trip(tmp_path):
    """grid3.out / photoSource.out in writeGrid's record order, read back as
    resetGrid reads them; the viewing angles come back shifted by one, as in
    the reference (written 0..nAngleBins, read into 1..nAngleBins)."""
    import dataclasses
    spec = dataclasses.replace(nebula.small_cases()[0], views=((0.5, 1.0), (1.2, -1.0)))
    neb = nebula.build(spec)
    p = gridio.model_parameters(neb, xhi_limit=0.02, max_iterate=12, min_convergence=90.0)
    gridio.write_parameters(str(tmp_path), p)
    q = gridio.read_parameters(str(tmp_path))
    for k in ("nGrids", "lgSymmetricXYZ", "nbins", "maxIterateMC", "lgDust", "lgGas", "nAngleBins", "nstages",
              "lgMultistars", "abundanceFile", "dustSpeciesFile", "nSizes", "lgEcho", "lgNosource"):
        assert q[k] == p[k], k
    for k in ("nuMax", "nuMin", "XHIlimit", "minConvergence", "R_in"):
        assert abs(q[k] - p[k]) <= 1e-7 * max(abs(p[k]), 1.0), k
    assert q["nbins"] == neb.nbins and q["XHIlimit"] == pytest.approx(0.02)
    assert q["viewPointTheta"][1:] == pytest.approx(p["viewPointTheta"][:2])
    src = open(tmp_path / "photoSource.out").read().split("\n")
    assert int(src[0].split()[0]) == len(spec.stars)


def test_summary_lines_follow_the_reference(tmp_path):
    """summary.out carries iterateMC's per-iteration lines (converged, no
    hit, no ion balance, no Te balance, total, packets)."""
    from mocassin_gb300 import iterate
    li = iterate.LambdaIteration.__new__(iterate.LambdaIteration)  # the history alone, no GPU context
    li.neb = nebula.build(nebula.small_cases()[0])
    li.history = [{"iteration": 1, "converged_pct": 12.5, "hit": li.neb.ncells // 2, "no_ion_balance": 3,
                   "no_te_balance": li.neb.ncells // 4}]
    li.write_summary(str(tmp_path))
    lines = [l for l in open(tmp_path / "summary.out").read().split("\n") if l]
    assert len(lines) == 6 and all("[Summary] Iteration" in l for l in lines)
    words = [" ".join(l.split()) for l in lines]
    assert "; 12% converged cells in grid 1" in words[0]
    assert "; 50% no hit cells in grid 1" in words[1]
    assert "; 50% Te balance not reached in grid 1" in words[3]
    assert "energy packets used" in words[5]
