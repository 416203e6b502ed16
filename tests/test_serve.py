"""Batched serving of independent nebulae (mocassin_gb300.serve)."""
import numpy as np
import pytest

from mocassin_gb300 import nebula, serve


def test_batch_specs_follow_the_distribution():
    sp = nebula.batch64()
    assert len(sp) == 64
    ns = np.array([s.n for s in sp])
    assert ns.min() >= 17 and ns.max() <= 65 and np.all(ns % 2 == 1)
    t = np.array([s.stars[0].t_star for s in sp])
    assert t.min() >= 30000 and t.max() <= 100000
    lognh = np.log10([s.nh_median for s in sp])
    assert lognh.min() >= 1 and lognh.max() <= 4
    rout = np.array([s.r_out for s in sp])
    assert rout.min() >= 1e18 and rout.max() <= 1e19 and all(s.extent == s.r_out for s in sp)
    npk = np.array([s.stars[0].n_packets for s in sp])
    assert abs(npk.sum() - 2e8) < 2e8 * 1e-3
    # packets follow the cell count
    assert np.corrcoef(npk, ns.astype(float) ** 3)[0, 1] > 0.999
    assert nebula.batch64(seed=2)[0].n != sp[0].n or nebula.batch64(seed=2)[0].nh_median != sp[0].nh_median


@pytest.mark.gpu
def test_server_runs_every_model(gpu_lib):
    specs = nebula.batch64(n_models=6, packets_total=600_000, n_min=17, n_max=25)
    srv = serve.ModelServer(memory_budget=4e9, workers=3, iterations=2, autotune_packets=20_000)
    for s in specs:
        srv.submit(s)
    rep = srv.run()
    assert rep["errors"] == [] and rep["models"] == 6 and rep["iterations"] == 12
    assert rep["latency_ms_p99"] >= rep["latency_ms_p50"] > 0
    assert 1 <= rep["peak_resident_models"] <= 3 and rep["crossings_per_s"] > 0
    assert all(len(r["latency_s"]) == 2 for r in srv.results)


@pytest.mark.gpu
def test_memory_budget_limits_resident_models(gpu_lib):
    specs = nebula.batch64(n_models=4, packets_total=200_000, n_min=17, n_max=19)
    one = serve.device_bytes(nebula.build(specs[0]))
    srv = serve.ModelServer(memory_budget=one * 1.05, workers=4, iterations=1)
    for s in specs:
        srv.submit(s)
    rep = srv.run()
    assert rep["errors"] == [] and rep["models"] == 4
    assert rep["peak_resident_models"] <= 2
