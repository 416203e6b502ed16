"""Host logic of bench.py's records (no GPU): the other workloads' record
(crossings/s from the device time of the timed steps, the Lambda keys kept,
the warm start only on the two-star grid and only with training rows, an
error in one workload reported in its own record)."""
import importlib.util
import os
import types

import pytest

from mocassin_gb300 import nebula, transport

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture()
def bench(monkeypatch):
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(HERE, "..", "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    runs = []

    class FakeCtx:
        def __init__(self, neb):
            self.neb = neb

        def run(self, **kw):
            runs.append(kw)
            return {"crossings": 1000 + kw["seed"], "kernel_ms": 2.0}

        def close(self):
            pass

    monkeypatch.setattr(transport, "TransportContext", FakeCtx)
    monkeypatch.setattr(b, "workload", lambda name: nebula.small_cases()[0])
    b._runs = runs
    return b


def test_other_workloads_record(bench, monkeypatch):
    calls = []

    def fake_lambda(neb, form, args, rows):
        calls.append(form)
        return {"wall_s": 1.5, "iterations": 3, "converged": True, "not_kept": 1}, None

    monkeypatch.setattr(bench, "_lambda_form", fake_lambda)
    out = bench.other_workloads(types.SimpleNamespace(lambda_max=12), rows=("x", "t"))
    assert set(out) == {"octant21", "dusty81", "twostar101"}
    rec = out["dusty81"]
    # 2 warm-up steps, then 3 timed steps whose device time is 2 ms each
    timed = [r["seed"] for r in bench._runs[2:5]]
    assert timed == [910, 911, 912]
    assert rec["crossings_per_step"] == pytest.approx(1911.0)
    assert rec["crossings_per_s"] == pytest.approx(3 * 1911.0 / 6e-3)
    assert rec["converged_model"]["chosen"] == {"wall_s": 1.5, "iterations": 3, "converged": True}
    assert "chosen_surrogate" not in rec["converged_model"]
    assert set(out["twostar101"]["converged_model"]) == {"chosen", "chosen_surrogate"}
    assert calls == ["chosen", "chosen", "chosen", "chosen_surrogate"]
    # no training rows: no warm start anywhere
    calls.clear()
    out = bench.other_workloads(types.SimpleNamespace(lambda_max=12), rows=None)
    assert "chosen_surrogate" not in out["twostar101"]["converged_model"]
    # no Lambda iterations asked: transport only
    out = bench.other_workloads(types.SimpleNamespace(lambda_max=0), rows=None)
    assert all("converged_model" not in r for r in out.values())


def test_a_failing_workload_is_reported_in_its_record(bench, monkeypatch):
    def boom(neb, form, args, rows):
        raise RuntimeError("no box")

    monkeypatch.setattr(bench, "_lambda_form", boom)
    out = bench.other_workloads(types.SimpleNamespace(lambda_max=12), rows=None)
    assert out["octant21"] == {"error": "RuntimeError: no box"}
    assert set(out) == {"octant21", "dusty81", "twostar101"}
