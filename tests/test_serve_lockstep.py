"""Host logic of the lockstep server (no GPU): models are admitted in
request order into groups bounded by the group size and the memory budget,
every group advances one Lambda iteration at a time through
iterate.batched_step (gas-only and dusty models in separate batches), and
every request is served with its own number of iterations."""
from mocassin_gb300 import iterate, nebula, serve


class _FakeModel:
    made = []

    def __init__(self, neb, form="wave", update="fp32"):
        self.neb = neb
        self.dust = object() if neb.flags & nebula.FLAG_DUST else None
        self.history = []
        self.closed = False
        _FakeModel.made.append(self)

    def close(self):
        self.closed = True


def _fake_step(calls):
    def step(models, seeds, pool=None):
        calls.append(([m.neb.nx for m in models], [m.dust is not None for m in models], list(seeds)))
        out = []
        for m in models:
            m.history.append(1)
            out.append({"wall_s": 0.01, "crossings": 10 * m.neb.nx, "converged_pct": 50.0})
        return out
    return step


def test_groups_follow_the_group_size_and_iterations(monkeypatch):
    calls = []
    _FakeModel.made = []
    monkeypatch.setattr(iterate, "LambdaIteration", _FakeModel)
    monkeypatch.setattr(iterate, "batched_step", _fake_step(calls))
    cases = nebula.small_cases()
    gas = [s for s in cases if not s.dust]
    srv = serve.ModelServer(workers=2, iterations=2, lockstep=True, group=2)
    srv.submit(gas[0])
    srv.submit(gas[1], iterations=3)
    srv.submit(gas[2])
    rep = srv.run()
    assert rep["errors"] == [] and rep["models"] == 3 and rep["iterations"] == 7
    # group 1: gas[0] (2 iterations) and gas[1] (3) together, then gas[1] alone; group 2: gas[2]
    assert [len(c[0]) for c in calls] == [2, 2, 1, 1, 1]
    # every model draws its own stream per iteration, as in threaded serving
    seed = lambda spec, it: serve.model_seed(spec.name, it)
    assert [c[2] for c in calls] == [[seed(gas[0], 0), seed(gas[1], 0)], [seed(gas[0], 1), seed(gas[1], 1)],
                                     [seed(gas[1], 2)], [seed(gas[2], 0)], [seed(gas[2], 1)]]
    assert len({serve.model_seed(s.name, 0) for s in gas}) == len(gas)
    assert all(m.closed for m in _FakeModel.made)
    assert rep["peak_resident_models"] == 2
    assert rep["mode"].startswith("lockstep")


def test_memory_budget_splits_groups_and_kinds_batch_apart(monkeypatch):
    calls = []
    _FakeModel.made = []
    monkeypatch.setattr(iterate, "LambdaIteration", _FakeModel)
    monkeypatch.setattr(iterate, "batched_step", _fake_step(calls))
    cases = nebula.small_cases()
    gas = [s for s in cases if not s.dust]
    dusty = [s for s in cases if s.dust]
    # a budget below two models' footprint: one model per group
    one = serve.device_bytes(nebula.build(gas[0]))
    srv = serve.ModelServer(memory_budget=1.5 * one, iterations=1, lockstep=True, group=8)
    for s in gas[:2]:
        srv.submit(s)
    rep = srv.run()
    assert rep["models"] == 2 and [len(c[0]) for c in calls] == [1, 1]
    assert srv._resident == 0 and srv._resident_models == 0
    # gas and dusty models of one group go to separate batched steps
    calls.clear()
    srv = serve.ModelServer(iterations=1, lockstep=True, group=8)
    srv.submit(gas[0])
    srv.submit(dusty[0])
    rep = srv.run()
    assert rep["models"] == 2
    assert sorted(c[1] for c in calls) == [[False], [True]]


def test_two_lanes_serve_groups_at_once(monkeypatch):
    """With lanes=2 two groups are in flight: every request is served once,
    each group steps its own models, and the resident count returns to 0."""
    import threading
    import time
    calls = []
    inflight, peak = [0], [0]
    lock = threading.Lock()
    _FakeModel.made = []
    monkeypatch.setattr(iterate, "LambdaIteration", _FakeModel)
    step = _fake_step(calls)

    def slow_step(models, seeds, pool=None):
        with lock:
            inflight[0] += 1
            peak[0] = max(peak[0], inflight[0])
        time.sleep(0.05)
        try:
            return step(models, seeds, pool)
        finally:
            with lock:
                inflight[0] -= 1

    monkeypatch.setattr(iterate, "batched_step", slow_step)
    gas = [s for s in nebula.small_cases() if not s.dust]
    srv = serve.ModelServer(iterations=2, lockstep=True, group=1, lanes=2)
    for s in gas[:4]:
        srv.submit(s)
    rep = srv.run()
    assert rep["errors"] == [] and rep["models"] == 4 and rep["iterations"] == 8
    assert sorted(r["model"] for r in srv.results) == sorted(s.name for s in gas[:4])
    assert peak[0] == 2 and len(calls) == 8
    assert srv._resident == 0 and srv._resident_models == 0
    assert all(m.closed for m in _FakeModel.made)
