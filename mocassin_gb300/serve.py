"""Batched models served on one GPU: a request loop that admits nebulae by
device memory and runs their Lambda iterations concurrently.

Each request is a nebula (NebulaSpec) and a number of Lambda iterations
(transport, cell update, opacity rebuild; mocassin_gb300.iterate).  A pool
of worker threads takes requests in order; a worker builds the nebula on the
host, waits until the model's device footprint fits in the memory budget
next to the models already resident, creates its context (own CUDA stream),
picks the march's scheduling parameters (autotuned once per grid size and
reused), runs the iterations, and frees the device memory.  The C-ABI calls
release the Python interpreter lock, so the models' kernels run concurrently
on their streams and the host-side builds overlap with the GPU work.

With lockstep=True the server instead admits a group of models (in request
order, up to ``group`` of them and the memory budget) and advances the
group one Lambda iteration at a time: the group's transports are one
mc_batch_run (the rounds of all its models in step, one persistent march
launch per round), then every model's cell update, opacity and emission
CDFs run at once, one thread per model of the group.  ``lanes`` groups are
in flight at once (one thread each), so one group's transports overlap
another group's updates.

Reported: wall time, aggregate cell crossings per second, the p50 / p99 of
the per-iteration latency, the peak number of resident models and bytes.
"""
import threading
import time
import zlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import autotune, iterate, nebula


def model_seed(name, iteration):
    """Philox seed of one model's Lambda iteration: distinct per model (from
    its name) and per iteration, the same in threaded and lockstep serving."""
    return 1000 + (zlib.crc32(name.encode()) & 0xFFFFF) * 64 + iteration


def device_bytes(neb):
    """Device footprint of a resident model: opacity (4 B), recPDF as given
    and re-laid out (8 B), Jste (8 B), escapedPackets (8 B), the moments of
    the cell update (67 x 4 B per cell), the cell state and scratch, the
    per-packet queues (~120 B per packet)."""
    nc1, nb = neb.ncells + 1, neb.nbins
    per_cell_bin = 4 + 8 + 8 + 8
    per_cell = 67 * 4 + 56 * 8 * 2 + 56 * 4 + 26 * 4 + 200
    return int(nc1 * nb * per_cell_bin + nc1 * per_cell + sum(neb.n_packets) * 120 + (64 << 20))


class ModelServer:
    def __init__(self, memory_budget=200e9, workers=4, iterations=3, form="graph", update="fp32",
                 autotune_packets=0, lockstep=False, group=16, lanes=1):
        self.lockstep = bool(lockstep)
        self.lanes = int(lanes)
        self.group = int(group)
        self.budget = float(memory_budget)
        self.workers = int(workers)
        self.iterations = int(iterations)
        self.form, self.update = form, update
        self.autotune_packets = int(autotune_packets)
        self.requests = []
        self._lock = threading.Condition()
        self._resident = 0
        self._resident_models = 0
        self.peak_bytes = 0
        self.peak_models = 0
        self.tuning = {}
        self.results = []
        self.errors = []

    def submit(self, spec, iterations=None):
        self.requests.append((spec, self.iterations if iterations is None else int(iterations)))

    def _admit(self, nbytes):
        with self._lock:
            while self._resident > 0 and self._resident + nbytes > self.budget:
                self._lock.wait()
            self._resident += nbytes
            self._resident_models += 1
            self.peak_bytes = max(self.peak_bytes, self._resident)
            self.peak_models = max(self.peak_models, self._resident_models)

    def _release(self, nbytes):
        with self._lock:
            self._resident -= nbytes
            self._resident_models -= 1
            self._lock.notify_all()

    def _serve_one(self, spec, iters):
        t_req = time.perf_counter()
        neb = nebula.build(spec)
        nbytes = device_bytes(neb)
        self._admit(nbytes)
        try:
            li = iterate.LambdaIteration(neb, form=self.form, update=self.update)
            key = neb.nx
            with self._lock:
                tuned = self.tuning.get(key)
            if tuned is None and self.autotune_packets > 0:
                tuned, _ = autotune.autotune(li.ctx, min(self.autotune_packets, sum(neb.n_packets)), repeats=1,
                                             candidates=((4, 4), (8, 4), (8, 8), (8, 16), (16, 8)), form=self.form)
                with self._lock:
                    self.tuning[key] = tuned
            if tuned is not None:
                li.ctx.set_tuning(*tuned)
            t0 = time.perf_counter()
            lat = []
            cross = 0
            for it in range(iters):
                rec = li.step(seed=model_seed(spec.name, it))
                lat.append(rec["wall_s"])
                cross += rec["crossings"]
            t1 = time.perf_counter()
            li.close()
            self.results.append({"model": spec.name, "cells": neb.ncells, "packets": int(sum(neb.n_packets)),
                                 "iterations": iters, "latency_s": lat, "crossings": cross,
                                 "converged_pct": rec["converged_pct"], "run_s": t1 - t0,
                                 "queue_s": t0 - t_req, "bytes": nbytes})
        finally:
            self._release(nbytes)

    def _tune(self, li, neb, form):
        key = neb.nx
        with self._lock:
            tuned = self.tuning.get(key)
        if tuned is None and self.autotune_packets > 0:
            tuned, _ = autotune.autotune(li.ctx, min(self.autotune_packets, sum(neb.n_packets)), repeats=1,
                                         candidates=((4, 4), (8, 4), (8, 8), (8, 16), (16, 8)), form=form)
            with self._lock:
                self.tuning[key] = tuned
        if tuned is not None:
            li.ctx.set_tuning(*tuned)

    def _run_lockstep(self):
        todo = list(self.requests)
        nxt = [0]
        take_lock = threading.Lock()

        def lane():
            # one thread per model of a group: every model's update, opacity
            # and CDFs run at once on their own streams after the batched
            # transport
            with ThreadPoolExecutor(max(1, self.workers, self.group)) as pool:
                while True:
                    with take_lock:
                        if nxt[0] >= len(todo):
                            return
                        group = todo[nxt[0]:nxt[0] + self.group]
                        nxt[0] += len(group)
                    self._serve_group(group, pool)

        # `lanes` groups in flight: one group's transports overlap another's updates
        threads = [threading.Thread(target=lane) for _ in range(max(1, self.lanes))]
        for t in threads:
            t.start()
        for t in threads:
            t.join()

    def _serve_group(self, group, pool):
        t_req = time.perf_counter()
        nebs = list(pool.map(lambda r: nebula.build(r[0]), group))
        while group:
            # the group's models that fit in the budget (at least one); the rest form the next group
            take, total = 0, 0
            for neb in nebs:
                nb = device_bytes(neb)
                if take and total + nb > self.budget:
                    break
                take, total = take + 1, total + nb
            self._serve_admitted(group[:take], nebs[:take], total, pool, t_req)
            group, nebs = group[take:], nebs[take:]

    def _serve_admitted(self, group, nebs, total, pool, t_req):
        take = len(group)
        self._admit(total)
        with self._lock:
            self._resident_models += take - 1
            self.peak_models = max(self.peak_models, self._resident_models)
        lis = []
        try:
            # the group's models are set up (context, tables, tuning) on the pool's threads at once
            def setup(neb):
                li = iterate.LambdaIteration(neb, form="wave", update=self.update)
                try:
                    self._tune(li, neb, "wave")
                except Exception:
                    li.close()
                    raise
                return li
            futs = [pool.submit(setup, neb) for neb in nebs]
            err = None
            for f in futs:
                try:
                    lis.append(f.result())
                except Exception as exc:
                    err = err or exc
            if err is not None:
                raise err
            t0 = time.perf_counter()
            lat = [[] for _ in lis]
            cross = [0] * len(lis)
            last = [None] * len(lis)
            for it in range(max(r[1] for r in group)):
                live = [k for k, r in enumerate(group) if it < r[1]]
                # mc_batch_run takes gas-only or dusty grids, not both
                for dusty in (False, True):
                    ks = [k for k in live if bool(lis[k].dust is not None) == dusty]
                    if not ks:
                        continue
                    recs = iterate.batched_step([lis[k] for k in ks],
                                                [model_seed(group[k][0].name, it) for k in ks], pool=pool)
                    for k, rec in zip(ks, recs):
                        lat[k].append(rec["wall_s"])
                        cross[k] += rec["crossings"]
                        last[k] = rec
            t1 = time.perf_counter()
            for k, (spec, iters) in enumerate(group):
                self.results.append({"model": spec.name, "cells": nebs[k].ncells,
                                     "packets": int(sum(nebs[k].n_packets)), "iterations": iters,
                                     "latency_s": lat[k], "crossings": cross[k],
                                     "converged_pct": last[k]["converged_pct"] if last[k] else None,
                                     "run_s": t1 - t0, "queue_s": t0 - t_req,
                                     "bytes": device_bytes(nebs[k])})
        except Exception as exc:  # reported, the next group goes on
            self.errors.append("%s: %s" % (",".join(r[0].name for r in group), exc))
        finally:
            for li in lis:
                li.close()
            with self._lock:
                self._resident_models -= take - 1
            self._release(total)

    def run(self):
        """Serves every submitted request; returns the report."""
        if self.lockstep:
            t0 = time.perf_counter()
            self._run_lockstep()
            return self._report(time.perf_counter() - t0)
        todo = list(self.requests)
        idx = [0]
        lock = threading.Lock()

        def worker():
            while True:
                with lock:
                    if idx[0] >= len(todo):
                        return
                    spec, iters = todo[idx[0]]
                    idx[0] += 1
                try:
                    self._serve_one(spec, iters)
                except Exception as exc:  # reported, the other models go on
                    self.errors.append("%s: %s" % (spec.name, exc))

        t0 = time.perf_counter()
        threads = [threading.Thread(target=worker) for _ in range(self.workers)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        return self._report(time.perf_counter() - t0)

    def _report(self, wall):
        lat = np.array([x for r in self.results for x in r["latency_s"]]) * 1e3
        cross = sum(r["crossings"] for r in self.results)
        return {"models": len(self.results), "errors": self.errors, "wall_s": wall,
                "cells": int(sum(r["cells"] for r in self.results)),
                "packets_per_iteration": int(sum(r["packets"] for r in self.results)),
                "iterations": int(sum(r["iterations"] for r in self.results)),
                "crossings_per_s": cross / wall if wall > 0 else 0.0,
                "latency_ms_p50": float(np.percentile(lat, 50)) if len(lat) else None,
                "latency_ms_p99": float(np.percentile(lat, 99)) if len(lat) else None,
                "peak_resident_models": self.peak_models, "peak_resident_bytes": self.peak_bytes,
                "workers": self.workers, "memory_budget_bytes": self.budget,
                "mode": "lockstep (mc_batch_run)" if self.lockstep else "threads (one context and stream each)",
                "tuning": {str(k): list(v) for k, v in self.tuning.items()}}
