"""Benchmark of the GPU energy-packet transport: cell crossings/s.

One step = one transport iteration of the clumpy 61^3 full-sphere nebula
(lognormal nH, median 300 cm^-3, sigma_ln 1, 3-cell Gaussian correlation,
seed 1; 60 kK blackbody star of 5e37 erg/s; 600 bins; 2e7 packets), FP32
march with FP64 estimator sums.  A crossing is one pathSegment loop body
ending in a full crossing or an interaction (source/photon_mod.f90:1517,
:1817).

  value   crossings / device time of the step, grid resident in HBM (the
          estimators are zeroed inside the step, as iterateMC does)
  e2e     the same metric through the drop-in call mc_transport_run_f32 with
          HOST (pinned) buffers: grid upload, transport, download of the
          estimators into the grid's own FP32 arrays
  roofline  16 algorithmic bytes per crossing (4 B opacity + 4 B active +
          8 B FP64 Jste) over the transport kernel's CUDA-event time, against
          the measured HBM copy bandwidth
  cpu_baseline  the FP32 oracle (a C++ restatement of the reference's Fortran
          path, FP32 sums like the reference's `real` Jste) on the host cores,
          on a bounded sample of the same workload
  converged_model  wall time to a converged model (Lambda iterations of
          transport, cell update, opacity and emission CDFs) of the chosen
          form, of the chosen form with the learned warm start (trained on the
          batch's FP64 cell states), and of the plain form (FP64 update), with
          the converged states compared against the plain form's
  batched_models  the request loop over the first --batch-models of the
          64-model batch: wall, p50 / p99 latency per Lambda iteration; the
          same requests served in lockstep (the resident models' transports in
          one mc_batch_run per iteration); one transport iteration of those
          models one call after another against one batched call

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "cell crossings/s"
UNIT = "crossings/s"
BYTES_PER_CROSSING = 16


def workload(name):
    from mocassin_gb300 import nebula
    return {"clumpy61": nebula.clumpy61, "octant21": nebula.octant21, "dusty81": nebula.dusty81,
            "twostar101": nebula.twostar101}[name]()


def measured_peak():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_crossing():
    """DRAM bytes per crossing from the committed ncu summary, if any."""
    p = os.path.join(HERE, "profiles", "wave_march_dram.txt")
    try:
        for line in open(p):
            if line.startswith("dram_bytes_per_crossing:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(s[0]) for s in self.samples if len(s) >= 7 and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) >= 7 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 7 for i in range(4)
                          if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def workload_config(neb):
    """The workload of one step, the same in both arms' JSON lines."""
    l2 = "inputs larger than L2 (opacity %d MB, Jste %d MB)" % (neb.opacity.nbytes // 2**20,
                                                                  2 * neb.opacity.nbytes // 2**20)
    return {"workload": neb.spec.name, "grid": "%d^3" % neb.nx, "cells": neb.ncells, "nbins": neb.nbins,
            "stars": len(neb.n_packets), "packets_per_step": int(sum(neb.n_packets)), "l2": l2}


class OracleStep:
    """One transport iteration of the FP32 oracle (the C++ restatement of the
    reference's Fortran path) on the host cores: all packets of every star
    (or n_packets per star), estimators zeroed inside the step as iterateMC
    zeroes them; the grid marshalling and the estimator allocation are made
    once, outside."""

    def __init__(self, neb, n_packets=None, threads=None):
        from mocassin_gb300 import abi
        self.neb = neb
        self.n = n_packets
        self.threads = threads or os.cpu_count() or 1
        self.m = abi.Marshalled(neb, n_packets=n_packets)
        self.out = abi.estimator_arrays(neb)
        for a in self.out:
            a.fill(1.0)  # touch the pages once

    def __call__(self, seed):
        from oracle import runner
        t0 = time.perf_counter()
        st = runner.run(self.neb, n_packets=self.n, precision="fp32", seed=seed, threads=self.threads, out=self.out,
                        marshalled=self.m)[3]
        return time.perf_counter() - t0, st["crossings"]


def cpu_baseline(args):
    """FP32 oracle on the host cores: one full step of the reference arm (a
    bounded warm-up sample, then every packet of the step), run as a child
    process so that it times exactly what --impl reference times (about
    10 s of CPU work on the 61^3 workload)."""
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--steps", "1", "--warmup", "1",
           "--config", args.config]
    if args.packets:
        cmd += ["--packets", str(args.packets)]
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    out = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=1200)
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    cb = dict(line["cpu_baseline"])
    cb["sample"] = ("the full %d-packet step after a %d-packet warm-up step, timed by --impl reference in a "
                    "child process (FP32 march, FP64 sums; estimators zeroed inside, allocated outside)"
                    % (line["config"]["packets_per_step"], line["impl_detail"]["warmup_packets"]))
    return cb


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    """The reference arm: the reference's CPU path for this transport, the
    FP32 oracle (the Fortran cannot be built on either machine), on all host
    cores, over the same step as the GPU arm: every packet of the workload's
    transport iteration per timed step.  Warm-up steps are bounded samples
    (--ref-packets) of the same workload."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from mocassin_gb300 import nebula
    spec = workload(args.config)
    if args.packets:
        for st in spec.stars:
            st.n_packets = int(args.packets // len(spec.stars))
    neb = nebula.build(spec)
    warm = OracleStep(neb, n_packets=args.ref_packets)
    for w in range(args.warmup):
        warm(100 + w)
    del warm
    step = OracleStep(neb)
    cross, total = 0, 0.0
    for k in range(args.steps):
        dt, c = step(1 + k)
        total += dt
        cross += c
    value = cross / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(neb),
            "impl_detail": {"crossings_per_step": cross / args.steps, "threads": step.threads,
                            "warmup_packets": args.ref_packets},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": step.threads, "kind": "port",
                             "sample": "the full %d-packet step x %d steps, FP32 oracle (C++ restatement of "
                                       "photon_mod.f90; the Fortran reference has no compiler here)"
                                       % (sum(neb.n_packets), args.steps)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# Lambda-iteration forms: transport form, march arithmetic, cell update, opacity build, surrogate.
#  plain: the method without the three patterns on the best kernel (the frequency-sorted wave march
#         with host-driven rounds, all FP64 but the FP32 CUDA-core opacity; no warm start, one model)
#  naive: one thread per packet history (FP32 march), FP64 update
#  chosen: the precision pattern (FP32 march, FP32 update, split-BF16 tensor-core opacity) with the
#         rounds in one CUDA graph; chosen_surrogate: plus the learned warm start
LAMBDA_FORMS = {"chosen": ("graph", "fp32", "fp32", "bf16x3", None),
                "chosen_surrogate": ("graph", "fp32", "fp32", "bf16x3", {"train_after": 2}),
                "plain": ("wave", "fp64", "fp64", "fp32", None),
                "naive": ("plain", "fp32", "fp64", "fp32", None)}
DTE_RULE_PCT = 50.0  # the |dTe| < 1 % rule: this share of the updated cells changed Te by less than 1 %


def _wall_to_dte_rule(hist):
    """Wall time up to the first iteration after which >= DTE_RULE_PCT % of
    the updated cells changed Te by less than 1 % (None if none did)."""
    t = 0.0
    for h in hist:
        t += h["wall_s"]
        if h["dte_lt_1pc_pct"] >= DTE_RULE_PCT and h["iteration"] > 1:
            return t, h["iteration"]
    return None, None


def _lambda_form(neb, name, args, rows):
    from mocassin_gb300 import iterate
    form, march, upd, opac, sur = LAMBDA_FORMS[name]
    if sur is not None and rows is not None:
        sur = {"rows": rows, "train_after": None, "steps": 2000, "batch": 4096, "lr": 2e-3}
    li = iterate.LambdaIteration(neb, form=form, march=march, update=upd, opacity_method=opac, surrogate=sur)
    pre = li.pretrain
    wall, hist = li.run(seed=1000, max_iterations=args.lambda_max)
    state = li.ctx.get_cell_state()
    li.close()
    last = hist[-1]
    dte_wall, dte_it = _wall_to_dte_rule(hist)
    rec = {"transport": form, "march": march, "update": upd, "opacity": opac, "surrogate": sur is not None,
           "wall_s": wall, "iterations": len(hist), "surrogate_s": sum(h["surrogate_s"] for h in hist),
           "converged": last["converged_pct"] >= 95.0, "converged_pct": last["converged_pct"],
           "dte_lt_1pc_pct": last["dte_lt_1pc_pct"],
           "wall_to_dte_rule_s": dte_wall, "iterations_to_dte_rule": dte_it,
           "transport_s": sum(h["transport_s"] for h in hist), "update_s": sum(h["update_s"] for h in hist),
           "opacity_s": sum(h["opacity_s"] for h in hist),
           "t_steps_per_cell": float(np.mean([h["t_steps_per_cell"] for h in hist])),
           "warm_fallback_pct": float(np.mean([h["warm_fallback_pct"] for h in hist]))}
    if pre is not None:
        rec["pretrain"] = pre
    return rec, state


def converged_model(neb, args, keep=None):
    """Wall time to a converged model: Lambda iterations (transport, cell
    update, opacity and emission-CDF rebuild) until 95 % of the cells have
    |dX(H0)/X(H0)| <= 5 % (the reference's minConvergence / XHILimit), for
    the chosen form (persistent wave march in a CUDA graph, FP32 cell
    update), the same with the learned warm start, and the plain form (one
    thread per history, FP64 cell update), from the same initial state.  The
    warm start's network is trained before the first update on the batch's
    FP64 cell states (``--surrogate-rows``; its dataset and training times
    are reported apart: one network serves every model), or, with
    ``--surrogate-rows 0``, on the model's own first two iterations."""
    from mocassin_gb300 import iterate, nebula
    out = {"rule": "converged cells (|dX(H0)/X(H0)| <= 5%) >= 95% (iterateMC minConvergence)",
           "dte_rule": "wall_to_dte_rule_s: up to the first iteration after which >= %g%% of the updated cells "
                       "changed Te by less than 1%%" % DTE_RULE_PCT,
           "max_iterations": args.lambda_max, "packets_per_iteration": int(sum(neb.n_packets))}
    rows = None
    if args.surrogate_rows > 0:
        x, t, info = iterate.training_rows(nebula.batch64(), max_rows=args.surrogate_rows)
        rows = (x, t)
        out["surrogate_dataset"] = info
    if keep is not None:
        keep["rows"] = rows
    states = {}
    for name in LAMBDA_FORMS:
        out[name], states[name] = _lambda_form(neb, name, args, rows)
    # the converged states of the chosen forms against (vs_fp64_update) the naive form's, the same FP32
    # draws and march with the FP64 cell update, which isolates the update's precision, and against
    # (vs_plain) the plain FP64 method, whose march takes other paths, so that packet noise dominates:
    # Te and the ionic fractions above 1e-3 of every cell the last update reached and balanced in Te in
    # both forms (where the update gives up on Te balance, noTeBal, its Te means nothing)
    for ref in ("naive", "plain"):
        te_p, _, x_p = states[ref][:3]
        for name in ("chosen", "chosen_surrogate"):
            te, _, x = states[name][:3]
            reached = (states[ref][4] > 0) & ((states[ref][5] & 1) == 0) & ((states[name][5] & 1) == 0)
            dte = np.abs(te[reached] / te_p[reached] - 1)
            big = (x_p[reached] > 1e-3)
            dx = np.abs(x[reached][big] / x_p[reached][big] - 1)
            out[name]["vs_fp64_update" if ref == "naive" else "vs_plain"] = {
                "te_rel_median": float(np.median(dte)), "te_rel_p95": float(np.quantile(dte, 0.95)),
                "ion_frac_rel_median": float(np.median(dx)), "ion_frac_rel_p95": float(np.quantile(dx, 0.95)),
                "ion_frac_within_2pct": float(np.mean(dx <= 0.02)), "cells": int(reached.sum())}
    out["speedup_chosen_vs_plain"] = out["plain"]["wall_s"] / out["chosen"]["wall_s"]
    out["speedup_chosen_surrogate_vs_plain"] = out["plain"]["wall_s"] / out["chosen_surrogate"]["wall_s"]
    # where the chosen form's gain comes from, per Lambda iteration: the transport (FP64 wave march to the
    # FP32 march in a graph) and the cell update (FP64 to FP32); the warm start against the chosen form
    per = lambda n, k: out[n][k] / max(out[n]["iterations"], 1)
    out["speedup_parts"] = {"transport_per_iteration": per("plain", "transport_s") / per("chosen", "transport_s"),
                            "update_per_iteration": per("plain", "update_s") / per("chosen", "update_s"),
                            "warm_start_wall": out["chosen"]["wall_s"] / out["chosen_surrogate"]["wall_s"]}
    if args.repeats > 1:
        # the chosen form with and without the warm start, each run `repeats` times from the same initial
        # state (the warm start's network trained anew each time: its training sums in a different order
        # from run to run, so its spread is part of the warm start's)
        recs = {n: [out[n]] + [_lambda_form(neb, n, args, rows)[0] for _ in range(args.repeats - 1)]
                for n in ("chosen", "chosen_surrogate")}
        rep = {"runs": args.repeats}
        for n, rr in recs.items():
            rep[n] = {}
            for k in ("wall_s", "wall_to_dte_rule_s", "update_s", "transport_s", "iterations"):
                v = np.array([r[k] for r in rr if r[k] is not None], dtype=float)
                rep[n][k] = {"mean": float(v.mean()), "sd": float(v.std(ddof=1)) if len(v) > 1 else None,
                             "n": int(len(v))}
        a, b = rep["chosen"]["wall_s"], rep["chosen_surrogate"]["wall_s"]
        rep["warm_start_wall_ratio"] = a["mean"] / b["mean"]
        # difference of the means in units of its standard error (Welch)
        se = np.sqrt((a["sd"] or 0.0) ** 2 / a["n"] + (b["sd"] or 0.0) ** 2 / b["n"])
        rep["warm_start_gain_in_se"] = float((a["mean"] - b["mean"]) / se) if se > 0 else None
        out["repeats"] = rep
    return out


LAMBDA_KEYS = ("wall_s", "iterations", "converged", "converged_pct", "dte_lt_1pc_pct", "wall_to_dte_rule_s",
               "transport_s", "update_s", "t_steps_per_cell", "warm_fallback_pct")


def other_workloads(args, rows):
    """The other benchmark workloads, one record each: the octant 21^3 of
    the reference's CPU-runnable case, the dusty 81^3 and the two-star 101^3
    of the learned warm start.  The transport's crossings/s (graph form,
    FP32 march, device time of 3 steps after 2 warm-up steps) and the wall
    time to a converged model of the chosen form (and, on the two-star grid,
    with the warm start trained on the batch's FP64 cell states as for the
    main workload)."""
    out = {}
    for name, warm in (("octant21", False), ("dusty81", False), ("twostar101", True)):
        try:
            out[name] = _workload_record(name, warm, args, rows)
        except Exception as exc:  # reported in the record; the bench line still prints
            out[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}
    return out


def _workload_record(name, warm, args, rows):
    """One workload of other_workloads."""
    from mocassin_gb300 import nebula, transport
    neb = nebula.build(workload(name))
    ctx = transport.TransportContext(neb)
    try:
        for k in range(2):
            ctx.run(seed=900 + k, precision="fp32", zero_first=True, form="graph")
        sts = [ctx.run(seed=910 + k, precision="fp32", zero_first=True, form="graph") for k in range(3)]
    finally:
        ctx.close()
    cross = sum(st["crossings"] for st in sts)
    ms = sum(st["kernel_ms"] for st in sts)
    rec = {"workload": neb.spec.name, "cells": neb.ncells, "packets_per_step": int(sum(neb.n_packets)),
           "crossings_per_step": cross / len(sts), "step_ms": ms / len(sts),
           "crossings_per_s": cross / (ms / 1e3) if ms > 0 else None,
           "transport": "graph form, FP32 march, FP64 sums; device time of the whole call"}
    if args.lambda_max > 0:
        forms = ("chosen", "chosen_surrogate") if warm and rows is not None else ("chosen",)
        rec["converged_model"] = {}
        for f in forms:
            r = _lambda_form(neb, f, args, rows)[0]
            rec["converged_model"][f] = {k: r[k] for k in LAMBDA_KEYS if k in r}
    return rec


def breakdown(neb, args, runs):
    """mean +- sd over `runs` repetitions of each Lambda form: wall, transport
    and update time, iterations, wall to the |dTe| rule (the warm start's
    network trained on the batch's FP64 cell states, as in the main run)."""
    from mocassin_gb300 import iterate, nebula
    rows = None
    if args.surrogate_rows > 0:
        x, t, _ = iterate.training_rows(nebula.batch64(), max_rows=args.surrogate_rows)
        rows = (x, t)
    out = {}
    for name in LAMBDA_FORMS:
        recs = [_lambda_form(neb, name, args, rows)[0] for _ in range(runs)]
        stat = {}
        for k in ("wall_s", "transport_s", "update_s", "iterations", "wall_to_dte_rule_s"):
            v = np.array([r[k] for r in recs if r[k] is not None], dtype=float)
            stat[k] = {"mean": float(v.mean()) if len(v) else None,
                       "sd": float(v.std(ddof=1)) if len(v) > 1 else None, "n": int(len(v))}
        out[name] = stat
    return out


def batched_models(args):
    """The 64-model batch (grid sizes 17^3-65^3, 30-100 kK stars, log nH
    1-4, outer radius 1e18-1e19 cm, 33 packets per cell: 2e8 over the 64)
    served by the request loop of mocassin_gb300.serve: the first
    ``--batch-models`` of them, 3 Lambda iterations each, admitted by device
    memory, ``--batch-workers`` models resident at a time."""
    from mocassin_gb300 import nebula, serve
    specs = nebula.batch64()[: args.batch_models]
    srv = serve.ModelServer(memory_budget=200e9, workers=args.batch_workers, iterations=3,
                            autotune_packets=200_000)
    for sp in specs:
        srv.submit(sp)
    rep = srv.run()
    rep["batch"] = "%d of the 64-model batch (seed 1)" % len(specs)
    # the same requests served in lockstep: groups of 16 models, each group's
    # transports in one mc_batch_run per Lambda iteration (one march launch
    # per round), two groups in flight (one's transports overlap the other's
    # updates)
    lk = serve.ModelServer(memory_budget=200e9, workers=args.batch_workers, iterations=3,
                           autotune_packets=200_000, lockstep=True, group=16, lanes=2)
    for sp in specs:
        lk.submit(sp)
    lrep = lk.run()
    rep["lockstep"] = {k: lrep[k] for k in ("models", "errors", "wall_s", "crossings_per_s", "latency_ms_p50",
                                            "latency_ms_p99", "peak_resident_models", "mode")}
    rep["lockstep"]["groups"] = "16 models per group, 2 groups in flight"
    rep["one_launch_transport"] = batch_launch_transport(specs)
    return rep


def batch_launch_transport(specs):
    """One transport iteration of the same models, all resident: each model's
    own call in turn (mc_ctx_run, host-driven rounds) against one batched call
    whose rounds run in step with one persistent march launch per round over
    every model (mc_batch_run).  Same draws, so the same crossings."""
    from mocassin_gb300 import nebula, transport
    ctxs = [transport.TransportContext(nebula.build(sp)) for sp in specs]
    try:
        seeds = [101 + i for i in range(len(ctxs))]

        def one_by_one():
            return [c.run(seed=s, zero_first=True) for c, s in zip(ctxs, seeds)]

        def batched():
            return transport.batch_run(ctxs, seeds=seeds, zero_first=True)

        out = {"models": len(ctxs)}
        for name, fn in (("one_by_one", one_by_one), ("batched", batched)):
            fn()  # warm-up (both calls return after their device work)
            t0 = time.perf_counter()
            st = fn()
            wall = time.perf_counter() - t0
            cross = sum(x["crossings"] for x in st)
            out[name] = {"wall_ms": wall * 1e3, "crossings": int(cross), "crossings_per_s": cross / wall}
        out["speedup"] = out["one_by_one"]["wall_ms"] / out["batched"]["wall_ms"]
        return out
    finally:
        for c in ctxs:
            c.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="clumpy61")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--packets", type=int, default=0, help="override packets per step")
    ap.add_argument("--grid", type=int, default=0, help="override the grid size n (odd for full grids)")
    ap.add_argument("--ref-packets", type=int, default=200000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--form", default="graph", choices=["graph", "wave", "plain"],
                    help="graph: the chosen form with its rounds in one CUDA graph; wave: the same with host-driven "
                         "rounds; plain: one thread per history")
    ap.add_argument("--roof-steps", type=int, default=2,
                    help="host-driven steps that time the march alone for the roofline (graph form)")
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--no-opacity", action="store_true")
    ap.add_argument("--lambda-max", type=int, default=12, help="Lambda iterations at most per form (0: skip)")
    ap.add_argument("--batch-models", type=int, default=64,
                    help="batched serving: models of the 64-model batch to serve (0: skip)")
    ap.add_argument("--batch-workers", type=int, default=4)
    ap.add_argument("--surrogate-rows", type=int, default=1_000_000,
                    help="batch cell states (FP64 update) the warm start is trained on; 0: the model's own")
    ap.add_argument("--no-other-workloads", dest="other_workloads", action="store_false",
                    help="skip the octant 21^3, dusty 81^3 and two-star 101^3 records")
    ap.add_argument("--repeats", type=int, default=5,
                    help="runs of the chosen form with and without the warm start (mean and sd of their times)")
    ap.add_argument("--breakdown", type=int, default=0,
                    help="only the Lambda forms, each run this many times: mean and sd of their times")
    ap.add_argument("--lambda-only", default="", choices=["", "chosen", "chosen_surrogate", "plain", "naive"],
                    help="run only the Lambda iteration of one form and print its record (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)

    from mocassin_gb300 import build, nebula, transport
    build.build()
    spec = workload(args.config)
    if args.packets:
        spec.stars[0].n_packets = args.packets
    if args.grid:
        spec.n = args.grid
    neb = nebula.build(spec)
    npk = sum(neb.n_packets)
    if args.lambda_only:
        from mocassin_gb300 import iterate
        form, march, upd, opac, sur = LAMBDA_FORMS[args.lambda_only]
        li = iterate.LambdaIteration(neb, form=form, march=march, update=upd, opacity_method=opac, surrogate=sur)
        wall, hist = li.run(seed=1000, max_iterations=max(args.lambda_max, 1))
        li.close()
        print(json.dumps({"lambda_only": args.lambda_only, "workload": neb.spec.name, "wall_s": wall,
                          "iterations": hist}))
        return 0
    if args.breakdown > 0:
        print(json.dumps({"breakdown": breakdown(neb, args, args.breakdown), "workload": neb.spec.name,
                          "runs": args.breakdown, "packets_per_iteration": int(sum(neb.n_packets))}))
        return 0

    ctx = transport.TransportContext(neb)
    for w in range(args.warmup):
        ctx.run(seed=1000 + w, iteration=1, precision=args.precision, zero_first=True, form=args.form)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(torch.cuda.current_device() if ws == 1 else local)
    clocks.start()
    # the library's kernels run on its own stream; its CUDA events bracket
    # each step (zeroing + transport + counter read-back) and the call
    # synchronises that stream before returning
    stats = []
    for k in range(args.steps):
        stats.append(ctx.run(seed=1 + rank * 1000003 + k, iteration=1, precision=args.precision, zero_first=True,
                             form=args.form))
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = np.array([s["kernel_ms"] for s in stats])
    cross = int(sum(s["crossings"] for s in stats))
    t_dev = float(step_ms.sum()) / 1e3
    if ws > 1:
        t = torch.tensor([t_dev], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        c = torch.tensor([cross], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(c)
        t_dev, cross_all = float(t.item()), float(c.item())
    else:
        cross_all = float(cross)
    value = cross_all / t_dev
    march_ms = np.array([s["march_ms"] for s in stats])
    if args.form == "graph":
        # the march alone is timed only with host-driven rounds: the same work
        rs = [ctx.run(seed=1 + rank * 1000003 + k, iteration=1, precision=args.precision, zero_first=True,
                      form="wave") for k in range(max(args.roof_steps, 1))]
        march_ms = np.array([s["march_ms"] for s in rs])
        roof_cross = int(sum(s["crossings"] for s in rs))
    else:
        roof_cross = cross
    plain = None
    if args.form in ("wave", "graph") and args.plain_steps > 0:
        ctx.run(seed=999, iteration=1, precision=args.precision, zero_first=True, form="plain")
        ps = [ctx.run(seed=2 + k, iteration=1, precision=args.precision, zero_first=True, form="plain")
              for k in range(args.plain_steps)]
        pms = np.array([s["kernel_ms"] for s in ps])
        pc = sum(s["crossings"] for s in ps)
        plain = {"value": pc / (pms.sum() / 1e3), "unit": UNIT, "ms_per_step": float(pms.mean()),
                 "steps": args.plain_steps, "kernel": "transport_plain_kernel<float>",
                 "roofline_frac": pc * BYTES_PER_CROSSING / (pms.sum() / 1e3) / 1e9 / measured_peak()[0]}
    # photoionisation sums of the cell update on the resident Jste (one moment per ion)
    moments = None
    if not args.no_opacity:
        from mocassin_gb300 import rates
        w = rates.photo_weights(neb.xs, neb.nu)
        ctx.jste_moments(w, 1e-9)
        ts = [ctx.jste_moments(w, 1e-9)[1] for _ in range(5)]
        t = float(np.median(ts)) / 1e3
        jb = neb.nbins * (neb.ncells + 1) * 8
        ob = w.shape[1] * (neb.ncells + 1) * 4
        moments = {"kernel": "jmoment_tc_kernel (tcgen05 kind::f16, split BF16 x3, FP32 accumulate)",
                   "outputs": int(w.shape[1]), "ms": t * 1e3, "achieved_gbs": (jb + ob) / t / 1e9,
                   "frac_of_hbm": (jb + ob) / t / 1e9 / measured_peak()[0],
                   "bound": "hbm (reads 8 B of Jste per cell and bin)",
                   "download_bytes": ob, "instead_of": jb}
    # opacity build on the resident grid (addOpacity + dust add as one contraction)
    opac = None
    if not args.no_opacity:
        den = np.ascontiguousarray(neb.ion_den.T)
        kk = den.shape[0]
        res = {}
        for meth in ("bf16x3", "fp32"):
            ctx.build_opacity(den, neb.xs, None, method=meth)
            ts = [ctx.build_opacity(den, neb.xs, None, method=meth) for _ in range(5)]
            res[meth] = float(np.median(ts))
        out_bytes = neb.nbins * (neb.ncells + 1) * 4
        in_bytes = kk * (neb.ncells + 1) * 4
        flops = 2.0 * (neb.ncells + 1) * kk * neb.nbins
        t = res["bf16x3"] / 1e3
        opac = {"kernel": "opacity_pipe_kernel (tcgen05 kind::f16, split BF16 x3, FP32 accumulate, stores of a tile "
                          "overlapping the next tile's MMAs)",
                "species": kk, "ms": res["bf16x3"], "fp32_cuda_core_ms": res["fp32"],
                "achieved_gbs": (out_bytes + in_bytes) / t / 1e9, "frac_of_hbm": (out_bytes + in_bytes) / t / 1e9 / measured_peak()[0],
                "useful_tflops": flops / t / 1e12, "tensor_tflops_issued": 3 * flops * (((kk + 15) // 16) * 16 / kk) / t / 1e12,
                "bound": "hbm (writes 4 B per cell and bin)"}
        # the table the transport used is restored
        ctx.update(neb)
    ctx.close()

    # e2e: the drop-in call with host (pinned) buffers, copies inside the timed region
    import ctypes as C
    from mocassin_gb300 import abi
    pinned = []  # keeps every pinned buffer alive while the grid struct points at it

    def pin(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        pinned.append(t)
        return t

    lib = transport.library()
    m = abi.Marshalled(neb)
    fields = [("opacity", neb.opacity), ("rec_pdf", neb.rec_pdf), ("total_lines", neb.total_lines),
              ("x_axis", neb.x_axis), ("y_axis", neb.y_axis), ("z_axis", neb.z_axis), ("nu_array", neb.nu)]
    h2d = 0
    for name, arr in fields:
        t = pin(arr.astype(np.float32))
        setattr(m.grid, name, C.cast(t.data_ptr(), C.POINTER(C.c_float)))
        h2d += t.numel() * 4
    ta = pin(neb.active.astype(np.int32))
    m.grid.active = C.cast(ta.data_ptr(), C.POINTER(C.c_int32))
    h2d += ta.numel() * 4
    if neb.sca_opac is not None:
        t = pin(neb.sca_opac)
        m.grid.sca_opac = C.cast(t.data_ptr(), C.POINTER(C.c_float))
        h2d += t.numel() * 4
    # the grid's own 4-byte estimator arrays (mc_transport_run_f32): FP64 sums on the device, rounded once
    js = torch.zeros((neb.nbins, neb.ncells + 1), dtype=torch.float32).pin_memory()
    es = torch.zeros((neb.nbins + 1, neb.ncells + 1), dtype=torch.float32).pin_memory()
    # the estimators start each iteration at zero: the Fortran driver zeroes
    # Jste and escapedPackets before every iteration (iteration_mod.f90:458-472),
    # here between calls, outside the timed region; MC_RUN_HOST_ZEROED then
    # brings back only the entries the transport made nonzero
    e2e_t, e2e_c, h2d, d2h = 0.0, 0, 0, 0
    for k in range(args.e2e_steps + 1):
        js.zero_()
        es.zero_()
        opts = abi.make_opts(seed=77 + k, iteration=1, precision=abi.MC_PREC_FP32 if args.precision == "fp32"
                             else abi.MC_PREC_FP64,
                             run_flags={"plain": abi.MC_RUN_FORM_PLAIN, "graph": abi.MC_RUN_GRAPH}.get(args.form, 0)
                             | abi.MC_RUN_HOST_ZEROED)
        st = abi.McStats()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc = lib.mc_transport_run_f32(C.byref(m.grid), m.sources, m.nsrc, C.byref(opts),
                                      C.cast(js.data_ptr(), C.POINTER(C.c_float)), None,
                                      C.cast(es.data_ptr(), C.POINTER(C.c_float)), C.byref(st))
        dt = time.perf_counter() - t0
        if rc != 0:
            raise transport.TransportError(rc, lib.mc_last_error().decode())
        if k > 0:  # first call is a warm-up
            e2e_t += dt
            e2e_c += st.crossings
            h2d += st.h2d_bytes
            d2h += st.d2h_bytes
    ne2e = max(args.e2e_steps, 1)
    e2e = {"value": e2e_c / e2e_t if e2e_t > 0 else None, "unit": UNIT, "h2d_bytes_per_step": int(h2d // ne2e),
           "d2h_bytes_per_step": int(d2h // ne2e),
           "call": "mc_transport_run_f32 with MC_RUN_HOST_ZEROED (host pinned buffers: grid upload (the opacity "
                   "rows a packet can march in, recPDF re-laid out on a side stream during round 0), transport, "
                   "download into the grid's own FP32 Jste of the frequency rows that received a deposit and "
                   "scatter of the nonzero escapedPackets entries, FP64 sums rounded once on the device; the "
                   "caller's estimators zeroed between calls outside the timed region, as the Fortran driver "
                   "zeroes them before each iteration; device buffers kept between calls of the same grid "
                   "shape, the entries a call made nonzero cleared on the device once copied); bytes are those "
                   "the call reports having copied"}

    peak, peak_kind = measured_peak()
    # dominant kernel: the march (its own CUDA events on the library stream)
    achieved = roof_cross / (float(march_ms.sum()) / 1e3) * BYTES_PER_CROSSING / 1e9
    tpc = traffic_per_crossing()
    per_launch_cross = cross / max(len(stats), 1)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": (tpc * per_launch_cross) if tpc else None,
            "kernel": "transport_plain_kernel<float>" if args.form == "plain" else "wave_march_kernel<float,true>",
            "kernel_ms_per_step": float(march_ms.mean()), "peak_kind": peak_kind + " hbm_gbs (copy)",
            "algorithmic_bytes_per_crossing": BYTES_PER_CROSSING}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(step_ms.mean()), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": args.precision.replace("fp", "f"),
            "data": "synthetic",
            "config": workload_config(neb),
            "impl_detail": {"crossings_per_step": per_launch_cross, "march": args.precision, "estimators": "f64",
                            "form": args.form, "parallelism": "replicas" if ws > 1 else "1 GPU"},
            # per step and round: sample, scan, scatter, emit, march (+ the round control in the graph
            # form), or one kernel (plain)
            "roofline": roof, "e2e": e2e,
            "gpu_launches": int(sum(s["rounds"] for s in stats) * {"wave": 5, "graph": 6, "plain": 1}[args.form]),
            "rounds_per_step": float(np.mean([s["rounds"] for s in stats])),
            "clocks": clk}
    if plain:
        line["plain_form"] = plain
    if opac:
        line["opacity_build"] = opac
    if moments:
        line["jste_moments"] = moments
    keep = {}
    if args.lambda_max > 0 and rank == 0:
        line["converged_model"] = converged_model(neb, args, keep)
    if args.other_workloads and rank == 0 and ws == 1:
        line["other_workloads"] = other_workloads(args, keep.get("rows"))
    if args.batch_models > 0 and rank == 0:
        line["batched_models"] = batched_models(args)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
