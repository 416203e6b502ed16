"""The Lambda iteration on one GPU: transport, cell update, opacity rebuild,
until the model converges (iterateMC, source/iteration_mod.f90:33-1140).

Each iteration runs, on the grid resident in HBM,
  1. the energy-packet transport of every star (energyPacketDriver, :474-496),
  2. the cell update of every active cell from the normalised Jste
     (updateCell over the grid, :800-840; Jste x 1e-9, / 8 in a symmetric
     octant, :705-724),
  3. the convergence test: the percentage of cells with
     |dX(H0)/X(H0)| <= XHILimit (0.05, set_input_mod.f90:117) against
     minConvergence (95 %, set_input_mod.f90:105; test :1135), at most
     maxIterateMC (30) iterations,
  4. the opacity of the next transport from the new ion densities
     (ionizationDriver, ionization_mod.f90:26-129, on the tensor cores),
  5. the re-emission CDFs of the next transport (recPDF rows and totalLines,
     emissionDriver / setDiffusePDF, emission_mod.f90:32-1311, on the GPU),
     built from the initial state before the first transport too, as the
     reference builds them at the top of every iteration.
On a grid with grains the grain temperatures (getDustT) follow the update,
the grains' opacity (Ndust x (abs + sca) per grain, the dust add of
iteration_mod.f90:166-227) is added to every opacity rebuild, and their
thermal emission joins the recPDF rows.  A size bin whose grain temperature
reaches the sublimation temperature drops out of the opacity and the
scattering table of the cell (iteration_mod.f90:193-210).  With
``photoelectric`` (lgPhotoelectric, on by default in the reference) every T
step of the update also charges the grains and adds the photoelectric
heating and the gas-grain collisional cooling to the gas (setGrainPotential,
setPhotoelHeatCool, setDustGasCollHeatCool, update_mod.f90:527-930), and the
grain temperatures take the matching terms (getDustT :1886-1889).

``form`` picks the transport ("graph": the frequency-sorted persistent march
with its rounds in one CUDA graph; "wave": the same with host-driven rounds;
"plain": one thread per history), ``march`` its arithmetic ("fp32", or
"fp64": the exact per-crossing method) and ``update`` the arithmetic of the
cell update ("fp64": the FP64 method; "fp32": the reference's own 4-byte
precision).  ``surrogate`` adds the learned warm start: the cell states of
the first iterations train an MLP on the GPU, which then predicts the state
each later update starts from (mc_ctx_update_cells_warm).
"""
import time

import numpy as np

from . import balance, nebula, transport


def _ions():
    return np.array([tuple(int(v) for v in r) for r in nebula.atomic_table()["ions"]], dtype=np.int32)


class LambdaIteration:
    """A nebula resident on the GPU with its cell state."""

    def __init__(self, neb, form="graph", update="fp32", xhi_limit=0.05, opacity_method="bf16x3", surrogate=None,
                 emission="auto", march="fp32", photoelectric=True):
        """surrogate: None (updates start from the previous state, as the
        reference's) or a dict with train_after (cold iterations whose cell
        states train the MLP first; None: never), steps, batch, lr,
        finetune_steps (after every later iteration), capacity (training rows
        kept), rows (an (x, t) pair of training rows from other models, e.g.
        training_rows(); the network is trained on them before the first
        update and warm-starts every update), rule ((accept_res, near_res) of
        mc_ctx_surrogate_rule)."""
        self.neb = neb
        self.form = form
        self.march = march
        self.update = update
        self.xhi = xhi_limit
        self.opacity_method = opacity_method
        self.ctx = transport.TransportContext(neb)
        self.ctx.set_update_tables(balance.tables(), neb.hden, balance.abundances())
        te, ne, X = balance.initial_state(neb)
        self.ctx.set_cell_state(te, ne, X)
        self.dust = None
        if neb.flags & nebula.FLAG_DUST:
            from . import dust
            xs_abs, gw, _ = dust.grains(neb.nu)
            self.dust = (dust.absorption_weights(xs_abs), dust.emission_table(xs_abs, neb.nu), gw)
            from . import emission as _em
            self.ctx.set_grain_opacity(*dust.grain_opacity(neb.nu), neb.ndust, _em.T_SUBLIME)
            if photoelectric:
                self.ctx.set_grain_physics(dust.grain_physics(neb))
        if emission == "auto":
            emission = True
        self.emission = bool(emission)
        if self.emission:
            self.ctx.set_emission_tables()
            self.ctx.build_emission()
        self.species = _ions()
        self.w = balance.moment_weights(neb.xs, neb.nu, self.species)
        self.scale = 1e-9 / (8.0 if neb.flags & nebula.FLAG_SYMMETRIC_XYZ else 1.0)
        self.history = []
        self.sur = None
        self.trained = False
        self.pretrain = None
        if surrogate is not None:
            self.sur = dict({"train_after": 2, "steps": 500, "batch": 4096, "lr": 3e-3, "finetune_steps": 0,
                             "capacity": 1_000_000, "seed": 1, "rows": None, "rule": None}, **surrogate)
            rows = self.sur["rows"]
            cap = max(self.sur["capacity"], (len(rows[0]) if rows is not None else 0) + neb.ncells + 1)
            self.ctx.surrogate_init(seed=self.sur["seed"], capacity=cap)
            if self.sur["rule"] is not None:
                self.ctx.surrogate_rule(*self.sur["rule"])
            if rows is not None:
                self.ctx.surrogate_load(*rows)
                loss, ms = self.ctx.surrogate_train(self.sur["steps"], self.sur["batch"], self.sur["lr"],
                                                    self.sur["seed"])
                self.trained = True
                self.pretrain = {"rows": int(len(rows[0])), "loss": loss, "train_ms": ms}

    def step(self, seed, n_packets=None):
        t0 = time.perf_counter()
        tr = self.ctx.run(n_packets=n_packets, seed=seed, iteration=len(self.history) + 1, precision=self.march,
                          zero_first=True, form=self.form)
        t1 = time.perf_counter()
        return self.after_transport(tr, t0, t1)

    def after_transport(self, tr, t0, t1):
        """The rest of a Lambda iteration once its transport (stats tr, timed
        t0..t1) has filled the resident Jste: cell update, surrogate, grain
        temperatures, opacity and emission CDFs."""
        warm = self.trained
        up = self.ctx.update_cells(self.w, self.scale, xhi_limit=self.xhi, precision=self.update, warm=warm)
        t2 = time.perf_counter()
        train_ms, loss = 0.0, None
        if self.sur is not None and (self.sur["rows"] is None or self.sur["finetune_steps"] > 0):
            self.ctx.surrogate_collect()
            if (not self.trained and self.sur["train_after"] is not None
                    and len(self.history) + 1 >= self.sur["train_after"]):
                loss, train_ms = self.ctx.surrogate_train(self.sur["steps"], self.sur["batch"], self.sur["lr"],
                                                          self.sur["seed"])
                self.trained = True
            elif self.trained and self.sur["finetune_steps"] > 0:
                loss, train_ms = self.ctx.surrogate_train(self.sur["finetune_steps"], self.sur["batch"],
                                                          0.3 * self.sur["lr"], self.sur["seed"])
        t2b = time.perf_counter()
        if self.dust is not None:
            self.ctx.dust_temperatures(*self.dust, self.scale)
        op_ms = self.ctx.opacity_from_state(self.species, self.neb.xs, method=self.opacity_method)
        em_ms = self.ctx.build_emission() if self.emission else 0.0
        t3 = time.perf_counter()
        rec = {"iteration": len(self.history) + 1, "transport_s": t1 - t0, "update_s": t2 - t1,
               "surrogate_s": t2b - t2, "surrogate_train_ms": train_ms, "surrogate_loss": loss, "warm": warm,
               "opacity_s": t3 - t2b,
               "wall_s": t3 - t0, "crossings": tr["crossings"], "transport_kernel_ms": tr["kernel_ms"],
               "update_ms": up["update_ms"], "moments_ms": up["moments_ms"], "opacity_ms": op_ms,
               "emission_ms": em_ms,
               "hit": up["hit"], "converged_pct": 100.0 * up["converged"] / max(up["hit"], 1),
               "dte_lt_1pc_pct": 100.0 * up["frac_dte_1pc"], "t_steps_per_cell": up["t_iterations"] / max(up["hit"], 1),
               "no_te_balance": up["no_te_balance"], "no_ion_balance": up["no_ion_balance"],
               "warm_fallback_pct": 100.0 * up["warm_fallback"] / max(up["hit"], 1)}
        self.history.append(rec)
        return rec

    def run(self, seed=1, max_iterations=30, min_convergence=95.0, n_packets=None):
        """Iterates until converged_pct >= min_convergence; returns the wall time and the history."""
        t0 = time.perf_counter()
        for it in range(max_iterations):
            rec = self.step(seed + it, n_packets=n_packets)
            if rec["converged_pct"] >= min_convergence:
                break
        return time.perf_counter() - t0, self.history

    def state(self):
        return self.ctx.get_cell_state()

    def write_grid(self, path):
        """Snapshot of the cell state in the reference's grid files (writeGrid)."""
        from . import gridio
        te, ne, X, conv, niter, flags = self.ctx.get_cell_state()
        gridio.write_grid(path, self.neb, te, ne, X, conv=conv, black=(flags != 0).astype(np.int32))
        gridio.write_parameters(path, gridio.model_parameters(self.neb, xhi_limit=self.xhi))

    def write_summary(self, path):
        """output/summary.out of the iterations so far, with the reference's
        per-iteration lines (iterateMC, iteration_mod.f90:1003-1065): converged,
        no-hit, no-ion-balance and no-Te-balance percentages of the grid, the
        total converged percentage and the packets used."""
        import os
        os.makedirs(path, exist_ok=True)
        nc = max(self.neb.ncells, 1)
        npk = int(sum(self.neb.n_packets))
        with open(os.path.join(path, "summary.out"), "w") as fh:
            for h in self.history:
                it = h["iteration"]
                pre = " ! iterateMC: [Summary] Iteration %12d ; " % it
                hit = max(h["hit"], 1)
                fh.write(pre + "%12d%% converged cells in grid %12d\n" % (int(h["converged_pct"]), 1))
                fh.write(pre + "%12d%% no hit cells in grid %12d\n" % (int(100.0 * (nc - h["hit"]) / nc), 1))
                fh.write(pre + "%12d%% Ion balance not reached in grid %12d\n"
                         % (int(100.0 * h["no_ion_balance"] / hit), 1))
                fh.write(pre + "%12d%% Te balance not reached in grid %12d\n"
                         % (int(100.0 * h["no_te_balance"] / hit), 1))
                fh.write(pre + "Total:  %16.8E%% converged cells over all grids\n" % h["converged_pct"])
                fh.write(pre + "%12d  energy packets used\n" % npk)
                fh.write("\n")

    def restart_from(self, path):
        """Sets the cell state from grid files (resetGrid), e.g. for a warm restart."""
        from . import gridio
        g = gridio.read_grid(path)
        if (g["nx"], g["ny"], g["nz"], g["ncells"]) != (self.neb.nx, self.neb.ny, self.neb.nz, self.neb.ncells):
            raise ValueError("the snapshot is of another grid")
        self.ctx.set_cell_state(g["te"], g["ne"], g["X"])
        self.ctx.opacity_from_state(self.species, self.neb.xs, method=self.opacity_method)
        if self.emission:
            self.ctx.build_emission()

    def close(self):
        self.ctx.close()


def batched_step(models, seeds, pool=None):
    """One Lambda iteration of several resident models in step: their
    transports in one mc_batch_run (the rounds of all models in step, one
    persistent march launch per round), then each model's cell update,
    opacity and emission CDFs (on ``pool``'s threads when given: every model
    has its own stream).  Returns the models' iteration records; a model's
    wall_s is the batched transport plus its own rest."""
    t0 = time.perf_counter()
    stats = transport.batch_run([m.ctx for m in models], seeds=seeds, iteration=len(models[0].history) + 1,
                                precision="fp32", zero_first=True)
    t1 = time.perf_counter()
    if pool is None:
        return [m.after_transport(st, t0, t1) for m, st in zip(models, stats)]
    futs = [pool.submit(m.after_transport, st, t0, t1) for m, st in zip(models, stats)]
    return [f.result() for f in futs]


def training_rows(specs, max_rows=1_000_000, iterations=2, update="fp64", form="graph", seed=1):
    """Training rows for the warm start from other models: the cell states
    that the plain update (FP64 by default) produced in the first
    ``iterations`` Lambda iterations of each model of ``specs`` in turn (e.g.
    the 64-model batch), until ``max_rows`` rows (a seeded subsample of the
    last model's rows fills the count).  Returns (x, t, info)."""
    t0 = time.perf_counter()
    xs, ts, used, upd_s = [], [], [], 0.0
    n = 0
    rng = np.random.default_rng(seed)
    for spec in specs:
        neb = nebula.build(spec)
        li = LambdaIteration(neb, form=form, update=update,
                             surrogate={"train_after": None, "capacity": (neb.ncells + 1) * iterations})
        for it in range(iterations):
            upd_s += li.step(seed=seed + 101 * it)["update_s"]
        x, t = li.ctx.surrogate_rows()
        li.close()
        if n + len(x) > max_rows:
            keep = np.sort(rng.choice(len(x), max_rows - n, replace=False))
            x, t = x[keep], t[keep]
        xs.append(x)
        ts.append(t)
        n += len(x)
        used.append(spec.name)
        if n >= max_rows:
            break
    x = np.concatenate(xs) if xs else np.zeros((0, 80), np.float32)
    t = np.concatenate(ts) if ts else np.zeros((0, 48), np.float32)
    return x, t, {"models": used, "rows": int(n), "iterations_per_model": iterations, "update": update,
                  "update_s": upd_s, "wall_s": time.perf_counter() - t0}

