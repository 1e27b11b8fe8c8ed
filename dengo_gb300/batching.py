"""Batching for repeated hydro steps: an autotuner over the engine's launch
variants and CUDA-graph capture of a hydro step.

Engine variants (``dengo_solver_config``):

* ``warps_per_cell`` 1 -- the single-lane engine, one cell per lane,
  ``block`` 32/64/128 cells per CTA -- or 2/4 -- the split engine, 32 cells
  per CTA and each cell's Newton sweep divided over 2 or 4 warps;
* ``schedule`` -- the persistent work queue (lanes take the next cell from an
  atomic counter when theirs finishes), a static stride, or one cell per
  thread with no refill (the plain one-cell-per-thread launch);
* the longest-first cell order from a cost hint (the previous step's sweep
  counts), or none.

``autotune`` times every candidate on a seeded sample of the caller's cells
(each trial on the device, CUDA events, a warm-up launch first) and returns
the fastest; the measured table is kept in a JSON cache keyed by network,
precision, GPU and sample, so a process tunes once per workload.

``StepGraph`` captures one hydro step -- atol = 1e-6 x state, then the
solve with the previous step's sweep counts as cost hint (with a sweep
budget: both launches of the stiff-cell redistribution and the list built
between them) -- into a CUDA graph over fixed device buffers, and replays it
for every later step.
"""

import hashlib
import json
import os

import numpy as np

from .runtime import (SCHED_PER_THREAD, SCHED_QUEUE, SCHED_STRIDE, Solver)

SCHEDULES = {"queue": SCHED_QUEUE, "stride": SCHED_STRIDE, "per_thread": SCHED_PER_THREAD}


def candidates():
    """The launch variants the tuner compares."""
    out = []
    for wpc, blocks in ((4, (0,)), (2, (0,)), (1, (32, 64, 128))):
        for block in blocks:
            for sched in ("queue", "stride"):
                for order in (True, False):
                    out.append(dict(warps_per_cell=wpc, block=block, schedule=sched, order=order))
    return out


def make_config(c, precision=0, max_substeps=50000):
    cfg = Solver.default_config()
    cfg.warps_per_cell = c["warps_per_cell"]
    cfg.block = c["block"]
    cfg.schedule = SCHEDULES[c["schedule"]]
    cfg.precision = precision
    cfg.max_substeps = max_substeps
    return cfg


def _cache_path():
    base = os.environ.get("DENGO_AUTOTUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "dengo_gb300", "autotune.json")
    return base


def _key(solver, precision, state, dtf, max_substeps):
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    h = hashlib.sha256(np.ascontiguousarray(state).tobytes())
    h.update(np.ascontiguousarray(dtf).tobytes())
    return "%s|p%d|%s|%dsm|%d|%s" % (solver.name, precision, p.name, p.multi_processor_count,
                                    max_substeps, h.hexdigest()[:16])


def time_variant(solver, c, d_state, d_dtf, precision=0, max_substeps=50000, repeats=2,
                 hint=None):
    """Median device time (ms) of one solve of the sample with variant ``c``
    (from the same initial state each time) and the sweeps it took."""
    import torch
    n, nsp = d_state.shape
    cfg = make_config(c, precision, max_substeps)
    stream = torch.cuda.current_stream()
    st = torch.empty_like(d_state)
    at = torch.empty_like(d_state)
    status = torch.empty(n, dtype=torch.int32, device=d_state.device)
    sweeps = torch.empty(n, dtype=torch.int32, device=d_state.device)
    times = []
    for k in range(repeats + 1):
        st.copy_(d_state)
        torch.mul(st, 1e-6, out=at)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.solve_device(st, n, nsp, 1, at, rtol_scalar=1e-6, dtf=d_dtf, status=status,
                            sweeps=sweeps, config=cfg, stream=stream,
                            cost_hint=hint if c["order"] else None)
        e1.record(stream)
        e1.synchronize()
        if k:
            times.append(e0.elapsed_time(e1))
    return float(np.median(times)), int(sweeps.sum(dtype=torch.int64).item())


def autotune(solver, state, dtf, precision=0, sample=4096, max_substeps=2000, repeats=2,
             cands=None, cache=True, seed=0):
    """Pick the fastest launch variant for cells like ``state`` (AoS host
    array) with step lengths ``dtf``.  The sample is a seeded subset of at
    most ``sample`` cells; ``max_substeps`` bounds each trial (the variants
    are compared on the same bounded work).  Returns ``(best, table)``."""
    import torch
    state = np.asarray(state, np.float64)
    dtf = np.broadcast_to(np.asarray(dtf, np.float64), (state.shape[0],))
    if state.shape[0] > sample:
        idx = np.sort(np.random.Generator(np.random.PCG64(seed)).choice(
            state.shape[0], sample, replace=False))
        state, dtf = state[idx], dtf[idx]
    key = _key(solver, precision, state, dtf, max_substeps)
    path = _cache_path()
    if cache and os.path.exists(path):
        try:
            with open(path) as f:
                hit = json.load(f).get(key)
            if hit:
                return hit["best"], hit["table"]
        except (OSError, ValueError):
            pass
    dev = torch.device("cuda", torch.cuda.current_device())
    d_state = torch.tensor(state, device=dev)
    d_dtf = torch.tensor(np.ascontiguousarray(dtf), device=dev)
    # cost hint for the ordered variants: the sweeps of a plain solve
    hint = torch.empty(state.shape[0], dtype=torch.int32, device=dev)
    _hint_from_solve(solver, d_state, d_dtf, hint, precision, max_substeps)
    table = []
    for c in (cands or candidates()):
        ms, sw = time_variant(solver, c, d_state, d_dtf, precision, max_substeps, repeats, hint)
        table.append(dict(c, ms=ms, sweeps=sw))
    best = min(table, key=lambda r: r["ms"])
    best = {k: best[k] for k in ("warps_per_cell", "block", "schedule", "order")}
    if cache:
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            data = {}
            if os.path.exists(path):
                with open(path) as f:
                    data = json.load(f)
            data[key] = dict(best=best, table=table)
            with open(path, "w") as f:
                json.dump(data, f, indent=1)
        except (OSError, ValueError):
            pass
    return best, table


def _hint_from_solve(solver, d_state, d_dtf, hint, precision, max_substeps):
    import torch
    n, nsp = d_state.shape
    st = d_state.clone()
    at = st * 1e-6
    cfg = make_config(dict(warps_per_cell=4, block=0, schedule="queue", order=False), precision,
                      max_substeps)
    solver.solve_device(st, n, nsp, 1, at, rtol_scalar=1e-6, dtf=d_dtf, sweeps=hint, config=cfg,
                        stream=torch.cuda.current_stream())
    torch.cuda.current_stream().synchronize()


class StepGraph:
    """One hydro step over resident device buffers, captured as a CUDA graph.

    ``state`` is a (cells, N) CUDA tensor (AoS) updated in place by every
    ``replay``; ``dtf`` a per-cell CUDA tensor.  The step sets atol = 1e-6 x
    state and solves with the previous step's sweep counts as the cost hint
    (when the variant orders cells).  Two eager steps run before capture: they
    size the solver's scratch, so the captured launches allocate nothing."""

    def __init__(self, solver, state, dtf, config, order=True, stream=None):
        import torch
        self.torch = torch
        self.solver, self.state, self.dtf, self.config = solver, state, dtf, config
        n = state.shape[0]
        self.atol = torch.empty_like(state)
        self.status = torch.zeros(n, dtype=torch.int32, device=state.device)
        self.sweeps = torch.zeros(n, dtype=torch.int32, device=state.device)
        self.order = order
        self.stream = stream or torch.cuda.Stream(device=state.device)
        self.graph = None

    def _step(self):
        n, nsp = self.state.shape
        self.torch.mul(self.state, 1e-6, out=self.atol)
        self.solver.solve_device(self.state, n, nsp, 1, self.atol, rtol_scalar=1e-6, dtf=self.dtf,
                                 status=self.status, sweeps=self.sweeps, config=self.config,
                                 stream=self.stream,
                                 cost_hint=self.sweeps if self.order else None)

    def eager(self):
        """One step without the graph (also sizes scratch before capture)."""
        with self.torch.cuda.stream(self.stream):
            self._step()

    def capture(self, warm_state=None):
        """Capture the step.  The warm-up steps solve a copy of the state
        (or ``warm_state``), so the caller's state is not advanced."""
        torch = self.torch
        keep = self.state
        self.state = (warm_state if warm_state is not None else keep.clone())
        self.eager()
        self.eager()
        self.stream.synchronize()
        self.state = keep
        self.sweeps.zero_()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._step()
        return self

    def replay(self):
        with self.torch.cuda.stream(self.stream):
            self.graph.replay()


def compare(network="primordial", config="config3", cells=16384, steps=3, precision=0, seed=None,
            sweep_budget=2000):
    """Config-3 comparison: the plain one-cell-per-thread launch (block 64,
    no refill, no ordering, eager launches) against the persistent work queue
    with the autotuned variant, stiff-cell redistribution after
    ``sweep_budget`` sweeps and graph-captured steps, on the same seeded
    cells and the same number of hydro steps.  Returns a dict with both arms'
    device times and converged cells/s."""
    import torch
    from .workloads import primordial_cells
    solver = Solver(network)
    state, dtf = primordial_cells(cells, config, seed=seed)
    dev = torch.device("cuda", torch.cuda.current_device())
    d_dtf = torch.tensor(dtf, device=dev)
    out = {"network": network, "workload": config, "cells": cells, "steps": steps}

    def run(graph_step, label):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(steps)]
        ok = 0
        for k in range(steps):
            ev[k][0].record(graph_step.stream)
            graph_step.replay() if graph_step.graph is not None else graph_step.eager()
            ev[k][1].record(graph_step.stream)
            graph_step.stream.synchronize()
            ok += int((graph_step.status == 0).sum().item())
        ms = [a.elapsed_time(b) for a, b in ev]
        out[label] = {"step_ms": ms, "total_ms": float(sum(ms)),
                      "converged_cells_per_s": ok / (sum(ms) / 1e3)}

    base_cfg = make_config(dict(warps_per_cell=1, block=64, schedule="per_thread", order=False),
                           precision)
    run(StepGraph(solver, torch.tensor(state, device=dev), d_dtf, base_cfg, order=False),
        "one_cell_per_thread")
    best, table = autotune(solver, state, dtf, precision=precision)
    out["autotuned"] = best
    out["autotune_table"] = table
    cfg = make_config(best, precision)
    cfg.sweep_budget = sweep_budget
    out["sweep_budget"] = sweep_budget
    g = StepGraph(solver, torch.tensor(state, device=dev), d_dtf, cfg, order=best["order"])
    g.capture()
    run(g, "persistent_graph_autotuned")
    out["speedup"] = (out["one_cell_per_thread"]["total_ms"] /
                      out["persistent_graph_autotuned"]["total_ms"])
    return out


if __name__ == "__main__":
    import argparse
    p = argparse.ArgumentParser(description="one-cell-per-thread vs persistent + graph + "
                                            "autotuned, on seeded cells")
    p.add_argument("--network", default="primordial")
    p.add_argument("--config", default="config3")
    p.add_argument("--cells", type=int, default=16384)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--precision", type=int, default=0)
    p.add_argument("--sweep-budget", type=int, default=2000)
    a = p.parse_args()
    print(json.dumps(compare(a.network, a.config, a.cells, a.steps, a.precision,
                             sweep_budget=a.sweep_budget)))
