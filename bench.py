#!/usr/bin/env python
"""Benchmark of the GB300 chemistry solver.

Workload: the primordial network (10 equations) on seeded cells drawn from
the 128^3 configuration's distributions (nH ~ logU(1, 1e6) cm^-3,
T ~ logU(10, 1e8) K, dtf = 0.1 t_ff per cell, rtol = 1e-6, atol = 1e-6 x),
SoA state resident on the device.  One "step" is one hydro step: one
solver launch over every cell, each cell integrated to its dtf with the
reference's per-cell backward-Euler driver; the state carries over from step
to step (atol is reset to 1e-6 x before each step).

Metric: converged cell-steps per second -- cells whose solve ended with
status OK, summed over the timed steps, divided by the summed device time of
the solver launches (CUDA events on the launching stream, L2 flushed before
every step).  A seeded sample of the first step is checked against the
oracle (C restatement of the reference) and the fraction within 1e-6 and
1e-10 relative is reported.

--impl reference times the reference's CPU algorithm (the oracle, the
reference's own code when it was built here) on the host cores instead.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic FP64 work of one Newton sweep of one primordial cell: RHS 258 +
# Jacobian 354 + interpolation 5*44 + T 40 + residual 60 + scaling of I-dtJ
# 310 + Gauss elimination 805 + update/test 40 (sympy op counts of the
# generated expressions and exact LU flop count, N = 10).
F_SWEEP = 2090.0
NSPECIES = 10


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cells", type=int, default=32768, help="cells per GPU")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--config", default="config2")
    p.add_argument("--schedule", type=int, default=3, help="1 per-thread, 2 stride, 3 queue")
    p.add_argument("--block", type=int, default=0)
    p.add_argument("--parity-sample", type=int, default=48)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--order", type=int, default=1, help="start the costliest cells first")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--warps-per-cell", type=int, default=4, choices=[1, 2, 4])
    p.add_argument("--sweep-budget", type=int, default=2000,
                   help="> 0: redistribute cells still running after this many Newton "
                        "sweeps into a second, densely packed launch (same results)")
    p.add_argument("--tail-grid", type=int, default=0)
    p.add_argument("--max-substeps", type=int, default=50000,
                   help="the reference's cap; lower only to profile a short launch")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(rows[0][2]),
                "reasons": sorted(reasons), "samples": len(rows)}


# DRAM bytes per cell of one solver launch, from the ncu captures of the
# split engine on 14 592 cells (read + write; the state and tolerances, the
# tables stay in L2).
DRAM_BYTES_PER_CELL = {"fp64": 2.876928e6 / 14592, "mixed": 5.14512e6 / 14592}


def temperatures(state):
    """Gas temperature of each cell (mass densities + ge), gamma = 5/3."""
    from dengo_gb300.workloads import KB, MH, PRIMORDIAL_ORDER, PRIMORDIAL_WEIGHTS
    w = np.array([PRIMORDIAL_WEIGHTS[s] for s in PRIMORDIAL_ORDER[:-1]])
    n = state[:, :-1] / (w * MH)
    density = (n[:, :-1] * w[:-1]).sum(axis=1)
    return density * state[:, -1] * MH / (KB * 1.5 * n.sum(axis=1))


def measure_fp64_peak():
    from dengo_gb300.build import PKG
    lib = C.CDLL(os.path.join(PKG, "lib", "libdg_peak.so"))
    lib.dg_measure_fma_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    best = 0.0
    for _ in range(3):
        t = C.c_double()
        if lib.dg_measure_fma_peak(1, 4000, C.byref(t)) == 0:
            best = max(best, t.value)
    return best


def cpu_baseline(state, dtf, seconds, nthreads=0):
    """The oracle on a bounded sample of the workload, all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    from dengo_gb300.tablefile import read_table_file
    from dengo_gb300.build import network_dir
    from dengo_gb300.runtime import load_library
    lib = load_library("primordial")
    order = [lib.primordial_table_name(k).decode() for k in range(lib.primordial_ntables())]
    tabs = read_table_file(os.path.join(network_dir("primordial"), "primordial_tables.dgt"))
    tables = [tabs[k] for k in order]
    orc = Oracle("primordial")
    cores = nthreads or os.cpu_count()
    m, elapsed, res = 64, 0.0, None
    while True:
        m = min(m, len(dtf))
        t0 = time.perf_counter()
        res = orc.evolve_cells(tables, state[:m], dtf[:m], nthreads=cores)
        elapsed = time.perf_counter() - t0
        if elapsed >= seconds / 3 or m >= len(dtf) or m >= 8192:
            break
        m *= 2
    ok = int((res["status"] == 0).sum())
    return {"value": ok / elapsed, "unit": "cells/s", "cores": cores, "kind": "port",
            "sample": "%d cells of the first step (seeded subsample), one hydro step each, "
                      "%.1f s wall" % (m, elapsed)}, res, m


def metric_name(precision):
    """The metric both arms report."""
    return ("converged cell-steps/s (primordial, per-cell BE Newton, %s path)"
            % ("FP64 plain" if precision == "fp64" else "mixed FP32-LU"))


def workload_name(cells, steps):
    return ("primordial network, %d cells per GPU drawn from the 128^3 configuration's "
            "distributions, %d consecutive hydro steps, state resident on the device"
            % (cells, steps))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from dengo_gb300.workloads import primordial_cells
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    state, dtf = primordial_cells(args.cells, args.config)
    per_step = max(2.0, 150.0 / max(1, args.steps + args.warmup))
    base, _, m = cpu_baseline(state, dtf, per_step * 3)
    from oracle import Oracle
    from dengo_gb300.tablefile import read_table_file
    from dengo_gb300.build import network_dir
    from dengo_gb300.runtime import load_library
    lib = load_library("primordial")
    order = [lib.primordial_table_name(k).decode() for k in range(lib.primordial_ntables())]
    tabs = read_table_file(os.path.join(network_dir("primordial"), "primordial_tables.dgt"))
    tables = [tabs[k] for k in order]
    orc = Oracle("primordial")
    cur = state[:m].copy()
    for _ in range(args.warmup):
        orc.evolve_cells(tables, cur[:8], dtf[:8], nthreads=base["cores"])
    ok_total, t_total = 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r = orc.evolve_cells(tables, cur, dtf[:m], nthreads=base["cores"])
        t_total += time.perf_counter() - t0
        ok_total += int((r["status"] == 0).sum())
        cur = r["state"]
    value = ok_total / t_total
    line = {"impl": "reference", "metric": metric_name("fp64"),
            "value": value, "unit": "cells/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": workload_name(args.cells, args.steps),
                       "sample": "%d of the cells per step (%s distributions), on the host "
                                 "cores" % (m, args.config),
                       "cells_per_step": m},
            "cpu_baseline": dict(base, value=value,
                                 sample="%d cells per step x %d steps" % (m, args.steps)),
            "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import PRIMORDIAL_CONFIGS, primordial_cells

    n, N = args.cells, NSPECIES
    seed = PRIMORDIAL_CONFIGS[args.config]["seed"] + 1000 * rank
    state0, dtf = primordial_cells(n, args.config, seed=seed)
    solver = Solver("primordial")
    stream = torch.cuda.current_stream()
    cfg = Solver.default_config()
    cfg.schedule, cfg.block = args.schedule, args.block
    cfg.precision = 1 if args.precision == "mixed" else 0
    cfg.warps_per_cell = args.warps_per_cell
    cfg.sweep_budget, cfg.tail_grid = args.sweep_budget, args.tail_grid
    cfg.max_substeps = args.max_substeps

    def device_batch(st_host):
        st = torch.tensor(np.ascontiguousarray(st_host.T), device=dev)   # SoA: [species][cell]
        return st

    st = device_batch(state0)
    at = torch.empty_like(st)
    d_dtf = torch.tensor(dtf, device=dev)
    status = torch.zeros(n, dtype=torch.int32, device=dev)
    sweeps = torch.zeros(n, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)

    def step(state, atol, cells, ld):
        torch.mul(state, 1e-6, out=atol)
        solver.solve_device(state, cells, 1, ld, atol, rtol_scalar=1e-6, dtf=d_dtf,
                            status=status, sweeps=sweeps, config=cfg, stream=stream)

    # warm-up: W steps over a subset copy (same kernel, same code path)
    wn = min(n, 4096)
    wst = st[:, :wn].contiguous()
    wat = torch.empty_like(wst)
    for _ in range(args.warmup):
        step(wst, wat, wn, wn)
    torch.cuda.synchronize()
    del wst, wat

    t_hint = torch.tensor(np.minimum(temperatures(state0), 2e9).astype(np.int32), device=dev)
    ok_count = torch.zeros((), dtype=torch.int64, device=dev)
    sweep_sum = torch.zeros((), dtype=torch.int64, device=dev)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sample = min(args.parity_sample, n)
    step1_in = state0[:sample].copy()
    step1_out = None
    clocks = Clocks(dev.index)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        torch.mul(st, 1e-6, out=at)
        ev0[k].record(stream)
        # longest-first order: the previous step's sweep counts, or for the
        # first step the initial temperature (the stiff cells are the hot ones)
        solver.solve_device(st, n, 1, n, at, rtol_scalar=1e-6, dtf=d_dtf, status=status,
                            sweeps=sweeps, config=cfg, stream=stream,
                            cost_hint=(t_hint if k == 0 else sweeps) if args.order else None)
        ev1[k].record(stream)
        ok_count += (status == 0).sum()
        sweep_sum += sweeps.sum(dtype=torch.int64)
        if k == 0:
            step1_out = st[:, :sample].T.contiguous().cpu().numpy()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    total_ms = float(sum(step_ms))
    ok_local = int(ok_count.item())
    flops = float(sweep_sum.item()) * F_SWEEP
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
        c = torch.tensor([ok_local], device=dev, dtype=torch.int64)
        dist.all_reduce(c)
        ok_all = int(c.item())
    else:
        ok_all = ok_local
    value = ok_all / (total_ms / 1e3)

    # end to end through the host-buffer C entry point
    e2e = None
    if not args.no_e2e:
        hst = state0.copy()
        e2e_ok, e2e_t = 0, 0.0
        h2d = d2h = 0
        e2e_steps = max(1, min(args.steps, args.e2e_steps))
        for k in range(e2e_steps):
            atol_h = 1e-6 * hst
            t0 = time.perf_counter()
            r = solver.solve_host(hst, dtf, atol=atol_h)
            e2e_t += time.perf_counter() - t0
            hst = r["state"]
            e2e_ok += int((r["status"] == 0).sum())
        h2d = 2 * n * N * 8 + 2 * n * 8              # state, atol, dtf, dt
        d2h = 2 * n * N * 8 + 2 * n * 8 + n * 4      # state, atol, dt, ttot, status
        e2e = {"value": e2e_ok * world / e2e_t, "unit": "cells/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "seconds": e2e_t, "steps": e2e_steps,
               "path": "primordial_solve_cells_host (host buffers, copies inside the call)"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    peak = measure_fp64_peak()
    achieved = flops / (total_ms / 1e3) / 1e12
    line = {
        "metric": metric_name(args.precision),
        "value": value, "unit": "cells/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f64 residual + f32 LU",
        "data": "synthetic (seeded)",
        "config": {"workload": workload_name(n, args.steps),
                   "cells_per_gpu": n, "precision": args.precision, "schedule": args.schedule,
                   "order": "costliest first" if args.order else "input order",
                   "warps_per_cell": args.warps_per_cell,
                   "sweep_budget": args.sweep_budget,
                   "l2": "flushed (256 MB write) before every step",
                   "warmup": "%d steps over a %d-cell copy" % (args.warmup, wn)},
        "wall_s": wall, "step_ms": step_ms, "gpu_launches": args.steps * ((4 if args.sweep_budget > 0 else 1) + (3 if args.order else 0)),
        "clocks": clk,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                     "traffic": DRAM_BYTES_PER_CELL[args.precision] * n,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "14 592-cell launch (profiles/evolve_split_%s_cold14592.md)"
                                       ", scaled by cells" % args.precision,
                     "peak_source": "measured FP64 FMA throughput (dg_peak.cu), this run",
                     "flop_per_sweep": F_SWEEP},
    }
    if e2e:
        line["e2e"] = e2e
    # parity sample and CPU baseline (oracle on the host cores)
    if not args.no_cpu_baseline:
        base, res, m = cpu_baseline(state0, dtf, args.cpu_seconds)
        line["cpu_baseline"] = base
        ref = res["state"][:sample]
        okm = res["status"][:sample] == 0
        with np.errstate(invalid="ignore", divide="ignore"):
            rel = np.abs(step1_out - ref) / np.maximum(np.abs(ref), 1e-300)
        rel[step1_out == ref] = 0
        r_ok = rel[okm]
        # relative error with entries below the solve's absolute tolerance
        # (1e-6 x the input) measured against that tolerance
        floored = (np.abs(step1_out - ref) / np.maximum(np.abs(ref), 1e-6 * np.abs(step1_in)))[okm]
        line["parity"] = {"sample_cells": int(sample), "ok_in_oracle": int(okm.sum()),
                          "max_rel_err_ok": float(r_ok.max(initial=0.0)),
                          "max_floored_err_ok": float(floored.max(initial=0.0)),
                          "frac_floored_within_1e-6": float(np.mean(np.all(floored <= 1e-6, axis=1)))
                          if okm.any() else None,
                          "frac_within_1e-6": float(np.mean(np.all(r_ok <= 1e-6, axis=1)))
                          if okm.any() else None,
                          "frac_within_1e-10": float(np.mean(np.all(r_ok <= 1e-10, axis=1)))
                          if okm.any() else None,
                          "bit_identical": int(np.all(step1_out == ref, axis=1).sum())}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
