#!/usr/bin/env python
"""Benchmark of the GB300 chemistry solver.

Workload: the primordial network (10 equations) on seeded cells drawn from
the 128^3-cell configuration's distributions (nH ~ logU(1, 1e6) cm^-3,
T ~ logU(10, 1e8) K, dtf = 0.1 t_ff per cell, rtol = 1e-6, atol = 1e-6 x);
``--config config3`` draws the heterogeneous-stiffness population instead
(nH ~ logU(1e-3, 1e12), T ~ logU(10, 1e9), 5 % in the thermally unstable
band).  One "step" is one hydro step: every cell integrated to its dtf with
the reference's per-cell backward-Euler driver; each step starts from the
previous step's state (atol reset to 1e-6 x before each step).

Every timed step is one call of the C entry point
``primordial_solve_cells_host`` with pinned host buffers: the call copies
the step's inputs to the device, solves, and copies the results back.
  * value: converged cell-steps per second of device time -- the solve's
    kernels between the copies, CUDA events recorded on the call's stream
    (``primordial_last_solve_ms``) -- counting cells whose solve ended OK and,
    by the seeded parity sample, within 1e-6 of the FP64 oracle;
  * e2e: the same count per second of wall time of the host calls (copies,
    launches, synchronisation included);
  * mixed: the same measurement with precision = DENGO_MIXED.
L2 is flushed (a 256 MB device write) before every step, outside the call.

Parity: the first ``--parity-sample`` cells are evolved through the same
steps by the oracle (the C restatement of the reference, pinned bit for bit
to the reference's own compiled solver) on the host cores; per step, cells
the oracle solved OK (in this and every earlier step) are compared.

--impl reference times the reference's CPU algorithm (the oracle) on the
host cores on a seeded subsample of the same cells, on the same config.
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
METRIC = "cells/s at <=1e-6 rel err vs FP64 oracle (mixed vs plain)"

# DRAM bytes per cell of one solver launch, from the ncu captures of the
# split engine on 14 592 cells (read + write; the state and tolerances, the
# tables stay in L2).
DRAM_BYTES_PER_CELL = {"fp64": 2.876928e6 / 14592, "mixed": 5.14512e6 / 14592,
                       "mixed_xf": 5.14512e6 / 14592}
# solver kernels per hydro step with a cost hint and a sweep budget: the
# three order kernels, the first launch, and two resume launches each after
# two list kernels (with the wide tail, FP64 and mixed: each resume launch
# followed by the wide engine's)
LAUNCHES_PER_STEP = 3 + 1 + 2 * (2 + 1)


def launches_per_step(precision, wide_tail):
    return LAUNCHES_PER_STEP + (2 if precision in ("fp64", "mixed") and wide_tail else 0)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cells", type=int, default=32768, help="cells per GPU")
    p.add_argument("--config", default="config2")
    p.add_argument("--precision", default="both",
                   choices=["both", "all", "fp64", "mixed", "mixed_xf"],
                   help="both: fp64 and mixed; all: also mixed_xf (the Newton matrix built "
                        "in extended-range FP32)")
    p.add_argument("--schedule", type=int, default=3, help="1 per-thread, 2 stride, 3 queue")
    p.add_argument("--block", type=int, default=0)
    p.add_argument("--parity-sample", type=int, default=256)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--order", type=int, default=1, help="start the costliest cells first")
    p.add_argument("--warps-per-cell", type=int, default=4, choices=[1, 2, 4])
    p.add_argument("--sweep-budget", type=int, default=2000,
                   help="> 0: redistribute cells still running after this many Newton "
                        "sweeps into later, densely packed launches (same results)")
    p.add_argument("--tail-grid", type=int, default=0)
    p.add_argument("--wide-tail", type=int, default=3,
                   help="FP64: set-aside cells per SM the wide engine takes (0: off)")
    p.add_argument("--max-substeps", type=int, default=50000,
                   help="the reference's cap; lower only to profile a short launch")
    p.add_argument("--no-parity", action="store_true")
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


def config_dict(args):
    """The workload both arms report (identical keys and values)."""
    return {"workload": "primordial network (10 equations), %d cells per GPU drawn from the "
                        "%s distributions (the 128^3 = 2,097,152-cell configuration's; a full "
                        "128^3 hydro step is minutes of device time because ~30%% of cells need "
                        "the 50,000-substep cap, so a seeded power-of-two subsample is timed), "
                        "%d consecutive hydro steps, per-cell dt control"
                        % (args.cells, args.config, args.steps),
            "network": "primordial", "cells": args.cells, "distributions": args.config,
            "hydro_steps": args.steps, "rtol": 1e-6, "atol": "1e-6 x state",
            "max_newton_sweeps": 10, "max_substeps": args.max_substeps,
            "l2": "flushed (256 MB device write) before every step"}


def oracle_tables():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    orc = Oracle("primordial")
    path = os.path.join(ROOT, "dengo_gb300", "generated", "primordial", "primordial_tables.dgt")
    return orc, orc.tables_from_bundle(path)


def oracle_steps(state, dtf, steps, nthreads=0):
    """The oracle through `steps` hydro steps (atol = 1e-6 x state at each
    step's start).  Returns per-step states and statuses and the wall time."""
    orc, tables = oracle_tables()
    cur = np.array(state, copy=True)
    out, t = [], 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        r = orc.evolve_cells(tables, cur, dtf, nthreads=nthreads)
        t += time.perf_counter() - t0
        out.append((r["state"].copy(), r["status"].copy()))
        cur = r["state"]
    return out, t


def cpu_baseline(state, dtf, seconds, nthreads=0):
    """The oracle on a bounded sample of the first step, all host cores."""
    orc, tables = oracle_tables()
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
            "sample": "the first %d of the cells, first hydro step, %.1f s wall" % (m, elapsed)}, m


def parity(gpu_steps, ref_steps, first_in):
    """Per step, the cells the oracle solved OK in this and every earlier
    step: relative error (and error floored at the solve's absolute
    tolerance, 1e-6 x the step's input) of the GPU's state."""
    alive = np.ones(len(first_in), bool)
    inp = first_in
    n_ok = n_ok_gpu = n6 = n10 = nbit = 0
    worst, worst_f = 0.0, 0.0
    for (g_st, g_status), (r_st, r_status) in zip(gpu_steps, ref_steps):
        alive &= r_status == 0
        sel = alive & (g_status == 0)
        if sel.any():
            d = np.abs(g_st[sel] - r_st[sel])
            with np.errstate(invalid="ignore", divide="ignore"):
                rel = np.where(d == 0, 0.0, d / np.abs(r_st[sel]))
                fl = np.where(d == 0, 0.0, d / np.maximum(np.abs(r_st[sel]), 1e-6 * np.abs(inp[sel])))
            rel = np.nan_to_num(rel, nan=np.inf)
            fl = np.nan_to_num(fl, nan=np.inf)
            worst = max(worst, float(rel.max()))
            worst_f = max(worst_f, float(fl.max()))
            n6 += int(np.all(fl <= 1e-6, axis=1).sum())
            n10 += int(np.all(rel <= 1e-10, axis=1).sum())
            nbit += int(np.all(g_st[sel] == r_st[sel], axis=1).sum())
        n_ok += int(alive.sum())
        n_ok_gpu += int(sel.sum())
        inp = r_st
    return {"sample_cells": int(len(first_in)), "steps": len(gpu_steps),
            "oracle_ok_cell_steps": n_ok, "gpu_ok_cell_steps": n_ok_gpu,
            "within_1e-6": n6, "within_1e-10": n10, "bit_identical": nbit,
            "frac_within_1e-6": (n6 / n_ok_gpu) if n_ok_gpu else None,
            "max_rel_err": worst, "max_floored_err": worst_f}


class HostArm:
    """K hydro steps of one precision through primordial_solve_cells_host
    with pinned host buffers."""

    def __init__(self, solver, state0, dtf, args, precision, torch):
        from dengo_gb300.runtime import CellBatch, DENGO_MIXED, DENGO_MIXED_XF, DENGO_FP64
        self.solver, self.args, self.torch = solver, args, torch
        n = len(dtf)
        self.n = n
        pin = lambda shape, dt: torch.empty(shape, dtype=dt, pin_memory=True).numpy()
        self.st = pin((n, NSPECIES), torch.float64)
        self.st[:] = state0
        self.at = pin((n, NSPECIES), torch.float64)
        self.dtf = pin((n,), torch.float64)
        self.dtf[:] = dtf
        self.dt = pin((n,), torch.float64)
        self.ttot = pin((n,), torch.float64)
        self.status = pin((n,), torch.int32)
        self.sweeps = pin((n,), torch.int32)
        self.hint = pin((n,), torch.int32)
        self.hint[:] = np.minimum(temperatures(state0), 2e9).astype(np.int32)
        cfg = solver.default_config()
        cfg.schedule, cfg.block = args.schedule, args.block
        cfg.precision = {"fp64": DENGO_FP64, "mixed": DENGO_MIXED,
                         "mixed_xf": DENGO_MIXED_XF}[precision]
        cfg.warps_per_cell = args.warps_per_cell
        cfg.sweep_budget, cfg.tail_grid = args.sweep_budget, args.tail_grid
        cfg.wide_tail = args.wide_tail
        cfg.max_substeps = args.max_substeps
        self.cfg = cfg
        a = lambda x: x.ctypes.data
        self.batch = CellBatch(n, NSPECIES, 1, a(self.st), a(self.at), None, 1e-6, a(self.dtf),
                               0.0, a(self.dt), a(self.ttot), a(self.status), None,
                               a(self.sweeps), None, a(self.hint) if args.order else None)
        self.fn = getattr(solver.lib, "primordial_solve_cells_host")
        self.ms = getattr(solver.lib, "primordial_last_solve_ms")
        # bytes the call copies per step: state, atol, dtf, dt, cost hint in;
        # state, atol, dt, ttot, status, sweeps out
        self.h2d = 2 * n * NSPECIES * 8 + 2 * n * 8 + (n * 4 if args.order else 0)
        self.d2h = 2 * n * NSPECIES * 8 + 2 * n * 8 + 2 * n * 4

    def step(self, first):
        """One hydro step; returns (wall seconds of the call, device ms of
        its solve)."""
        np.multiply(self.st, 1e-6, out=self.at)
        self.dt[:] = -1.0
        if not first and self.args.order:
            self.hint[:] = self.sweeps
        t0 = time.perf_counter()
        rc = self.fn(self.solver.data, C.byref(self.batch), -1.0, C.byref(self.cfg))
        t1 = time.perf_counter()
        if rc != 0:
            raise RuntimeError("primordial_solve_cells_host failed: " + self.solver.last_error())
        return t1 - t0, float(self.ms(self.solver.data))


def run_arm(solver, state0, dtf, args, precision, torch, flush, sample):
    """Warm-up on a 4096-cell copy, then the timed steps.  Returns a dict."""
    wn = min(len(dtf), 4096)
    warm = HostArm(solver, state0[:wn], dtf[:wn], args, precision, torch)
    for k in range(args.warmup):
        warm.step(k == 0)
    arm = HostArm(solver, state0, dtf, args, precision, torch)
    wall, dev, ok, sw = [], [], 0, 0
    samples = []
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        w, d = arm.step(k == 0)
        wall.append(w)
        dev.append(d)
        ok += int((arm.status == 0).sum())
        sw += int(arm.sweeps.astype(np.int64).sum())
        samples.append((arm.st[:sample].copy(), arm.status[:sample].copy()))
    return {"wall_s": wall, "dev_ms": dev, "ok": ok, "sweeps": sw, "samples": samples,
            "h2d": arm.h2d, "d2h": arm.d2h}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from dengo_gb300.workloads import primordial_cells, PRIMORDIAL_CONFIGS
    state, dtf = primordial_cells(args.cells, args.config,
                                  seed=PRIMORDIAL_CONFIGS[args.config]["seed"])
    per_step = max(2.0, 150.0 / max(1, args.steps + args.warmup))
    base, m = cpu_baseline(state, dtf, per_step * 3)
    orc, tables = oracle_tables()
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
    sample = ("the first %d of the same seeded cells (a subsample of the GPU arm's %d), "
              "%d hydro steps, all %d host cores (OpenMP over cells)"
              % (m, args.cells, args.steps, base["cores"]))
    line = {"impl": "reference", "metric": METRIC,
            "value": value, "unit": "cells/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": config_dict(args),
            "cpu_baseline": dict(base, value=value, sample=sample),
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

    n = args.cells
    seed = PRIMORDIAL_CONFIGS[args.config]["seed"] + 1000 * rank
    state0, dtf = primordial_cells(n, args.config, seed=seed)
    solver = Solver("primordial")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    sample = 0 if args.no_parity else min(args.parity_sample, n)
    precisions = {"both": ["fp64", "mixed"], "all": ["fp64", "mixed", "mixed_xf"]}.get(
        args.precision, [args.precision])

    clocks = Clocks(dev.index)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    arms = {p: run_arm(solver, state0, dtf, args, p, torch, flush, sample) for p in precisions}
    torch.cuda.synchronize()
    clk = clocks.stop()
    # whole-job figures: device time and wall time are the max over ranks,
    # converged cells the sum
    for p, a in arms.items():
        a["dev_total_ms"] = float(sum(a["dev_ms"]))
        a["wall_total_s"] = float(sum(a["wall_s"]))
        if dist:
            t = torch.tensor([a["dev_total_ms"], a["wall_total_s"]], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            a["dev_total_ms"], a["wall_total_s"] = float(t[0]), float(t[1])
            c = torch.tensor([a["ok"], a["sweeps"]], device=dev, dtype=torch.int64)
            dist.all_reduce(c)
            a["ok_all"], a["sweeps_all"] = int(c[0]), int(c[1])
        else:
            a["ok_all"], a["sweeps_all"] = a["ok"], a["sweeps"]
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    par = {}
    if sample:
        ref_steps, _ = oracle_steps(state0[:sample], dtf[:sample], args.steps)
        for p, a in arms.items():
            par[p] = parity(a["samples"], ref_steps, state0[:sample])

    def figures(p):
        a = arms[p]
        frac = par[p]["frac_within_1e-6"] if p in par and par[p]["frac_within_1e-6"] is not None \
            else 1.0
        conv = a["ok_all"] / (a["dev_total_ms"] / 1e3)
        return {"value": conv * frac, "converged_cells_per_s": conv,
                "frac_within_1e-6": frac,
                "ms_per_step": a["dev_total_ms"] / args.steps,
                "step_ms": a["dev_ms"],
                "e2e": {"value": a["ok_all"] * frac / a["wall_total_s"], "unit": "cells/s",
                        "h2d_bytes_per_step": a["h2d"], "d2h_bytes_per_step": a["d2h"],
                        "seconds": a["wall_total_s"], "steps": args.steps,
                        "path": "primordial_solve_cells_host, pinned host buffers, the same "
                                "steps and solver configuration as value"},
                "parity": par.get(p)}

    peak = measure_fp64_peak()
    main = precisions[0]
    f = figures(main)
    a = arms[main]
    achieved = a["sweeps_all"] * F_SWEEP / (a["dev_total_ms"] / 1e3) / 1e12
    engine = {"precision": main, "warps_per_cell": args.warps_per_cell,
              "schedule": args.schedule, "sweep_budget": args.sweep_budget,
              "wide_tail": args.wide_tail,
              "order": "costliest first (cost hint)" if args.order else "input order",
              "warmup": "%d steps over a 4096-cell copy" % args.warmup}
    line = {
        "metric": METRIC, "value": f["value"], "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if main == "fp64" else "f64 residual + f32 LU",
        "data": "synthetic (seeded)", "config": config_dict(args), "engine": engine,
        "converged_cells_per_s": f["converged_cells_per_s"],
        "frac_within_1e-6": f["frac_within_1e-6"], "step_ms": f["step_ms"],
        "gpu_launches": args.steps * sum(launches_per_step(p, args.wide_tail)
                                         for p in precisions),
        "clocks": clk,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                     "traffic": DRAM_BYTES_PER_CELL[main] * n,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "14 592-cell launch (profiles/evolve_split_%s_cold14592.md)"
                                       ", scaled by cells" % main,
                     "peak_source": "of measured: FP64 FMA throughput of this GPU "
                                    "(dg_peak.cu), this run; MEASURED_PEAKS.json has no "
                                    "FP64 figure; the path cannot contract its multiply-adds "
                                    "(the reference's rounding), so peak/2 is its ceiling",
                     "flop_per_sweep": F_SWEEP},
        "e2e": f["e2e"], "parity": f["parity"],
    }
    for other in ("mixed", "mixed_xf"):
        if other in arms and main != other:
            m = figures(other)
            m["speedup_vs_fp64"] = m["value"] / f["value"] if f["value"] else None
            m["e2e_speedup_vs_fp64"] = (m["e2e"]["value"] / f["e2e"]["value"]
                                        if f["e2e"]["value"] else None)
            line[other] = m
    if not args.no_cpu_baseline:
        base, _ = cpu_baseline(state0, dtf, args.cpu_seconds)
        line["cpu_baseline"] = base
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
