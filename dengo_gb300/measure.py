"""Measurement runs of the configurations the bench line does not cover.

    python -m dengo_gb300.measure config4 [--cells N]
        The oxygen ion-by-ion network (16 equations, 8192-bin tables) on
        seeded cells (T ~ logU(1e4, 1e9) K, nH ~ logU(1e-4, 1e2) cm^-3,
        O/H = 4.9e-4, ionisation state a seeded Dirichlet draw per element,
        dtf ~ logU(1e10, 1e12) s): one hydro step of every cell in FP64 and in
        mixed precision (state resident on the device, CUDA events on the
        launching stream), converged cells/s of each, and each species'
        error against the FP64 oracle on a seeded sample.

    python -m dengo_gb300.measure config5 [--rate R --duration S ...]
        The serving loop (dengo_gb300.serving) under Poisson arrivals of
        cubic cell patches, 70/30 primordial (config-3 distributions) /
        oxygen (config-4 distributions), dtf ~ logU(1e8, 1e12) s, an HBM
        budget; p50/p99/p99.9 latency, the served throughput against the same
        requests submitted at once, and for every served request its
        critical-path floor: its stiffest cell's Newton sweeps times the
        measured time of one sweep of a lone cell -- the latency no schedule
        can beat, since a cell's sweeps run one after another.

    python -m dengo_gb300.measure tail [--per-sm 1 2 3 6 --budget 50 --precision fp64]
        The last launches of a hydro step: one stiff primordial cell (the
        config-2 "hot" seeded set) copied k times per SM, set aside after
        --budget sweeps and resumed, once by the split engine (wide_tail 0)
        and once by the wide engine (wide_tail k); microseconds per Newton
        sweep of each, the time a step's stiffest cells take per sweep.

Each prints one JSON line.
"""
import json
import os
import sys
import time

import numpy as np

from .runtime import DENGO_FP64, DENGO_MIXED, Solver


def _device_step(torch, solver, state, dtf, precision, stream):
    """One hydro step of every cell on the device (SoA); returns
    (ms, status, sweeps, final state AoS)."""
    n, N = state.shape
    st = torch.tensor(np.ascontiguousarray(state.T), device="cuda")
    at = st * 1e-6
    d_dtf = torch.tensor(dtf, device="cuda")
    status = torch.zeros(n, dtype=torch.int32, device="cuda")
    sweeps = torch.zeros(n, dtype=torch.int32, device="cuda")
    cfg = Solver.default_config()
    cfg.precision = precision
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    solver.solve_device(st, n, 1, n, at, rtol_scalar=1e-6, dtf=d_dtf, status=status,
                        sweeps=sweeps, config=cfg, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return (e0.elapsed_time(e1), status.cpu().numpy(), sweeps.cpu().numpy(),
            st.T.contiguous().cpu().numpy())


def config4(cells=1 << 20, sample=256, seed=20246):
    import torch
    from .workloads import OXYGEN_ORDER, oxygen_cells
    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    solver = Solver("oxygen")
    state, dtf = oxygen_cells(cells, seed=seed)
    # warm-up on a small copy
    _device_step(torch, solver, state[:4096], dtf[:4096], DENGO_FP64, stream)
    _device_step(torch, solver, state[:4096], dtf[:4096], DENGO_MIXED, stream)
    out = {"workload": "oxygen ion-by-ion network (16 equations, 8192-bin tables), %d seeded "
                       "cells, one hydro step, state resident on the device" % cells,
           "cells": cells}
    res = {}
    for name, prec in (("fp64", DENGO_FP64), ("mixed", DENGO_MIXED)):
        ms, status, sweeps, final = _device_step(torch, solver, state, dtf, prec, stream)
        ok = int((status == 0).sum())
        res[name] = final, status
        out[name] = {"ms": ms, "converged": ok, "converged_cells_per_s": ok / (ms / 1e3),
                     "sweeps": int(sweeps.astype(np.int64).sum())}
    out["mixed"]["speedup_vs_fp64"] = (out["mixed"]["converged_cells_per_s"] /
                                       out["fp64"]["converged_cells_per_s"])
    # per-species error of both paths against the FP64 oracle on a sample
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    from oracle import Oracle
    orc = Oracle("oxygen")
    tabs = orc.tables_from_bundle(os.path.join(root, "dengo_gb300", "generated", "oxygen",
                                               "oxygen_tables.dgt"))
    ref = orc.evolve_cells(tabs, state[:sample], dtf[:sample])
    okr = ref["status"] == 0
    for name in ("fp64", "mixed"):
        final, status = res[name]
        g = final[:sample]
        sel = okr & (status[:sample] == 0)
        d = np.abs(g[sel] - ref["state"][sel])
        err = np.where(d == 0, 0.0, d / np.maximum(np.abs(ref["state"][sel]),
                                                     1e-6 * np.abs(state[:sample][sel])))
        out[name]["sample"] = {"cells": sample, "oracle_converged": int(okr.sum()),
                               "both_converged": int(sel.sum()),
                               "cells_within_1e-6": int(np.all(err <= 1e-6, axis=1).sum()),
                               "species": {s: {"max": float(err[:, j].max(initial=0.0)),
                                               "median": float(np.median(err[:, j]))
                                               if len(err) else 0.0,
                                               "within_1e-6": int((err[:, j] <= 1e-6).sum())}
                                           for j, s in enumerate(OXYGEN_ORDER)}}
    return out


def sweep_latency_us(precision=DENGO_FP64, seed=20245):
    """Time of one Newton sweep of a lone stiff cell (one cell solved alone,
    the default engine): the floor per sweep of a cell's critical path."""
    import torch
    from .workloads import primordial_cells
    solver = Solver("primordial")
    stream = torch.cuda.current_stream()
    state, dtf = primordial_cells(64, "hot", seed=seed)
    best = None
    for c in range(16):
        ms, status, sweeps, _ = _device_step(torch, solver, state[c:c + 1], dtf[c:c + 1],
                                             precision, stream)
        if sweeps[0] >= 2000:
            us = ms * 1e3 / sweeps[0]
            best = us if best is None else min(best, us)
    return best


def config5(rate=50.0, duration=60.0, edge_range=(16, 128), budget_gb=40.0, slots=4,
            precision=DENGO_MIXED, admit_until=None, seed=5):
    import torch
    from .serving import ServingLoop, Request, _pool, _by_edge, poisson_requests
    torch.cuda.set_device(0)
    cfg = Solver.default_config()
    cfg.precision = precision
    reqs = poisson_requests(rate, duration, edge_range, seed=seed, primordial_config="config3")
    offered = sum(r.ncells for r in reqs)
    loop = ServingLoop(slots=slots, hbm_budget=int(budget_gb * (1 << 30)), config=cfg)
    loop.run([Request(n, _pool(n, 4096, 99)[:512], 1e9, rid=-1 - i)
              for i, n in enumerate(loop.networks)])
    served = loop.run(reqs, timeout=3600.0, admit_until=admit_until)
    done = [r for r in reqs if r.t_done is not None]
    served["by_edge"] = _by_edge(done)
    t_sweep = sweep_latency_us(precision)
    floors = np.array([int(r.sweeps.max()) * t_sweep / 1e3 for r in done
                       if r.sweeps is not None and len(r.sweeps)])
    batch_reqs = [Request(r.network, r.state, r.dtf, r.steps, 0.0, r.rid) for r in done]
    loop2 = ServingLoop(slots=slots, hbm_budget=int(budget_gb * (1 << 30)), config=cfg)
    batch = loop2.run(batch_reqs, timeout=3600.0)
    same = all(np.array_equal(a.result.view(np.int64), b.result.view(np.int64))
               for a, b in zip(done, batch_reqs))
    q = (lambda p: float(np.percentile(floors, p))) if len(floors) else (lambda p: None)
    return {"workload": {"rate_per_s": rate, "duration_s": duration, "edge_range": edge_range,
                         "mix": "primordial (config-3 cells) 0.7 / oxygen 0.3",
                         "dt_range_s": (1e8, 1e12), "hbm_budget_gb": budget_gb, "slots": slots,
                         "precision": "mixed" if precision == DENGO_MIXED else "fp64",
                         "admit_until_s": admit_until},
            "offered_cells": int(offered),
            "offered_cells_per_s": offered / duration,
            "served": served, "batch_of_served": batch,
            "served_over_batch_throughput": (served["cells_per_s"] / batch["cells_per_s"])
            if served.get("cells_per_s") and batch.get("cells_per_s") else None,
            "results_identical_served_vs_batch": same,
            "sweep_latency_us_lone_cell": t_sweep,
            "critical_path_floor_ms": {"p50": q(50), "p99": q(99), "max": q(100),
                                       "requests_under_20ms": int((floors < 20).sum()),
                                       "requests": int(len(floors))}}


def tail(per_sm=(1, 2, 3, 6), budget=50, kind="hot", cell=0, seed=20245, split=True,
         precision=DENGO_FP64):
    """Microseconds per Newton sweep of k copies per SM of one stiff cell
    resumed after ``budget`` sweeps: split engine vs wide engine."""
    import torch
    from .workloads import primordial_cells
    torch.cuda.set_device(0)
    solver = Solver("primordial")
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    state, dtf = primordial_cells(64, kind, seed=seed)
    rows = []
    for k in per_sm:
        n = nsm * k
        st = np.repeat(state[cell:cell + 1], n, axis=0)
        d = np.repeat(np.asarray(dtf)[cell:cell + 1], n)
        for wide in ((0, k) if split else (k,)):
            cfg = Solver.default_config()
            cfg.sweep_budget, cfg.wide_tail, cfg.precision = budget, wide, precision
            r = solver.solve_host(st, d, config=cfg, counters=True)
            sw = int(r["sweeps"].max())
            rows.append({"cells": n, "per_sm": k, "engine": "wide" if wide else "split",
                         "sweeps": sw, "ms": r["solve_ms"],
                         "us_per_sweep": r["solve_ms"] * 1e3 / max(sw - budget, 1)})
    return {"cell": {"kind": kind, "seed": seed, "index": cell}, "budget": budget,
            "precision": "mixed" if precision == DENGO_MIXED else "fp64", "sms": nsm,
            "rows": rows}


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="what", required=True)
    a4 = sub.add_parser("config4")
    a4.add_argument("--cells", type=int, default=1 << 20)
    a4.add_argument("--sample", type=int, default=256)
    a5 = sub.add_parser("config5")
    a5.add_argument("--rate", type=float, default=50.0)
    a5.add_argument("--duration", type=float, default=60.0)
    a5.add_argument("--edge-min", type=int, default=16)
    a5.add_argument("--edge-max", type=int, default=128)
    a5.add_argument("--budget-gb", type=float, default=40.0)
    a5.add_argument("--slots", type=int, default=4)
    a5.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    a5.add_argument("--admit-until", type=float, default=None,
                    help="stop admitting requests after this many seconds (the rest is "
                         "reported as backlog)")
    at = sub.add_parser("tail")
    at.add_argument("--per-sm", type=int, nargs="+", default=[1, 2, 3, 6])
    at.add_argument("--budget", type=int, default=50)
    at.add_argument("--kind", default="hot")
    at.add_argument("--cell", type=int, default=0)
    at.add_argument("--wide-only", action="store_true")
    at.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    a = ap.parse_args(argv)
    t0 = time.perf_counter()
    if a.what == "config4":
        out = config4(a.cells, a.sample)
    elif a.what == "tail":
        out = tail(a.per_sm, a.budget, a.kind, a.cell, split=not a.wide_only,
                   precision=DENGO_MIXED if a.precision == "mixed" else DENGO_FP64)
    else:
        out = config5(a.rate, a.duration, (a.edge_min, a.edge_max), a.budget_gb, a.slots,
                      DENGO_MIXED if a.precision == "mixed" else DENGO_FP64, a.admit_until)
    out["wall_s"] = time.perf_counter() - t0
    print(json.dumps(out))


if __name__ == "__main__":
    main()
