"""Serving loop: continuous batching of cell-patch requests on one GPU.

A request is one patch of cells of one network (mass densities + ge, the
reference's ``dengo_evolve_<n>`` input layout) with a hydro-step length
``dtf`` and a number of hydro steps to run with the patch's state resident
on the device.  The loop

* admits pending requests in arrival order while the device-memory budget
  (bytes of state, tolerances, per-cell dtf/status/counters) and a free slot
  allow;
* batches the admitted requests of one network into one launch group: their
  cells are copied into one device buffer and solved by one persistent
  work-queue launch per hydro step (``<n>_solve_cells_device``);
* runs each group on its own slot -- a CUDA stream with its own solver
  contexts -- so groups admitted while others are on the GPU overlap with
  them on the device;
* retires a group when its last step's event has completed, copies each
  request's cells back and returns the memory to the budget.

Every cell is solved independently of the cells beside it, so a request's
result is the same alone and in any mix (bit-identical for the FP64 path).
Latency is measured from a request's arrival to the completion of its copy
back; ``run`` reports p50/p99/p99.9 and the throughput in cells/s.
"""

import collections
import time
from dataclasses import dataclass, field

import numpy as np

from .runtime import DENGO_OK, Solver


@dataclass(eq=False)       # requests compare by identity
class Request:
    network: str
    state: np.ndarray          # (cells, N) float64, AoS
    dtf: float                 # seconds per hydro step
    steps: int = 1             # hydro steps solved with the state on the device
    arrival: float = 0.0       # seconds on the loop's clock
    rid: int = -1
    # filled in by the loop
    result: np.ndarray = None
    status: np.ndarray = None
    sweeps: np.ndarray = None      # Newton sweeps of each cell in its last step
    t_admit: float = None
    t_done: float = None

    @property
    def ncells(self):
        return int(self.state.shape[0])

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def request_bytes(req):
    """Device bytes a request holds while admitted: state and atol (N
    doubles each per cell), dtf (double), status and sweep count (ints)."""
    n, nsp = req.state.shape
    return n * (2 * nsp * 8 + 8 + 4 + 4)


def select_group(pending, used, budget, max_group_cells):
    """The next launch group: the oldest pending request (nothing while it
    does not fit the budget, so it is never overtaken indefinitely), then the
    pending requests behind it with its network and step count, in arrival
    order, while the group's cells and everyone's bytes fit."""
    if not pending:
        return []
    head = pending[0]
    nbytes = request_bytes(head)
    if used + nbytes > budget:
        return []
    take, cells = [head], head.ncells
    for r in list(pending)[1:]:
        if r.network != head.network or r.steps != head.steps:
            continue
        b = request_bytes(r)
        if cells + r.ncells > max_group_cells or used + nbytes + b > budget:
            continue
        take.append(r)
        cells += r.ncells
        nbytes += b
    return take


@dataclass
class _Group:
    network: str
    requests: list
    offsets: list
    ncells: int
    nbytes: int
    steps: int
    event: object = None
    tensors: dict = field(default_factory=dict)


class _Slot:
    """A CUDA stream and one solver context per network (contexts hold the
    work-queue counter, so concurrent launches need their own)."""

    def __init__(self, torch, device, networks, config):
        self.stream = torch.cuda.Stream(device=device)
        self.solvers = {n: Solver(n) for n in networks}
        self.config = config
        self.group = None


class ServingLoop:
    """Continuous-batching request loop over the GPU solvers.

    networks        networks served (one solver library each)
    slots           launch groups that may be on the device at once
    hbm_budget      bytes of request state the loop may hold on the device
    max_group_cells cells per launch group
    config          dengo_solver_config for every launch (default: the
                    split engine, 4 warps per cell, FP64, stiff cells
                    redistributed after 2000 sweeps)"""

    def __init__(self, networks=("primordial", "oxygen"), slots=4, hbm_budget=40 << 30,
                 max_group_cells=1 << 20, config=None, device=0):
        import torch
        self.torch = torch
        self.device = torch.device("cuda", device)
        if config is None:
            config = Solver.default_config()
            config.warps_per_cell = 4
            config.sweep_budget = 2000
        self.slots = [_Slot(torch, self.device, networks, config) for _ in range(slots)]
        self.networks = tuple(networks)
        self.budget = int(hbm_budget)
        self.used = 0
        self.max_group_cells = int(max_group_cells)
        self.pending = collections.deque()
        self.done = []
        self.t0 = time.perf_counter()
        self.launches = 0

    # -- clock ---------------------------------------------------------------
    def now(self):
        return time.perf_counter() - self.t0

    # -- submission ----------------------------------------------------------
    def submit(self, req):
        if req.network not in self.networks:
            raise KeyError("network %r is not served" % req.network)
        if request_bytes(req) > self.budget:
            raise ValueError("request %d needs %d bytes, above the whole budget of %d"
                             % (req.rid, request_bytes(req), self.budget))
        if req.ncells > self.max_group_cells:
            raise ValueError("request %d has %d cells, above max_group_cells = %d"
                             % (req.rid, req.ncells, self.max_group_cells))
        self.pending.append(req)

    # -- admission and launch ------------------------------------------------
    def _form_group(self):
        take = select_group(self.pending, self.used, self.budget, self.max_group_cells)
        if not take:
            return None
        for r in take:
            self.pending.remove(r)
        offs = np.cumsum([0] + [r.ncells for r in take]).tolist()
        return _Group(take[0].network, take, offs, offs[-1], sum(request_bytes(r) for r in take),
                      take[0].steps)

    def _launch(self, slot, g):
        torch = self.torch
        t = self.now()
        for r in g.requests:
            r.t_admit = t
        nsp = g.requests[0].state.shape[1]
        host = np.concatenate([r.state for r in g.requests]).astype(np.float64, copy=False)
        dtf = np.concatenate([np.full(r.ncells, r.dtf) for r in g.requests])
        with torch.cuda.stream(slot.stream):
            h_state = torch.from_numpy(host).pin_memory()
            h_dtf = torch.from_numpy(dtf).pin_memory()
            st = h_state.to(self.device, non_blocking=True)
            d_dtf = h_dtf.to(self.device, non_blocking=True)
            at = torch.empty_like(st)
            status = torch.empty(g.ncells, dtype=torch.int32, device=self.device)
            sweeps = torch.empty(g.ncells, dtype=torch.int32, device=self.device)
            solver = slot.solvers[g.network]
            for _ in range(g.steps):
                torch.mul(st, 1e-6, out=at)
                solver.solve_device(st, g.ncells, nsp, 1, at, rtol_scalar=1e-6, dtf=d_dtf,
                                    status=status, sweeps=sweeps, config=slot.config,
                                    stream=slot.stream)
                self.launches += 1
            out = torch.empty(host.shape, dtype=torch.float64, pin_memory=True)
            out.copy_(st, non_blocking=True)
            out_status = torch.empty(g.ncells, dtype=torch.int32, pin_memory=True)
            out_status.copy_(status, non_blocking=True)
            out_sweeps = torch.empty(g.ncells, dtype=torch.int32, pin_memory=True)
            out_sweeps.copy_(sweeps, non_blocking=True)
            g.event = torch.cuda.Event()
            g.event.record(slot.stream)
        g.tensors = dict(st=st, at=at, status=status, sweeps=sweeps, dtf=d_dtf, h_state=h_state,
                         h_dtf=h_dtf, out=out, out_status=out_status, out_sweeps=out_sweeps)
        self.used += g.nbytes
        slot.group = g

    def _retire(self, slot):
        g = slot.group
        t = self.now()
        out = g.tensors["out"].numpy()
        ost = g.tensors["out_status"].numpy()
        osw = g.tensors["out_sweeps"].numpy()
        for r, a, b in zip(g.requests, g.offsets[:-1], g.offsets[1:]):
            r.result = out[a:b].copy()
            r.status = ost[a:b].copy()
            r.sweeps = osw[a:b].copy()
            r.t_done = t
            self.done.append(r)
        self.used -= g.nbytes
        slot.group = None

    def poll(self):
        """Retire finished groups, then admit pending requests into free
        slots.  Returns the number of groups retired."""
        retired = 0
        for s in self.slots:
            if s.group is not None and s.group.event.query():
                self._retire(s)
                retired += 1
        for s in self.slots:
            if not self.pending:
                break
            if s.group is None:
                g = self._form_group()
                if g is None:
                    break
                self._launch(s, g)
        return retired

    def busy(self):
        return bool(self.pending) or any(s.group is not None for s in self.slots)

    def drain(self, timeout=600.0):
        t_end = time.perf_counter() + timeout
        while self.busy():
            if time.perf_counter() > t_end:
                raise TimeoutError("serving loop did not drain in %.0f s" % timeout)
            if not self.poll():
                time.sleep(2e-4)

    # -- a timed run over an arrival schedule --------------------------------
    def run(self, requests, timeout=600.0, admit_until=None):
        """Submit each request at its ``arrival`` time (seconds from now) and
        serve until all are done.  With ``admit_until`` (seconds) no request
        is admitted after that time: requests still pending then are left
        unserved (the backlog), groups already on the device finish.
        Returns the latency/throughput summary of the served requests."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        self.t0 = time.perf_counter()
        i = 0
        t_end = self.t0 + timeout
        while i < len(reqs) or self.busy():
            now = self.now()
            if admit_until is not None and now > admit_until:
                self.pending.clear()
                i = len(reqs)
                if not any(s.group is not None for s in self.slots):
                    break
            while i < len(reqs) and reqs[i].arrival <= now:
                self.submit(reqs[i])
                i += 1
            if not self.poll():
                time.sleep(1e-4)
            if time.perf_counter() > t_end:
                raise TimeoutError("serving run did not finish in %.0f s" % timeout)
        out = summarize([r for r in reqs if r.t_done is not None])
        out["offered_requests"] = len(reqs)
        out["backlog_requests"] = sum(1 for r in reqs if r.t_done is None)
        out["backlog_cells"] = int(sum(r.ncells for r in reqs if r.t_done is None))
        return out


def summarize(reqs):
    lat = np.array([r.latency for r in reqs if r.latency is not None])
    cells = sum(r.ncells for r in reqs)
    span = max(r.t_done for r in reqs) - min(r.arrival for r in reqs) if reqs else 0.0
    ok = sum(int(np.sum(r.status == DENGO_OK)) for r in reqs if r.status is not None)
    q = (lambda p: float(np.percentile(lat, p)) * 1e3) if len(lat) else (lambda p: None)
    return {"requests": len(reqs), "cells": int(cells), "converged_cells": int(ok),
            "span_s": float(span), "cells_per_s": cells / span if span > 0 else None,
            "latency_ms": {"p50": q(50), "p99": q(99), "p999": q(99.9),
                           "max": float(lat.max() * 1e3) if len(lat) else None}}


_POOLS = {}


def _pool(network, ncells, seed, primordial_config="config1"):
    """Seeded cell states of one network, generated once per process."""
    from .workloads import oxygen_cells, primordial_cells
    key = (network, ncells, seed, primordial_config)
    if key not in _POOLS:
        if network == "primordial":
            _POOLS[key] = primordial_cells(ncells, primordial_config, seed=seed)[0]
        else:
            _POOLS[key] = oxygen_cells(ncells, seed=seed)[0]
    return _POOLS[key]


def poisson_requests(rate, duration, edge_range=(16, 128), mix=(("primordial", 0.7),
                     ("oxygen", 0.3)), dt_range=(1e8, 1e12), seed=5, max_edge=None,
                     pool_cells=None, primordial_config="config1"):
    """The serving workload: Poisson arrivals at ``rate`` per second for
    ``duration`` seconds; cubic patches with edge ~ logU(edge_range) cells;
    networks drawn by ``mix``; dtf ~ logU(dt_range) s.  Patch contents are
    contiguous slices, at seeded offsets, of one seeded pool of cells per
    network (primordial cells of ``primordial_config``'s distributions;
    oxygen ion-by-ion cells)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    hi = min(edge_range[1], max_edge) if max_edge else edge_range[1]
    pool_cells = pool_cells or max(hi ** 3, 4096) * 2
    t, out = 0.0, []
    names = [m[0] for m in mix]
    p = np.array([m[1] for m in mix], float)
    p /= p.sum()
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        edge = int(round(np.exp(rng.uniform(np.log(edge_range[0]), np.log(edge_range[1])))))
        if max_edge:
            edge = min(edge, max_edge)
        n = edge ** 3
        net = names[rng.choice(len(names), p=p)]
        pool = _pool(net, pool_cells, seed + (0 if net == "primordial" else 1),
                     primordial_config)
        off = int(rng.integers(0, pool.shape[0] - n + 1))
        dtf = float(np.exp(rng.uniform(np.log(dt_range[0]), np.log(dt_range[1]))))
        out.append(Request(net, pool[off:off + n], dtf, arrival=t, rid=len(out)))
    return out


def _by_edge(reqs):
    """Latency percentiles per patch-edge band (16-32, 32-64, 64-128 cells)."""
    out = {}
    for lo, hi in ((16, 32), (32, 64), (56, 72), (64, 129)):
        lat = [r.latency for r in reqs if lo ** 3 <= r.ncells < hi ** 3 and r.latency is not None]
        if lat:
            out["%d-%d" % (lo, hi)] = {"n": len(lat), "p50_ms": float(np.percentile(lat, 50)) * 1e3,
                                       "p99_ms": float(np.percentile(lat, 99)) * 1e3}
    return out


def serve_benchmark(rate=50.0, duration=10.0, slots=4, budget_gb=40.0, edge_range=(16, 128),
                    dt_range=(1e8, 1e12), precision=0, seed=5, max_edge=None):
    """The serving workload under Poisson arrivals, then the same requests
    submitted at once (batch throughput); returns both summaries."""
    cfg = Solver.default_config()
    cfg.warps_per_cell, cfg.precision, cfg.sweep_budget = 4, precision, 2000
    reqs = poisson_requests(rate, duration, edge_range, dt_range=dt_range, seed=seed,
                            max_edge=max_edge)
    loop = ServingLoop(slots=slots, hbm_budget=int(budget_gb * (1 << 30)), config=cfg)
    # warm-up: one small request of each network
    loop.run([Request(n, _pool(n, 4096, 99)[:512], 1e9, rid=-1 - i)
              for i, n in enumerate(loop.networks)])
    served = loop.run(reqs)
    served["by_edge"] = _by_edge(reqs)
    served["launches"] = loop.launches
    batch_reqs = [Request(r.network, r.state, r.dtf, r.steps, 0.0, r.rid) for r in reqs]
    loop2 = ServingLoop(slots=slots, hbm_budget=int(budget_gb * (1 << 30)), config=cfg)
    batch = loop2.run(batch_reqs)
    same = all(np.array_equal(a.result.view(np.int64), b.result.view(np.int64))
               for a, b in zip(reqs, batch_reqs))
    ratio = (served["cells_per_s"] / batch["cells_per_s"]) if batch["cells_per_s"] else None
    return {"workload": {"rate_per_s": rate, "duration_s": duration, "edge_range": edge_range,
                         "mix": "primordial 0.7 / oxygen 0.3", "dt_range_s": dt_range,
                         "hbm_budget_gb": budget_gb, "slots": slots, "precision": precision,
                         "max_edge": max_edge},
            "served": served, "batch": batch, "served_over_batch_throughput": ratio,
            "results_identical_served_vs_batch": same}


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="serving loop under Poisson arrivals")
    ap.add_argument("--rate", type=float, default=50.0)
    ap.add_argument("--duration", type=float, default=10.0)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--budget-gb", type=float, default=40.0)
    ap.add_argument("--edge-min", type=int, default=16)
    ap.add_argument("--edge-max", type=int, default=128)
    ap.add_argument("--dt-min", type=float, default=1e8)
    ap.add_argument("--dt-max", type=float, default=1e12)
    ap.add_argument("--precision", type=int, default=0)
    a = ap.parse_args()
    print(json.dumps(serve_benchmark(a.rate, a.duration, a.slots, a.budget_gb,
                                     (a.edge_min, a.edge_max), (a.dt_min, a.dt_max),
                                     a.precision)))
