"""Autotuner and CUDA-graph capture of hydro steps (dengo_gb300/batching.py)."""
import numpy as np
import pytest

from dengo_gb300.batching import SCHEDULES, candidates, make_config


def test_candidates_cover_the_engine_variants():
    c = candidates()
    assert {x["warps_per_cell"] for x in c} == {1, 2, 4}
    assert {x["block"] for x in c if x["warps_per_cell"] == 1} == {32, 64, 128}
    assert {x["schedule"] for x in c} == {"queue", "stride"}
    assert len(c) == len({tuple(sorted(x.items())) for x in c})
    cfg = make_config(c[0], precision=1, max_substeps=77)
    assert cfg.precision == 1 and cfg.max_substeps == 77
    assert cfg.schedule == SCHEDULES[c[0]["schedule"]] and cfg.warps_per_cell == c[0]["warps_per_cell"]


@pytest.mark.gpu
def test_graph_replay_equals_eager_steps(solver):
    import torch
    from dengo_gb300.batching import StepGraph
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import primordial_cells
    state, dtf = primordial_cells(3000, "cold", seed=8)
    cfg = Solver.default_config()
    cfg.warps_per_cell = 4
    dev = torch.device("cuda")
    d_dtf = torch.tensor(dtf, device=dev)
    # both share the solver's context (its scratch), so they share a stream:
    # calls on one context must not overlap on the GPU
    stream = torch.cuda.Stream(device=dev)
    eager = StepGraph(solver, torch.tensor(state, device=dev), d_dtf, cfg, stream=stream)
    graph = StepGraph(solver, torch.tensor(state, device=dev), d_dtf, cfg,
                      stream=stream).capture()
    for _ in range(3):
        eager.eager()
        graph.replay()
    torch.cuda.synchronize()
    a, b = eager.state.cpu().numpy(), graph.state.cpu().numpy()
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    assert torch.equal(eager.status, graph.status) and torch.equal(eager.sweeps, graph.sweeps)
    assert not np.array_equal(a, state)


@pytest.mark.gpu
def test_autotune_picks_a_measured_candidate(solver, tmp_path, monkeypatch):
    from dengo_gb300.batching import autotune
    from dengo_gb300.workloads import primordial_cells
    monkeypatch.setenv("DENGO_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    state, dtf = primordial_cells(1024, "config3", seed=4)
    cands = [c for c in candidates() if c["schedule"] == "queue"]
    best, table = autotune(solver, state, dtf, sample=512, max_substeps=300, repeats=1, cands=cands)
    assert len(table) == len(cands) and all(r["ms"] > 0 for r in table)
    assert min(table, key=lambda r: r["ms"])["warps_per_cell"] == best["warps_per_cell"]
    # every variant did the same work (same sweeps: results do not depend on the variant)
    assert len({r["sweeps"] for r in table}) == 1
    again, _ = autotune(solver, state, dtf, sample=512, max_substeps=300, repeats=1, cands=cands)
    assert again == best and (tmp_path / "tune.json").exists()


@pytest.mark.gpu
def test_graph_replay_with_sweep_budget_equals_eager_steps(solver):
    """The redistributed solve (stiff-cell redistribution, three launches) captured in a graph
    gives the eager steps' bits."""
    import torch
    from dengo_gb300.batching import StepGraph
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import primordial_cells
    state, dtf = primordial_cells(2000, "config3", seed=18)
    cfg = Solver.default_config()
    cfg.warps_per_cell, cfg.sweep_budget, cfg.max_substeps = 4, 30, 2000
    dev = torch.device("cuda")
    d_dtf = torch.tensor(dtf, device=dev)
    # both share the solver's context (its scratch), so they share a stream:
    # calls on one context must not overlap on the GPU
    stream = torch.cuda.Stream(device=dev)
    eager = StepGraph(solver, torch.tensor(state, device=dev), d_dtf, cfg, stream=stream)
    graph = StepGraph(solver, torch.tensor(state, device=dev), d_dtf, cfg,
                      stream=stream).capture()
    for _ in range(2):
        eager.eager()
        graph.replay()
    torch.cuda.synchronize()
    a, b = eager.state.cpu().numpy(), graph.state.cpu().numpy()
    assert np.array_equal(a.view(np.int64), b.view(np.int64))
    assert torch.equal(eager.status, graph.status) and torch.equal(eager.sweeps, graph.sweeps)
