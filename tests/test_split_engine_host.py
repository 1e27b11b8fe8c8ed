"""The split CUDA engine (dg_split.cuh: 32 cells per CTA, each cell's sweep
shared by 4 warps -- the default engine) compiled for the host, its 128
lanes run as threads that meet at barriers (tests/host_engine.py), against
the single-lane engine compiled the same way: the two must agree bit for bit,
as they do on the GPU.  This covers the split engine's FP64 and mixed paths,
its suspension and resumption under a sweep budget, and the mixed path's
FP64 fallback for refinements that stop short (the shipped build), against
the lenient build that keeps them.  Each solve runs in a child process with
a time limit."""
import json
import os

import numpy as np
import pytest

import host_engine as he

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tables():
    from dengo_gb300.build import network_dir
    from dengo_gb300.tablefile import read_table_file
    with open(os.path.join(ROOT, "tests", "golden", "primordial_expressions.json")) as f:
        order = json.load(f)["tables"]
    t = read_table_file(os.path.join(network_dir("primordial"), "primordial_tables.dgt"))
    return [np.ascontiguousarray(t[k]) for k in order]


@pytest.fixture(scope="module")
def libs(tmp_path_factory):
    d = tmp_path_factory.mktemp("split_engine")
    return {"split": he.compile_engine("primordial", d, engine="split"),
            "split_lenient": he.compile_engine("primordial", d, strict=False, engine="split"),
            "lane": he.build("primordial", d),
            "lane_lenient": he.build("primordial", d, strict=False)}


def _same(a, b):
    for k in ("state", "atol", "dt", "ttot"):
        assert np.array_equal(a[k].view(np.int64), b[k].view(np.int64)), k
    for k in ("status", "substeps", "sweeps", "failures"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("mixed", [0, 1, 2])
def test_split_equals_lane(libs, tables, mixed):
    """32 cold cells (a few hundred sweeps each), one launch and with a
    sweep budget of 100 (cells set aside and resumed twice); FP64, mixed,
    and mixed with the Newton matrix in extended-range FP32 (2)."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(32, "cold", seed=11)
    lane = he.evolve(libs["lane"], tables, st, dtf, mixed=mixed)
    split = he.evolve_in_subprocess(libs["split"], tables, st, dtf, timeout=600, mixed=mixed)
    _same(split, lane)
    budget = he.evolve_in_subprocess(libs["split"], tables, st, dtf, timeout=600, mixed=mixed,
                                     sweep_budget=100)
    assert budget["resumed"] > 0
    _same(budget, lane)


@pytest.mark.parametrize("build", ["", "_lenient"])
def test_split_fallback_equals_lane_fallback(libs, tables, build):
    """Three config-3 cells whose mixed refinement sometimes stops short of
    2^-40: the split engine hands those systems to the FP64 elimination
    exactly as the single-lane engine does (shipped build), or keeps them
    exactly as it does (lenient build); the two builds end differently."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(256, "config3", seed=78)
    pick = [8, 174, 218]
    st, dtf = st[pick], dtf[pick]
    lane = he.evolve(libs["lane" + build], tables, st, dtf, mixed=True)
    split = he.evolve_in_subprocess(libs["split" + build], tables, st, dtf, timeout=900,
                                    mixed=True)
    _same(split, lane)
    other = he.evolve(libs["lane_lenient" if not build else "lane"], tables, st, dtf, mixed=True)
    assert not np.array_equal(other["state"].view(np.int64), lane["state"].view(np.int64))
