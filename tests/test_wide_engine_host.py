"""The wide engine (dg_wide.cuh: one cell per CTA of 4 warps, the FP64
path's engine for the last few set-aside cells of a solve) compiled for the
host with its 128 lanes as threads (tests/host_engine.py), against the split
engine compiled the same way: a solve whose resume launches all run on the
wide engine must equal, bit for bit, the same solve on the split engine
alone -- and hence the single-lane engine and the reference.  Each solve
runs in a child process with a time limit."""
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
    d = tmp_path_factory.mktemp("wide_engine")
    return {"split": he.compile_engine("primordial", d, engine="split"),
            "wide": he.compile_engine("primordial", d, engine="wide")}


def _same(a, b):
    for k in ("state", "atol", "dt", "ttot"):
        assert np.array_equal(a[k].view(np.int64), b[k].view(np.int64)), k
    for k in ("status", "substeps", "sweeps", "failures"):
        assert np.array_equal(a[k], b[k]), k


# (workload, cells, seed, picked cells, sweep budget); the picked config3
# and top cells take 400-2200 sweeps with 4-35 rejected substeps each
CASES = [("cold", 24, 23, None, 60),
         ("config3", 64, 23, [4, 11, 15, 41, 43, 48], 40),
         ("top", 64, 23, [11, 14, 47], 40)]


@pytest.mark.parametrize("kind,n,seed,pick,budget", CASES, ids=[c[0] for c in CASES])
def test_wide_resume_equals_split(libs, tables, kind, n, seed, pick, budget):
    """Cells set aside after a small sweep budget and resumed twice (at 16x
    the budget, then to the end): the wide engine's resumed cells equal the
    split engine's."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(n, kind, seed=seed)
    if pick is not None:
        st, dtf = st[pick], np.broadcast_to(np.asarray(dtf, np.float64), (n,))[pick]
    split = he.evolve_in_subprocess(libs["split"], tables, st, dtf, timeout=900,
                                    sweep_budget=budget)
    wide = he.evolve_in_subprocess(libs["wide"], tables, st, dtf, timeout=900,
                                   sweep_budget=budget)
    assert wide["resumed"] > 0 and wide["resumed"] == split["resumed"]
    _same(wide, split)


def test_wide_resume_nonfinite_scale(libs, tables):
    """A cell with a species at exactly 0 (its scale is 0, so the Newton
    matrix is built as the reference builds it with infinite inverse scales)
    next to ordinary cells, set aside and resumed on the wide engine."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(8, "cold", seed=5)
    st = st.copy()
    st[3, 1] = 0.0
    split = he.evolve_in_subprocess(libs["split"], tables, st, dtf, timeout=900,
                                    sweep_budget=20)
    wide = he.evolve_in_subprocess(libs["wide"], tables, st, dtf, timeout=900,
                                   sweep_budget=20)
    # the zero-scale cell fails every substep (34 sweeps to the dt floor):
    # it is set aside after 20 and ends on the wide engine
    assert split["sweeps"][3] > 20 and split["status"][3] == 2
    assert wide["resumed"] == split["resumed"]
    _same(wide, split)
