"""The wide engine (dg_wide.cuh: one cell per CTA of 4 warps, the engine for
the last few set-aside cells of a solve) compiled for the host with its 128
lanes as threads (tests/host_engine.py), against the split engine compiled
the same way: a solve whose resume launches all run on the wide engine must
equal, bit for bit, the same solve on the split engine alone -- and hence
the single-lane engine and, on the FP64 path, the reference.  FP64 and mixed
precision (its FP64 fallbacks and conservation re-solves included).  Each
solve runs in a child process with a time limit."""
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
            "wide": he.compile_engine("primordial", d, engine="wide"),
            "split_lenient": he.compile_engine("primordial", d, strict=False, engine="split"),
            "wide_lenient": he.compile_engine("primordial", d, strict=False, engine="wide")}


def _same(a, b):
    for k in ("state", "atol", "dt", "ttot"):
        assert np.array_equal(a[k].view(np.int64), b[k].view(np.int64)), k
    for k in ("status", "substeps", "sweeps", "failures"):
        assert np.array_equal(a[k], b[k]), k


# (workload, cells, seed, picked cells, sweep budget); the picked config3
# and top cells take 400-2200 sweeps with 4-35 rejected substeps each
CASES = [("cold", 24, 23, [0, 2, 5, 9, 13, 17], 60),
         ("config3", 64, 23, [4, 11, 41], 40),
         ("top", 64, 23, [11, 14, 47], 40)]


@pytest.mark.parametrize("mixed", [0, 1])
@pytest.mark.parametrize("kind,n,seed,pick,budget", CASES, ids=[c[0] for c in CASES])
def test_wide_resume_equals_split(libs, tables, kind, n, seed, pick, budget, mixed):
    """Cells set aside after a small sweep budget and resumed twice (at 16x
    the budget, then to the end): the wide engine's resumed cells equal the
    split engine's, FP64 and mixed precision."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(n, kind, seed=seed)
    if pick is not None:
        st, dtf = st[pick], np.broadcast_to(np.asarray(dtf, np.float64), (n,))[pick]
    split = he.evolve_in_subprocess(libs["split"], tables, st, dtf, timeout=900,
                                    sweep_budget=budget, mixed=mixed)
    wide = he.evolve_in_subprocess(libs["wide"], tables, st, dtf, timeout=900,
                                   sweep_budget=budget, mixed=mixed)
    assert wide["resumed"] > 0 and wide["resumed"] == split["resumed"]
    _same(wide, split)


@pytest.mark.parametrize("build", ["", "_lenient"])
def test_wide_mixed_fallback_equals_split(libs, tables, build):
    """Three config-3 cells whose mixed refinement sometimes stops short of
    2^-40, resumed on the wide engine: it hands those systems to the FP64
    elimination (shipped build) or keeps them (lenient build) exactly as the
    split engine does."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(256, "config3", seed=78)
    pick = [8, 174, 218]
    st, dtf = st[pick], np.asarray(dtf)[pick]
    split = he.evolve_in_subprocess(libs["split" + build], tables, st, dtf, timeout=900,
                                    mixed=True, sweep_budget=30)
    wide = he.evolve_in_subprocess(libs["wide" + build], tables, st, dtf, timeout=900,
                                   mixed=True, sweep_budget=30)
    assert wide["resumed"] > 0
    _same(wide, split)


def test_wide_conservation_resolve_equals_split(libs, tables):
    """A conservation tolerance below zero fails every converged mixed cell,
    which is re-solved from its input with FP64 linear solves: set aside and
    resumed on the wide engine, both the first solve and the re-solve equal
    the split engine's."""
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(4, "cold", seed=41)
    split = he.evolve_in_subprocess(libs["split"], tables, st, dtf, timeout=900, mixed=True,
                                    sweep_budget=40, cons_tol=-1.0)
    wide = he.evolve_in_subprocess(libs["wide"], tables, st, dtf, timeout=900, mixed=True,
                                   sweep_budget=40, cons_tol=-1.0)
    assert wide["resumed"] > 0
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


@pytest.fixture(scope="module")
def oxygen_libs(tmp_path_factory):
    d = tmp_path_factory.mktemp("wide_oxygen")
    return (he.compile_engine("oxygen", d, engine="split"),
            he.compile_engine("oxygen", d, engine="wide"))


@pytest.mark.parametrize("mixed", [0, 1])
def test_wide_oxygen_equals_split(oxygen_libs, mixed):
    """The 16-equation ion network, every RHS row and Jacobian entry from the
    sum-of-products tables (no scalar parts): two of the golden input cells
    set aside after 20 sweeps and resumed on the wide engine equal the split
    engine's, FP64 and mixed."""
    from dengo_gb300.build import network_dir
    from dengo_gb300.tablefile import read_table_file
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "oxygen_golden.npz")))
    t = read_table_file(os.path.join(network_dir("oxygen"), "oxygen_tables.dgt"))
    tabs = [np.ascontiguousarray(t[k]) for k in g["table_order"]]
    split_so, wide_so = oxygen_libs
    st, dtf = g["evolve_in"][:2], np.asarray(g["evolve_dtf"])[:2]
    split = he.evolve_in_subprocess(split_so, tabs, st, dtf, timeout=900, sweep_budget=20,
                                    mixed=mixed)
    wide = he.evolve_in_subprocess(wide_so, tabs, st, dtf, timeout=900, sweep_budget=20,
                                   mixed=mixed)
    assert wide["resumed"] > 0 and wide["resumed"] == split["resumed"]
    _same(wide, split)


def test_wide_compton_equals_split(tmp_path_factory):
    """The primordial network with Compton cooling, whose ge row reads the
    cell's temperature and the call's redshift directly (scalar parts):
    four cold cells at the golden set's highest redshift, set aside after 20
    sweeps and resumed on the wide engine, equal the split engine's."""
    from dengo_gb300.workloads import primordial_cells
    from dengo_gb300.build import network_dir
    from dengo_gb300.tablefile import read_table_file
    name = "primordial_compton"
    g = dict(np.load(os.path.join(ROOT, "tests", "golden", name + "_golden.npz")))
    t = read_table_file(os.path.join(network_dir(name), name + "_tables.dgt"))
    tabs = [np.ascontiguousarray(t[k]) for k in g["table_order"]]
    d = tmp_path_factory.mktemp("wide_compton")
    split_so = he.compile_engine(name, d, engine="split")
    wide_so = he.compile_engine(name, d, engine="wide")
    z = max(float(x) for x in g["redshifts"])
    st, dtf = primordial_cells(4, "cold", seed=29)
    split = he.evolve_in_subprocess(split_so, tabs, st, dtf, timeout=900, sweep_budget=20, z=z)
    wide = he.evolve_in_subprocess(wide_so, tabs, st, dtf, timeout=900, sweep_budget=20, z=z)
    assert wide["resumed"] > 0 and wide["resumed"] == split["resumed"]
    _same(wide, split)
