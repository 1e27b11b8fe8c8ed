"""dengo_evolve_<n> with the reference's lockstep strips (the default evolve
mode): the reference's dengo_evolve (rates_and_rate_tables.C.template:149-274)
runs a strip of cells with one dt and one Newton loop, and, when the network
was generated with write_intermediate_solutions, writes
<n>_intermediate_%06d after every accepted substep (C.template:212-241).

Pinned against the reference itself: ``lock_*`` of primordial_golden.npz
(its dengo_evolve over an 8-cell strip) and primordial_intermediate_golden.npz
(the intermediate files of the same call, written by the reference rendered
with write_intermediate_solutions; tests/golden/make_golden.py).  The kernel's
own source compiled for the host (tests/host_engine.py) is checked on the
CPU; the GPU tests call the library through the C ABI.
"""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def inter():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "primordial_intermediate_golden.npz")))


@pytest.fixture(scope="module")
def strip_so(tmp_path_factory):
    import host_engine as he
    return he.compile_engine("primordial", tmp_path_factory.mktemp("lock"), engine="strip")


def _bits(a, b):
    a, b = np.ascontiguousarray(a, np.float64), np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


def _dumps_equal(got, g):
    assert np.array_equal(np.asarray(got["siter"]), g["siter"])
    assert _bits(got["species"], g["species"])
    assert _bits(got["T"], g["T"])
    assert _bits(got["time"], g["time"]) and _bits(got["timestep"], g["timestep"])


def test_oracle_intermediate_dumps_match_reference(inter, tables_in_order, oracle):
    from oracle import evolve_strip
    r = evolve_strip(oracle, tables_in_order, inter["inp"], float(inter["dtf"]),
                     intermediate=True)
    d = r["intermediate"]
    got = dict(siter=[x["siter"] for x in d], species=np.array([x["species"] for x in d]),
               T=np.array([x["T"] for x in d]), time=np.array([x["time"] for x in d]),
               timestep=np.array([x["timestep"] for x in d]))
    _dumps_equal(got, inter)
    assert _bits(r["state"], inter["state"]) and _bits(r["atol"], inter["atol"])


def test_lockstep_kernel_on_host_matches_reference(golden, tables_in_order, strip_so):
    import host_engine as he
    r = he.lockstep_in_subprocess(strip_so, tables_in_order, golden["lock_in"],
                                  float(golden["lock_dtf"]))
    assert _bits(r["state"], golden["lock_state"]) and _bits(r["atol"], golden["lock_atol"])
    assert r["ttot"] == golden["lock_ttot"] and r["dt"] == golden["lock_dt"]


def test_lockstep_kernel_on_host_intermediate_dumps_match_reference(inter, tables_in_order,
                                                                     strip_so):
    import host_engine as he
    r = he.lockstep_in_subprocess(strip_so, tables_in_order, inter["inp"], float(inter["dtf"]),
                                  dump=True)
    _dumps_equal(r, inter)
    assert _bits(r["state"], inter["state"]) and _bits(r["atol"], inter["atol"])
    assert r["ttot"] == inter["ttot"] and r["dt"] == inter["dt"]


@pytest.fixture(scope="module")
def crlog_oracle():
    from oracle import Oracle
    return Oracle("primordial", crlog=True)


@pytest.mark.parametrize("seed", [3, 4])
def test_lockstep_kernel_on_host_matches_oracle(tables_in_order, crlog_oracle, strip_so, seed):
    """Neutral-gas strips of 40 cells (the strip converges in a few hundred
    substeps): the kernel equals the oracle's lockstep dengo_evolve built with
    a correctly rounded log T, as the device's is.  (Against the oracle on
    glibc's log these strips differ: in lockstep one of glibc's occasional
    mis-rounded logs anywhere in the strip changes the whole strip's
    trajectory; the reference's own 8-cell strip above has none.)"""
    import host_engine as he
    from oracle import evolve_strip
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(40, "cold", seed=seed)
    d = float(np.median(dtf))
    r = he.lockstep_in_subprocess(strip_so, tables_in_order, st, d)
    ref = evolve_strip(crlog_oracle, tables_in_order, st, d)
    assert _bits(r["state"], ref["state"]) and _bits(r["atol"], ref["atol"])
    assert r["ttot"] == ref["ttot"] and r["dt"] == ref["dt"]


@pytest.mark.gpu
def test_gpu_lockstep_evolve_matches_reference(solver, golden):
    """The default dengo_evolve_primordial on the reference's 8-cell strip."""
    st, at, ttot, dt = solver.evolve(golden["lock_in"], float(golden["lock_dtf"]))
    assert _bits(st, golden["lock_state"]) and _bits(at, golden["lock_atol"])
    assert ttot == golden["lock_ttot"] and dt == golden["lock_dt"]


@pytest.mark.gpu
def test_gpu_intermediate_files_match_reference(solver, inter, tmp_path, monkeypatch):
    """write_intermediate = 1: primordial_intermediate_%06d.dgt in the current
    directory after every accepted substep, each holding what the reference's
    .h5 file holds."""
    from dengo_gb300.runtime import Solver
    from dengo_gb300.tablefile import read_table_file
    monkeypatch.chdir(tmp_path)
    cfg = Solver.default_config()
    cfg.write_intermediate = 1
    solver.set_config(cfg)
    try:
        st, at, ttot, dt = solver.evolve(inter["inp"], float(inter["dtf"]))
    finally:
        solver.set_config(None)
    assert _bits(st, inter["state"]) and ttot == inter["ttot"] and dt == inter["dt"]
    files = sorted(p for p in os.listdir(tmp_path) if p.startswith("primordial_intermediate_"))
    assert files == ["primordial_intermediate_%06d.dgt" % k for k in inter["siter"]]
    got = dict(siter=inter["siter"], species=[], T=[], time=[], timestep=[])
    for f in files:
        t = read_table_file(str(tmp_path / f))
        got["species"].append(np.stack([t[s] for s in solver.species], axis=1))
        got["T"].append(t["T"])
        got["time"].append(t["time"][0])
        got["timestep"].append(t["timestep"][0])
    _dumps_equal({k: np.array(v) for k, v in got.items()}, inter)


@pytest.mark.gpu
def test_gpu_lockstep_two_strips_match_oracle(solver, crlog_oracle):
    """1064 cells: strips of 1024 and 40 cells, each the reference's lockstep
    call on its own (the oracle with a correctly rounded log T); the result
    is the smaller ttot and dt.  The cells are nearly neutral (ions and H-
    at 1e-14 of their element): the reference's electron consistency keeps a
    running total across the strip (rates_and_rate_tables.C.template:612-628),
    so in a long strip of ionised cells the later cells receive many times
    their own electrons and the strip thrashes to the substep cap, where no
    two implementations agree bit for bit.  Each cell within 1e-10 (glibc's
    pow(x, 3) in the oracle can differ from the device's correctly rounded
    cube by an ulp)."""
    from oracle import evolve_strip
    from dengo_gb300.workloads import primordial_cells
    st, dtf = primordial_cells(1064, "cold", seed=17)
    st = st.copy()
    for j in (1, 3, 4, 6, 7):         # H2+, H+, H-, He+, He++
        st[:, j] *= 1e-10
    d = float(np.median(dtf))
    got, at, ttot, dt = solver.evolve(st, d)
    refs = [evolve_strip(crlog_oracle, solver._tables, st[a:b], d)
            for a, b in ((0, 1024), (1024, 1064))]
    assert all(r["ttot"] == d for r in refs)
    want = np.concatenate([r["state"] for r in refs])
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-300)
    assert rel.max() <= 1e-10, rel.max()
    assert np.mean(np.all(got == want, axis=1)) >= 0.9
    assert ttot == min(r["ttot"] for r in refs)
    assert dt == min(r["dt"] for r in refs)


@pytest.mark.gpu
def test_gpu_intermediate_files_need_one_strip(solver):
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import primordial_cells
    cfg = Solver.default_config()
    cfg.write_intermediate = 1
    solver.set_config(cfg)
    try:
        st, dtf = primordial_cells(1100, "cold", seed=2)
        with pytest.raises(RuntimeError, match="one strip"):
            solver.evolve(st, float(dtf[0]))
    finally:
        solver.set_config(None)
