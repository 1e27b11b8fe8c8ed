"""The reference's Cython driver run_<n> (rates_and_rate_tables_run.pyx
.template:81-205) as a GPU driver mode (<n>_run_strip): one strip in
lockstep with the driver's own dt control, scale refresh, niter cap,
dt < 1e-30 tf stop and intermediate trajectories, against the oracle's
restatement of the same loop (oracle/be_oracle.c dgo_run_strip)."""
import numpy as np
import pytest

from dengo_gb300.workloads import PRIMORDIAL_ORDER, PRIMORDIAL_WEIGHTS, primordial_cells

W = np.array([PRIMORDIAL_WEIGHTS.get(s, 1.0) for s in PRIMORDIAL_ORDER])


def _ics(n, seed):
    """Initial conditions as the Cython driver takes them: number density x
    weight per species, ge in erg/g."""
    st, _ = primordial_cells(n, "config1", seed=seed)
    num = st / (W * 1.67e-24)
    num[:, -1] = st[:, -1]
    return {s: num[:, j] * W[j] for j, s in enumerate(PRIMORDIAL_ORDER)}


def test_oracle_run_strip_reaches_tf_or_stops(tables_in_order, oracle):
    from oracle import run_strip
    ics = _ics(16, 31)
    inp = np.stack([ics[s] / W[j] for j, s in enumerate(PRIMORDIAL_ORDER)], axis=1)
    r = run_strip(oracle, tables_in_order, inp, 1e8, 3000)
    assert r["ttot"] == 1e8 and r["iterations"] == r["substeps_ok"] + r["substeps_fail"]
    r = run_strip(oracle, tables_in_order, inp, 1e10, 3000)
    assert r["ttot"] < 1e10 and r["dt"] < 1e-30 * 1e10      # the dt floor ends the loop


@pytest.mark.parametrize("case", [0, 1, 2])
def test_oracle_run_strip_matches_reference_cython_driver(tables_in_order, oracle, case):
    """The oracle's loop against the reference's own Cython driver
    run_primordial (compiled from its rendered .pyx; goldens from
    tests/golden/make_golden.py run): final values, and per iteration the
    success flags, times, steps, temperatures and energies, bit for bit."""
    import os
    import platform
    from oracle import run_strip
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "primordial_run_golden.npz"))
    tf, niter = g["cases"][case]
    niter = int(niter)
    inp = g["ics"] / W
    r = run_strip(oracle, tables_in_order, inp, tf, niter, trajectories=True)
    tr = r["trajectories"]
    ige = PRIMORDIAL_ORDER.index("ge")
    got = dict(rv=r["state"] * W, successful=tr["successful"], t=tr["t"], dt=tr["dt"],
               T=tr["traj_T"].T, ge=tr["traj"][:, :, ige].T)
    for key, a in got.items():
        b = g["run%d_%s" % (case, key)]
        assert a.shape == b.shape, key
        if platform.machine() == "x86_64" or key in ("successful",):
            a = np.ascontiguousarray(a, b.dtype)
            assert np.array_equal(a.view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), key
        else:
            assert np.allclose(a, b, rtol=1e-12, atol=0), key
    assert r["iterations"] == int(np.count_nonzero(g["run%d_dt" % case]))


@pytest.mark.gpu
@pytest.mark.parametrize("tf,niter", [(1e8, 3000), (1e10, 3000), (1e9, 40)])
def test_gpu_run_strip_matches_oracle(solver, oracle, tables_in_order, tf, niter):
    from oracle import run_strip
    ics = _ics(16, 31)
    rv, rv_t = solver.run(ics, tf, niter=niter, intermediate=1)
    inp = np.stack([ics[s] / W[j] for j, s in enumerate(PRIMORDIAL_ORDER)], axis=1)
    ref = run_strip(oracle, tables_in_order, inp, tf, niter)
    last = solver.last_run
    assert last["iterations"] == ref["iterations"]
    assert last["ttot"] == ref["ttot"] and last["dt"] == ref["dt"]
    for j, s in enumerate(PRIMORDIAL_ORDER):
        assert np.array_equal((ref["state"][:, j] * W[j]).view(np.int64), rv[s].view(np.int64)), s
    assert np.array_equal(last["atol"].view(np.int64), ref["atol"].view(np.int64))
    it = ref["iterations"]
    assert rv_t["successful"].sum() == ref["substeps_ok"]
    assert rv_t["H_1"].shape == (16, niter) and rv_t["T"].shape == (16, niter)
    assert not rv_t["successful"][it:].any() and not rv_t["H_1"][:, it:].any()
    assert np.all(rv_t["T"][:, :it] > 0)
    assert np.all(np.diff(rv_t["t"][:it]) >= 0) and rv_t["dt"][0] == tf / 1e5


@pytest.mark.gpu
def test_generated_run_module(solver):
    """<n>_solver_run.py (generated beside the library) exposes run_<n> with
    the Cython module's signature."""
    import importlib.util
    import os
    from dengo_gb300.build import network_dir
    path = os.path.join(network_dir("primordial"), "primordial_solver_run.py")
    spec = importlib.util.spec_from_file_location("primordial_solver_run", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    ics = _ics(8, 44)
    rv, rv_t = mod.run_primordial(ics, 1e8, niter=500, intermediate=1)
    rv2, _ = solver.run(ics, 1e8, niter=500, intermediate=0)
    for s in PRIMORDIAL_ORDER:
        assert np.array_equal(rv[s].view(np.int64), rv2[s].view(np.int64)), s
    assert rv_t["H_1"].shape == (8, 500)


@pytest.mark.gpu
def test_main_driver_matches_evolve(solver, tmp_path):
    """primordial_main: initial-conditions file -> solution file, as the
    reference's stand-alone driver (stop_time, rtol = 1e-9, atol = 1e-9 x
    input); equal to dengo_evolve_primordial with the same arguments."""
    import ctypes as C
    from dengo_gb300.tablefile import read_table_file, write_table_file
    state, _ = primordial_cells(12, "cold", seed=61)
    write_table_file(str(tmp_path / "primordial_initial_conditions.dgt"),
                     {s: state[:, j] for j, s in enumerate(solver.species)})
    argv = (C.c_char_p * 2)(b"primordial_main", str(tmp_path).encode())
    rc = solver.lib.primordial_main(2, C.cast(argv, C.c_void_p))
    assert rc == 0, solver.last_error()
    sol = read_table_file(str(tmp_path / "primordial_solution.dgt"))
    ref, _, ttot, dt = solver.evolve(state, 3.1557e13, rtol=np.full_like(state, 1e-9),
                                     atol=state * 1e-9)
    for j, s in enumerate(solver.species):
        assert np.array_equal(sol[s].view(np.int64), ref[:, j].view(np.int64)), s
    assert sol["time"][0] == ttot and sol["timestep"][0] == dt
    assert np.array_equal(sol["T"], solver.temperature_from_mass_density(ref))


@pytest.fixture(scope="module")
def strip_so(tmp_path_factory):
    import host_engine as he
    return he.compile_engine("primordial", tmp_path_factory.mktemp("strip"), engine="strip")


@pytest.mark.parametrize("case", [0, 1, 2])
def test_run_strip_kernel_on_host_matches_reference_cython_driver(tables_in_order, case,
                                                                  strip_so):
    """run_strip_kernel (dg_strip.cuh, the GPU's <n>_run_strip) compiled for
    the host from its own source (tests/host_engine.py, its lanes as threads
    at barriers) against the reference's own Cython driver: final values and
    every per-iteration array, bit for bit."""
    import os
    import platform
    import host_engine as he
    if platform.machine() != "x86_64":
        pytest.skip("the goldens were made on x86-64")
    so = strip_so
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "primordial_run_golden.npz"))
    tf, niter = g["cases"][case]
    r = he.run_strip_in_subprocess(so, tables_in_order, g["ics"] / W, tf, int(niter), timeout=600)
    ige = PRIMORDIAL_ORDER.index("ge")
    got = dict(rv=r["state"] * W, successful=r["successful"], t=r["t"], dt=r["dt_traj"],
               T=r["traj_T"].T, ge=r["traj"][:, :, ige].T)
    for key, a in got.items():
        b = np.ascontiguousarray(g["run%d_%s" % (case, key)])
        a = np.ascontiguousarray(a, b.dtype)
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), key
    assert int(r["iterations"]) == int(np.count_nonzero(g["run%d_dt" % case]))


@pytest.mark.gpu
@pytest.mark.parametrize("case", [0, 1, 2])
def test_gpu_run_strip_matches_reference_cython_driver(solver, case):
    """Solver.run (<n>_run_strip on the GPU) against the reference's own
    Cython driver run_primordial: final values and every per-iteration
    array, bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "primordial_run_golden.npz"))
    tf, niter = g["cases"][case]
    ics = {s: np.ascontiguousarray(g["ics"][:, j]) for j, s in enumerate(PRIMORDIAL_ORDER)}
    rv, rv_t = solver.run(ics, float(tf), niter=int(niter), intermediate=1)
    got = dict(rv=np.stack([rv[s] for s in PRIMORDIAL_ORDER], axis=1),
               successful=rv_t["successful"], t=rv_t["t"], dt=rv_t["dt"], T=rv_t["T"],
               ge=rv_t["ge"])
    for key, a in got.items():
        b = np.ascontiguousarray(g["run%d_%s" % (case, key)])
        a = np.ascontiguousarray(a, b.dtype)
        assert a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8)), key
