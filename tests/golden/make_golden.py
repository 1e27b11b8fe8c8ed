"""Generates the golden vectors under tests/golden/ from the reference itself.

Run where the reference checkout exists (it is read, never modified):

    python tests/golden/make_golden.py

1. Builds the reference's own primordial solver (oracle/ref_build.py: the
   reference's templates rendered by its own ``write_solver``, compiled with
   its ``BE_chem_solve.C``).
2. Runs it on seeded inputs and stores inputs and outputs in
   ``primordial_golden.npz``:
   * ``evolve_*``: ``dengo_evolve_primordial`` called once per cell
     (dims = 1) on config-1 and config-3 cells plus edge cases (dtf = 0,
     a negative density, a zero density, a given initial dt, T at and above
     the table's upper bound, T below its lower bound);
   * ``strip_*``: calculate_temperature / interpolate_rates /
     calculate_rhs / calculate_jacobian on a 32-cell strip of number
     densities, and ensure_electron_consistency on that strip;
   * ``be_*``: one ``BE_chem_solve`` over an 8-cell strip in lockstep;
   * ``lock_*``: ``dengo_evolve_primordial`` over an 8-cell strip (dims = 8,
     the reference's lockstep semantics);
   (``python tests/golden/make_golden.py intermediate`` writes
   ``primordial_intermediate_golden.npz``: that strip's intermediate files,
   from the reference rendered with ``write_intermediate_solutions``;
   ``oxygen``, ``oxygen_uvb``, ``primordial_compton`` and ``run`` the other
   networks' and the Cython driver's vectors)
   * ``tables``: every rate and cooling table the reference wrote.
3. Stores the reference's printed expressions (RHS rows, Jacobian entries,
   T(ge), dT/dge, mass density) in ``primordial_expressions.json`` after
   checking that each appears verbatim in the reference's rendered C.
"""

import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from dengo_gb300.workloads import primordial_cells  # noqa: E402

P_D = C.POINTER(C.c_double)


def dp(a):
    return a.ctypes.data_as(P_D)


def edge_cells():
    """Hand-made cells exercising the driver's special paths."""
    base, dtf = primordial_cells(8, "config1", seed=777)
    cells = base.copy()
    dtfs = dtf.copy()
    dts = np.full(8, -1.0)
    dtfs[0] = 0.0                       # no substep at all
    cells[1, 3] = -1e-30                # a negative H+ density
    cells[2, 4] = 0.0                   # a zero H- density: scale 0 -> NaN
    dts[3] = dtfs[3] / 37.0             # caller-given initial dt
    cells[4, 9] *= 1e4                  # very hot: T clamps at the upper bound
    cells[5, 9] *= 1e-6                 # very cold: T clamps at the lower bound
    return cells, dtfs, dts


def compton_cells():
    """Config-1 cells, and config-1 cells made diffuse (x 1e-4 in every
    density) and hotter (ge x 10), where Compton cooling off the CMB is a
    large share of the cooling at the higher redshifts."""
    a, da = primordial_cells(32, "config1", seed=1971)
    b, db = primordial_cells(32, "config1", seed=1972)
    b = b.copy()
    b[:, :9] *= 1e-4
    b[:, 9] *= 10.0
    return np.concatenate([a, b]), np.concatenate([da, db * 100.0])


def main():
    import ref_build
    from oracle import Reference
    ref_build.build("primordial")
    ref = Reference("primordial")
    N = ref.N
    out = {}

    # -- per-cell evolve ----------------------------------------------------
    for tag, cfg, n in (("c1", "config1", 64), ("c3", "config3", 64)):
        st, dtf = primordial_cells(n, cfg)
        r = ref.evolve_cells(st, dtf, nthreads=8)
        out["evolve_%s_in" % tag] = st
        out["evolve_%s_dtf" % tag] = dtf
        for k in ("state", "atol", "dt", "ttot"):
            out["evolve_%s_%s" % (tag, k)] = r[k]
    st, dtf, dts = edge_cells()
    r = ref.evolve_cells(st, dtf, dt=dts, nthreads=8)
    out["evolve_edge_in"], out["evolve_edge_dtf"], out["evolve_edge_dt0"] = st, dtf, dts
    for k in ("state", "atol", "dt", "ttot"):
        out["evolve_edge_%s" % k] = r[k]

    # -- strip functions ------------------------------------------------------
    lib = ref.lib
    d = lib.ref_setup()
    st, _ = primordial_cells(32, "config1", seed=4242)
    w = np.array([2.0, 2.0, 1.00794, 1.00794, 1.00794, 4.002602, 4.002602, 4.002602, 1.0, 0.0])
    num = st.copy()
    num[:, :9] /= w[:9] * 1.67e-24
    out["strip_in"] = num.copy()
    lib.ref_temperature(d, dp(num), 32, N)
    out["strip_Ts"] = np.ctypeslib.as_array(lib.ref_Ts(d), (32,)).copy()
    out["strip_dTs_ge"] = np.ctypeslib.as_array(lib.ref_dTs_ge(d), (32,)).copy()
    lib.ref_interpolate(d, 32)
    nt = 44
    out["strip_rs"] = np.array([np.ctypeslib.as_array(lib.ref_rs(d, k), (32,)).copy()
                                for k in range(nt)])
    rhs = np.zeros_like(num)
    out["strip_rhs_rv"] = np.array(lib.ref_rhs(dp(num), dp(rhs), 32, N, C.c_void_p(d)))
    out["strip_rhs"] = rhs
    jac = np.zeros((32, N, N))
    out["strip_jac_rv"] = np.array(lib.ref_jac(dp(num), dp(jac), 32, N, C.c_void_p(d)))
    out["strip_jac"] = jac
    el = num.copy()
    lib.ref_electrons(dp(el), 32, N)
    out["strip_electrons"] = el

    # -- BE_chem_solve over a strip (lockstep) -------------------------------
    ns = 8
    u = num[:ns].copy()
    rtol = np.full_like(u, 1e-6)
    atol = 1e-6 * u
    scale = u.copy()
    out["be_in"], out["be_atol_in"] = u.copy(), atol.copy()
    out["be_dt"] = np.array(1e10)
    scratch = [np.zeros(ns * N), np.zeros(N), np.zeros(ns * N), np.zeros(ns * N * N)]
    rv = lib.ref_BE_chem_solve(dp(u), 1e10, dp(rtol), dp(atol), ns, N, dp(scale), C.c_void_p(d),
                               *[dp(a) for a in scratch])
    out["be_rv"], out["be_u"], out["be_atol"] = np.array(rv), u, atol

    # -- dengo_evolve over a strip (lockstep dims = 8) -----------------------
    st, dtf = primordial_cells(8, "config1", seed=99)
    x = st.copy()
    rt = np.full_like(x, 1e-6)
    at = 1e-6 * x
    dt = C.c_double(-1.0)
    ttot = lib.ref_evolve(d, float(dtf.min()), C.byref(dt), -1.0, dp(x), dp(rt), dp(at), 8)
    out["lock_in"], out["lock_dtf"] = st, np.array(dtf.min())
    out["lock_state"], out["lock_atol"] = x, at
    out["lock_ttot"], out["lock_dt"] = np.array(ttot), np.array(dt.value)

    # -- tables ----------------------------------------------------------------
    tdir = os.path.join(ROOT, "oracle", "_ref", "primordial", "primordial_tables.h5.d")
    names = sorted(f[:-4] for f in os.listdir(tdir))
    out["table_names"] = np.array(names)
    out["tables"] = np.array([np.fromfile(os.path.join(tdir, f + ".f64")) for f in names])
    np.savez_compressed(os.path.join(HERE, "primordial_golden.npz"), **out)

    # -- expressions -----------------------------------------------------------
    from dengo_gb300.codegen.spec import network_spec
    from dengo_gb300.networks import primordial_network
    spec = network_spec(primordial_network(), "primordial")
    src = open(os.path.join(ROOT, "oracle", "_ref", "primordial", "primordial_solver.C")).read()
    exprs = dict(rhs=spec.rhs_ref, jac=spec.jac_ref, T=spec.T_ref, Tge=spec.Tge_ref,
                 density=spec.mass_density_ref, species=[s.name for s in spec.species],
                 tables=[t.name for t in spec.tables])
    for text in spec.rhs_ref + [e for col in spec.jac_ref for e in col] + \
            [spec.T_ref, spec.Tge_ref, spec.mass_density_ref]:
        assert text in src, "expression not found in the reference's rendered C: %s" % text
    with open(os.path.join(HERE, "primordial_expressions.json"), "w") as f:
        json.dump(exprs, f, indent=1)
    print("wrote golden vectors to", HERE)


if __name__ == "__main__" and len(sys.argv) == 1:
    main()


def make_ion(name="oxygen", zs=(None,), cells=None):
    """Golden vectors of an ion-by-ion network (16 equations): the
    reference's own setup_ionization and templates, with the synthetic
    CHIANTI and UV-background stand-in tables (oracle/ref_build.py).  For a
    network whose terms depend on the redshift, one set of outputs per
    redshift.  ``cells``: (state, dtf), by default 48 seeded oxygen cells."""
    import hashlib
    import ref_build
    from oracle import Reference
    from dengo_gb300.codegen.spec import network_spec
    from dengo_gb300.networks import build_network
    from dengo_gb300.workloads import oxygen_cells
    ref_build.build(name)
    ref = Reference(name)
    out = {}
    st, dtf = cells if cells is not None else oxygen_cells(48, seed=515)
    out["evolve_in"], out["evolve_dtf"] = st, dtf
    for z in zs:
        r = ref.evolve_cells(st, dtf, nthreads=8, z=-1.0 if z is None else z)
        tag = "" if z is None else "_z%g" % z
        for k in ("state", "atol", "dt", "ttot"):
            out["evolve%s_%s" % (tag, k)] = r[k]
    if zs != (None,):
        out["redshifts"] = np.array(zs, dtype=float)
    # the solver's table order, and a SHA-256 of each table the reference wrote
    spec = network_spec(build_network(name), name)
    tdir = os.path.join(ROOT, "oracle", "_ref", name, "%s_tables.h5.d" % name)
    files = {f[:-4]: os.path.join(tdir, f) for f in os.listdir(tdir)}
    out["table_order"] = np.array([t.name for t in spec.tables])
    out["table_sha256"] = np.array([hashlib.sha256(np.fromfile(files[t.name]).tobytes()).hexdigest()
                                    for t in spec.tables])
    np.savez_compressed(os.path.join(HERE, "%s_golden.npz" % name), **out)
    print("wrote %s golden vectors" % name)


RUN_CASES = ((1e8, 3000), (1e10, 3000), (1e9, 40))


def make_run():
    """Golden vectors of the reference's own Cython driver run_primordial
    (rates_and_rate_tables_run.pyx.template:81-205, compiled by
    oracle/ref_build.py build_cython_driver) on one 16-cell config-1 strip:
    for each (tf, niter) the final state (rv), the per-iteration success
    flags, times and steps, and the temperature and ge trajectories."""
    import importlib
    import ref_build
    from dengo_gb300.workloads import PRIMORDIAL_ORDER, PRIMORDIAL_WEIGHTS
    odir = ref_build.build_cython_driver("primordial")
    W = np.array([PRIMORDIAL_WEIGHTS.get(s, 1.0) for s in PRIMORDIAL_ORDER])
    st, _ = primordial_cells(16, "config1", seed=31)
    num = st / (W * 1.67e-24)
    num[:, -1] = st[:, -1]
    ics = {s: np.ascontiguousarray(num[:, j] * W[j]) for j, s in enumerate(PRIMORDIAL_ORDER)}
    out = {"ics": np.stack([ics[s] for s in PRIMORDIAL_ORDER], axis=1),
           "cases": np.array(RUN_CASES, dtype=float)}
    cwd = os.getcwd()
    sys.path.insert(0, odir)
    os.chdir(odir)
    try:
        m = importlib.import_module("primordial_solver_run")
        for k, (tf, niter) in enumerate(RUN_CASES):
            rv, rv_t = m.run_primordial({s: a.copy() for s, a in ics.items()}, tf, niter=niter,
                                        intermediate=1)
            out["run%d_rv" % k] = np.stack([rv[s] for s in PRIMORDIAL_ORDER], axis=1)
            for key in ("successful", "t", "dt"):
                out["run%d_%s" % (k, key)] = np.asarray(rv_t[key])
            out["run%d_T" % k] = np.asarray(rv_t["T"])
            out["run%d_ge" % k] = np.asarray(rv_t["ge"])
    finally:
        os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, "primordial_run_golden.npz"), **out)
    print("wrote primordial_run_golden.npz")


def make_intermediate():
    """Golden vectors of the reference's intermediate files: the primordial
    network rendered with ``write_intermediate_solutions`` set
    (oracle/ref_build.py build(intermediate=True)); its
    ``dengo_evolve_primordial`` over an 8-cell config-1 strip (dims = 8, the
    ``lock_*`` inputs) writes ``primordial_intermediate_%06d.h5`` after every
    accepted substep (rates_and_rate_tables.C.template:212-241).  Stored in
    ``primordial_intermediate_golden.npz``: the inputs, the final state, and
    per file its number, the species (the state before that substep, number
    densities), T, and the time and timestep attributes."""
    import glob
    import shutil
    import ref_build
    from oracle import Reference
    ref_build.build("primordial", intermediate=True)
    ref = Reference("primordial", intermediate=True)
    outdir = os.environ["DGO_REF_TABLE_DIR"]
    for old in glob.glob(os.path.join(outdir, "primordial_intermediate_*.h5.d")):
        shutil.rmtree(old)
    d = ref.lib.ref_setup()
    st, dtf = primordial_cells(8, "config1", seed=99)
    x = st.copy()
    rt = np.full_like(x, 1e-6)
    at = 1e-6 * x
    dt = C.c_double(-1.0)
    ttot = ref.lib.ref_evolve(d, float(dtf.min()), C.byref(dt), -1.0, dp(x), dp(rt), dp(at), 8)
    dirs = sorted(glob.glob(os.path.join(outdir, "primordial_intermediate_*.h5.d")))
    species = ("H2_1", "H2_2", "H_1", "H_2", "H_m0", "He_1", "He_2", "He_3", "de", "ge")
    out = dict(inp=st, dtf=np.array(dtf.min()), state=x, atol=at, ttot=np.array(ttot),
               dt=np.array(dt.value))
    out["siter"] = np.array([int(p.rsplit("_", 1)[1].split(".")[0]) for p in dirs])
    out["species"] = np.array([np.stack([np.fromfile(os.path.join(p, s + ".f64"))
                                         for s in species], axis=1) for p in dirs])
    out["T"] = np.array([np.fromfile(os.path.join(p, "T.f64")) for p in dirs])
    out["time"] = np.array([np.fromfile(os.path.join(p, "@time.f64"))[0] for p in dirs])
    out["timestep"] = np.array([np.fromfile(os.path.join(p, "@timestep.f64"))[0] for p in dirs])
    for p in dirs:
        shutil.rmtree(p)
    np.savez_compressed(os.path.join(HERE, "primordial_intermediate_golden.npz"), **out)


if __name__ == "__main__" and len(sys.argv) > 1:
    if sys.argv[1] == "intermediate":
        make_intermediate()
    elif sys.argv[1] == "oxygen":
        make_ion("oxygen")
    elif sys.argv[1] == "oxygen_uvb":
        make_ion("oxygen_uvb", zs=(0.0, 2.5, 9.0, 20.0))
    elif sys.argv[1] == "run":
        make_run()
    elif sys.argv[1] == "primordial_compton":
        make_ion("primordial_compton", zs=(-1.0, 0.0, 3.0, 9.0, 19.0),
                 cells=compton_cells())
