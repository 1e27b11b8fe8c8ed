"""The oracle (C restatement) against the reference's own outputs.

The golden vectors were produced by the reference's generated solver
(tests/golden/make_golden.py).  On the machine that made them the oracle
must agree bit for bit; elsewhere (another libm) to 1e-12 relative.
"""
import platform

import numpy as np
import pytest

BITWISE = platform.machine() == "x86_64"


def _same(a, b, rtol=1e-12):
    if BITWISE:
        return np.array_equal(np.asarray(a).view(np.int64), np.asarray(b).view(np.int64))
    with np.errstate(invalid="ignore"):
        return np.allclose(a, b, rtol=rtol, atol=0, equal_nan=True)


@pytest.mark.parametrize("tag", ["c1", "c3", "edge"])
def test_oracle_matches_reference_per_cell(golden, tables_in_order, oracle, tag):
    g = golden
    dt0 = g.get("evolve_%s_dt0" % tag)
    r = oracle.evolve_cells(tables_in_order, g["evolve_%s_in" % tag], g["evolve_%s_dtf" % tag],
                            dt=dt0, nthreads=4)
    for k in ("state", "atol", "dt", "ttot"):
        assert _same(r[k], g["evolve_%s_%s" % (tag, k)]), k


def test_oracle_statuses_cover_all_outcomes(golden, tables_in_order, oracle):
    r = oracle.evolve_cells(tables_in_order, golden["evolve_c1_in"], golden["evolve_c1_dtf"],
                            nthreads=4)
    assert set(np.unique(r["status"])) == {0, 1, 2}
    ok = r["status"] == 0
    assert np.all(r["ttot"][ok] >= golden["evolve_c1_dtf"][ok])
    assert np.all(r["substeps"][r["status"] == 1] == 50000)


def test_edge_cases_behave_like_reference(golden, tables_in_order, oracle):
    g = golden
    r = oracle.evolve_cells(tables_in_order, g["evolve_edge_in"], g["evolve_edge_dtf"],
                            dt=g["evolve_edge_dt0"], nthreads=1)
    assert r["ttot"][0] == 0.0 and r["substeps"][0] == 0          # dtf = 0
    assert r["status"][1] == 2                                     # negative density
    assert r["status"][2] == 2                                     # zero density -> NaN
    assert np.array_equal(r["state"][0], g["evolve_edge_in"][0])  # untouched state


def test_oracle_correctly_rounded_log():
    """dgo_crlog (the oracle variant's log T) is log correctly rounded."""
    import ctypes as C
    mpmath = pytest.importorskip("mpmath")
    from oracle import build_oracle
    lib = C.CDLL(build_oracle("primordial", crlog=True))
    lib.dgo_crlog.restype = C.c_double
    lib.dgo_crlog.argtypes = [C.c_double]
    mpmath.mp.prec = 200
    xs = np.exp(np.random.default_rng(5).uniform(0.0, np.log(2e9), 5000))
    for x in xs:
        assert lib.dgo_crlog(float(x)) == float(mpmath.log(mpmath.mpf(float(x)))), x


def test_oracle_lockstep_strip_matches_reference(golden, tables_in_order, oracle):
    """dengo_evolve over an 8-cell strip in lockstep (the reference's dims > 1
    semantics: one dt, one Newton loop for the strip), bit for bit."""
    from oracle import evolve_strip
    g = golden
    r = evolve_strip(oracle, tables_in_order, g["lock_in"], float(g["lock_dtf"]))
    assert _same(r["state"], g["lock_state"]) and _same(r["atol"], g["lock_atol"])
    assert _same(np.array(r["ttot"]), g["lock_ttot"]) and _same(np.array(r["dt"]), g["lock_dt"])


def _strip(oracle, tables_in_order):
    from oracle import Network
    net = Network.in_dll(oracle.lib, "dgo_%s_network" % oracle.name)
    keep, tp = oracle._tables(tables_in_order)
    return net, net.alloc_data(tp), keep


def test_oracle_strip_functions_match_reference(golden, tables_in_order, oracle):
    """calculate_rhs (with its temperature and rate interpolation),
    calculate_jacobian and ensure_electron_consistency on a 32-cell strip."""
    import ctypes as C
    g = golden
    P = C.POINTER(C.c_double)
    net, data, keep = _strip(oracle, tables_in_order)
    try:
        num = g["strip_in"].copy()
        rhs = np.zeros_like(num)
        assert net.rhs(num.ctypes.data_as(P), rhs.ctypes.data_as(P), 32, 10, data) == \
            int(g["strip_rhs_rv"])
        assert _same(rhs, g["strip_rhs"])
        assert _same(np.ctypeslib.as_array(net.Ts(data), (32,)), g["strip_Ts"])
        jac = np.zeros((32, 10, 10))
        assert net.jac(num.ctypes.data_as(P), jac.ctypes.data_as(P), 32, 10, data) == \
            int(g["strip_jac_rv"])
        assert _same(jac, g["strip_jac"])
    finally:
        net.free_data(data)
    el = g["strip_in"].copy()
    net.electrons(el.ctypes.data_as(P), 32, 10)
    assert _same(el, g["strip_electrons"])


def test_oracle_be_chem_solve_lockstep_matches_reference(golden, tables_in_order, oracle):
    """One BE_chem_solve over an 8-cell strip (BE_chem_solve.C:79-241)."""
    import ctypes as C
    from oracle import Network
    g = golden
    P = C.POINTER(C.c_double)
    fn = oracle.lib.dgo_BE_chem_solve
    fn.restype = C.c_int
    F = Network._fields_[5][1]
    fn.argtypes = [F, F, P, C.c_double, P, P, C.c_int, C.c_int, P, C.c_void_p, P, P, P, P,
                   C.c_int, C.c_void_p]
    net, data, keep = _strip(oracle, tables_in_order)
    try:
        u = g["be_in"].copy()
        rtol = np.full_like(u, 1e-6)
        atol = g["be_atol_in"].copy()
        scale = u.copy()
        scratch = [np.zeros(80), np.zeros(10), np.zeros(80), np.zeros(800)]
        rv = fn(net.rhs, net.jac, u.ctypes.data_as(P), float(g["be_dt"]),
                rtol.ctypes.data_as(P), atol.ctypes.data_as(P), 8, 10, scale.ctypes.data_as(P),
                data, *[a.ctypes.data_as(P) for a in scratch], 10, None)
    finally:
        net.free_data(data)
    assert rv == int(g["be_rv"])
    assert _same(u, g["be_u"]) and _same(atol, g["be_atol"])
