"""Compton cooling off the CMB (the reference's ``compton`` cooling action,
primordial_cooling.py:280-292): ``primordial_compton`` is the primordial
network with that action, whose term ``-comp (1+z)^4 (T - 2.73 (1+z)) de``
reads the call's redshift and the cell's temperature directly.  Tables,
oracle and GPU solver against the reference's own outputs at five redshifts
(tests/golden/make_golden.py primordial_compton)."""
import hashlib
import os
import platform

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NAME = "primordial_compton"
RTOL = 1e-10
# The goldens were made on x86-64; elsewhere libm (and numpy's elementary
# functions) round some values differently.
BITWISE = platform.machine() == "x86_64"

_CACHE = {}


def gold():
    if "gold" not in _CACHE:
        _CACHE["gold"] = dict(np.load(os.path.join(ROOT, "tests", "golden", NAME + "_golden.npz")))
    return _CACHE["gold"]


def tables():
    """The shipped tables (the ones the GPU library loads), in the solver's
    order."""
    if "tables" not in _CACHE:
        from dengo_gb300.build import network_dir
        from dengo_gb300.tablefile import read_table_file
        t = read_table_file(os.path.join(network_dir(NAME), NAME + "_tables.dgt"))
        _CACHE["tables"] = [np.ascontiguousarray(t[k]) for k in gold()["table_order"]]
    return _CACHE["tables"]


def oracle(crlog=False):
    if ("oracle", crlog) not in _CACHE:
        from oracle import Oracle
        _CACHE["oracle", crlog] = Oracle(NAME, crlog=crlog)
    return _CACHE["oracle", crlog]


def redshifts():
    return [float(z) for z in gold()["redshifts"]]


def tag(z):
    return "_z%g" % z


def test_network_has_the_compton_term():
    from dengo_gb300.codegen.spec import network_spec
    from dengo_gb300.networks import build_network
    s = network_spec(build_network(NAME), NAME)
    assert [t.name for t in s.tables if t.name.startswith("compton")] == ["compton_comp"]
    assert not any(t.zdep for t in s.tables)
    assert "compton_comp[i]*de*pow(z + 1.0, 4)*(T - 2.73*z - 2.73)" in s.rhs_ref[s.ige]


def test_shipped_tables_are_the_references():
    g = gold()
    assert [hashlib.sha256(t.tobytes()).hexdigest() for t in tables()] == list(g["table_sha256"])


def test_write_solver_reproduces_the_tables(tmp_path):
    from dengo_gb300.networks import build_network
    from dengo_gb300.tablefile import read_table_file
    build_network(NAME).write_solver(NAME, output_dir=str(tmp_path))
    t = read_table_file(os.path.join(str(tmp_path), NAME + "_tables.dgt"))
    for name, ref in zip(gold()["table_order"], tables()):
        if BITWISE:
            assert np.array_equal(t[name].view(np.int64), ref.view(np.int64)), name
        else:
            assert np.allclose(t[name], ref, rtol=1e-13, atol=0), name


@pytest.mark.parametrize("z", [-1.0, 0.0, 3.0, 9.0, 19.0])
def test_oracle_matches_reference(z):
    """Bit for bit, every cell, at every redshift of the golden set."""
    g = gold()
    assert z in redshifts()
    r = oracle().evolve_cells(tables(), g["evolve_in"], g["evolve_dtf"], z=z, nthreads=0)
    for k in ("state", "atol", "dt", "ttot"):
        a, b = r[k], g["evolve%s_%s" % (tag(z), k)]
        if BITWISE:
            assert np.array_equal(a.view(np.int64), b.view(np.int64)), k
        else:
            assert np.allclose(a, b, rtol=1e-12, atol=0, equal_nan=True), k


def test_redshift_changes_the_result():
    """The reference's outputs differ between every pair of redshifts, so the
    golden set exercises the term."""
    g = gold()
    zs = redshifts()
    for a, b in zip(zs, zs[1:]):
        sa, sb = g["evolve%s_state" % tag(a)], g["evolve%s_state" % tag(b)]
        assert np.mean(np.any(sa != sb, axis=1)) > 0.9, (a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("wpc", [1, 4])
def test_gpu_matches_reference(wpc):
    """FP64 path at every redshift.  Against the oracle built with a
    correctly rounded log T (the device's log is correctly rounded): same
    status everywhere; converged cells within 1e-10 with the same sweep
    counts.  Against the reference's own outputs: within 1e-10 on every
    converged cell."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from dengo_gb300.build import build_network, library_path
    if not os.path.exists(library_path(NAME)):
        build_network(NAME)
    from dengo_gb300.runtime import Solver
    s = Solver(NAME)
    g = gold()
    cfg = Solver.default_config()
    cfg.warps_per_cell = wpc
    st, dtf = g["evolve_in"], g["evolve_dtf"]
    rel = lambda a, b: (np.abs(a - b) / np.maximum(np.abs(b), 1e-300)).max(axis=1)
    for z in redshifts():
        out = s.solve_host(st, dtf, rtol=1e-6, config=cfg, counters=True, z=z)
        cr = oracle(crlog=True).evolve_cells(tables(), st, dtf, z=z, nthreads=0)
        assert np.array_equal(out["status"], cr["status"]), z
        ok = cr["status"] == 0
        assert ok.sum() >= 0.75 * len(ok)
        assert rel(out["state"][ok], cr["state"][ok]).max(initial=0.0) <= RTOL, z
        assert np.array_equal(out["sweeps"][ok], cr["sweeps"][ok]), z
        gs = g["evolve%s_state" % tag(z)]
        assert rel(out["state"][ok], gs[ok]).max(initial=0.0) <= RTOL, z
