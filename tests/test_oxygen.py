"""The ion-by-ion networks (H, He and O ions + electrons + energy, 16
equations): ``oxygen`` and ``oxygen_uvb`` (the same ions under a UV
background: photoionisation and photoheating tabulated in redshift).
Generated tables, oracle and GPU solver against the reference's own outputs
(tests/golden/make_golden.py oxygen / oxygen_uvb)."""
import hashlib
import os
import platform

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BITWISE = platform.machine() == "x86_64"
NETWORKS = ("oxygen", "oxygen_uvb")


def _cases(gold):
    """(tag, z) pairs: one per redshift for networks with redshift tables."""
    if "redshifts" in gold:
        return [("_z%g" % z, float(z)) for z in gold["redshifts"]]
    return [("", -1.0)]


_GOLD, _TABLES, _ORACLES = {}, {}, {}


def gold(name):
    if name not in _GOLD:
        _GOLD[name] = dict(np.load(os.path.join(ROOT, "tests", "golden", "%s_golden.npz" % name)))
    return _GOLD[name]


def tables(name):
    if name not in _TABLES:
        from dengo_gb300.runtime import network_dir
        from dengo_gb300.tablefile import read_table_file
        t = read_table_file(os.path.join(network_dir(name), "%s_tables.dgt" % name))
        _TABLES[name] = [np.ascontiguousarray(t[k]) for k in gold(name)["table_order"]]
    return _TABLES[name]


def oracle_for(name, crlog=False):
    if (name, crlog) not in _ORACLES:
        from oracle import Oracle
        _ORACLES[name, crlog] = Oracle(name, crlog=crlog)
    return _ORACLES[name, crlog]


@pytest.mark.parametrize("name", NETWORKS)
def test_shipped_tables_are_the_references(name):
    g = gold(name)
    for tname, tab, sha in zip(g["table_order"], tables(name), g["table_sha256"]):
        assert hashlib.sha256(tab.tobytes()).hexdigest() == sha, tname


def test_uvb_tables_depend_on_redshift():
    g = gold("oxygen_uvb")
    zt = [n for n in g["table_order"] if n.endswith("_pi") or "_ph_" in n]
    assert len(zt) == 22
    from dengo_gb300.codegen.spec import network_spec  # noqa: F401  (import check only)
    lens = {len(t) for n, t in zip(g["table_order"], tables("oxygen_uvb")) if n in zt}
    assert lens == {100}


@pytest.mark.parametrize("name", NETWORKS)
def test_oracle_matches_reference(name):
    g = gold(name)
    for tag, z in _cases(g):
        r = oracle_for(name).evolve_cells(tables(name), g["evolve_in"], g["evolve_dtf"], z=z,
                                          nthreads=4)
        for k in ("state", "atol", "dt", "ttot"):
            a, b = r[k], g["evolve%s_%s" % (tag, k)]
            if BITWISE:
                assert np.array_equal(a.view(np.int64), b.view(np.int64)), (tag, k)
            else:
                assert np.allclose(a, b, rtol=1e-12, atol=0, equal_nan=True), (tag, k)


def test_uvb_redshift_changes_the_result():
    g = gold("oxygen_uvb")
    a, b = g["evolve_z2.5_state"], g["evolve_z20_state"]
    assert not np.array_equal(a, b)


def _solver(name):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from dengo_gb300.build import build_network, library_path
    if not os.path.exists(library_path(name)):
        build_network(name)
    from dengo_gb300.runtime import Solver
    return Solver(name)


@pytest.mark.gpu
@pytest.mark.parametrize("name,wpc", [("oxygen", 1), ("oxygen", 4), ("oxygen_uvb", 4)])
def test_gpu_matches_reference(name, wpc):
    """FP64 path at every redshift of the golden set (in the table range, and
    beyond it where the reference switches the photo terms off).

    Against the oracle built with a correctly rounded log T (the device's
    log is correctly rounded): same status everywhere; converged cells within
    1e-10 with the same sweep counts.  Against the reference's own outputs
    (libm log): within 1e-10 on every converged cell whose correctly-rounded
    oracle result also is -- the others are long trajectories on which libm's
    occasional mis-rounding of log T changes a Newton decision."""
    from dengo_gb300.runtime import Solver
    s = _solver(name)
    g = gold(name)
    cfg = Solver.default_config()
    cfg.warps_per_cell = wpc
    st, dtf = g["evolve_in"], g["evolve_dtf"]
    rel = lambda a, b: (np.abs(a - b) / np.maximum(np.abs(b), 1e-300)).max(axis=1)
    for tag, z in _cases(g):
        out = s.solve_host(st, dtf, rtol=1e-6, config=cfg, counters=True, z=z)
        cr = oracle_for(name, crlog=True).evolve_cells(tables(name), st, dtf, z=z, nthreads=4)
        assert np.array_equal(out["status"], cr["status"]), tag
        ok = cr["status"] == 0
        assert ok.sum() >= 0.5 * len(ok)
        assert rel(out["state"][ok], cr["state"][ok]).max(initial=0.0) <= 1e-10, tag
        assert np.array_equal(out["sweeps"][ok], cr["sweeps"][ok]), tag
        gs = g["evolve%s_state" % tag]
        same_as_ref = ok & (rel(cr["state"], gs) <= 1e-10)
        assert same_as_ref.sum() >= ok.sum() - 2, tag
        assert rel(out["state"][same_as_ref], gs[same_as_ref]).max(initial=0.0) <= 1e-10, tag


@pytest.mark.gpu
def test_gpu_mixed_within_1e6():
    """Mixed path on the 16-equation network: every cell ends with the FP64
    oracle's status; >= 80% of them within 1e-6 of it (floored relative
    error, atol = 1e-6 x the input).  On the rest the reference's unscaled
    FP64 elimination itself is inaccurate: an extended-precision solve
    departs from the FP64 oracle on the same cells, by up to O(1)."""
    from dengo_gb300.runtime import Solver
    s = _solver("oxygen")
    g = gold("oxygen")
    cfg = Solver.default_config()
    cfg.precision, cfg.warps_per_cell = 1, 4
    st, dtf = g["evolve_in"], g["evolve_dtf"]
    out = s.solve_host(st, dtf, rtol=1e-6, config=cfg)
    ref = oracle_for("oxygen").evolve_cells(tables("oxygen"), st, dtf, nthreads=4)
    assert np.array_equal(out["status"], ref["status"])
    conv = ref["status"] == 0
    err = np.abs(out["state"][conv] - ref["state"][conv]) / np.maximum(
        np.abs(ref["state"][conv]), 1e-6 * np.abs(st[conv]))
    from conftest import species_error_report, write_report
    write_report("mixed_species_oxygen", species_error_report(s.species, err, conv.sum(), 1e-6))
    assert np.mean(err.max(axis=1) <= 1e-6) >= 0.8, np.sort(err.max(axis=1))[-10:]


def test_ion_helpers_register_the_references_names():
    """The reference's ion-by-ion helpers (reaction_classes.py:167-198,
    200-271, 379-441, 443-514) exist under the same names and register the
    same terms: the shipped ion networks are built through them."""
    from dengo_gb300 import reaction_classes as rc
    from dengo_gb300.ion_by_ion import oxygen_uvb_network
    oxygen_uvb_network()
    o1, o2, o9 = (rc.species_registry[n] for n in ("O_1", "O_2", "O_9"))
    assert rc.chianti_rate("O", None, o1, o2) == ["O_1_i"]
    assert rc.chianti_rate("O", rc.species_registry["O_8"], o9, None) == ["O_9_r"]
    assert rc.ion_cooling_rate(o2, "O") == ["O_2_c"]
    assert rc.ion_photoionization_rate(o1) == ["O_1_pi"]
    assert rc.ion_photoionization_rate(o9) == []
    assert rc.ion_photoheating_rate(o1) == ["O_1_ph"]
    r = rc.reaction_registry["O_1_pi"]
    assert [s.name for _, s in r.left_side] == ["O_1"]
    assert sorted(s.name for _, s in r.right_side) == ["O_2", "de"]
    assert rc.cooling_registry["O_1_ph"]._equation == "O_1_ph * O_1"
