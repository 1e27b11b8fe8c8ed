"""The FP64 conservation check of the mixed-precision solve.

Every network's generated code carries the species combinations its
reactions conserve (Net::invariants: an integer basis of the left null space
of the stoichiometry, dengo_gb300/codegen/spec.py conservation_basis).  The
mixed solve compares them in FP64, at the end of every converged cell, with
the cell's input; a relative drift above dengo_solver_config.conservation_tol
(default 1e-9) re-solves the cell from its input with FP64 linear solves.
These tests check the invariants against the reactions, measure the FP64
oracle's own drift (the reference path), and run the engines' source
compiled for the host (tests/host_engine.py) with the check forced to fail:
every converged cell must then come out exactly as the FP64 path computes it.
"""
import os

import numpy as np
import pytest
import sympy

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
NETWORKS = ("primordial", "primordial_compton", "oxygen", "oxygen_uvb")


def _spec(name):
    from dengo_gb300.codegen.spec import network_spec
    from dengo_gb300.networks import build_network
    net = build_network(name)
    return net, network_spec(net, name)


@pytest.mark.parametrize("name", NETWORKS)
def test_every_reaction_conserves_the_invariants(name):
    net, spec = _spec(name)
    species = [s.name for s in spec.species]
    assert spec.conservation, name
    for rn, r in net.reactions.items():
        delta = np.zeros(len(species))
        for n, x in r.right_side:
            delta[species.index(x.name)] += float(n)
        for n, x in r.left_side:
            delta[species.index(x.name)] -= float(n)
        for c in spec.conservation:
            assert float(np.dot(c, delta)) == 0.0, (name, rn, c)
    # a basis: as many independent vectors as the null space has
    assert sympy.Matrix(spec.conservation).rank() == len(spec.conservation)


def test_primordial_invariants_are_the_nuclei():
    """H and He nuclei; the reference's k12 (H2 + e -> 2 H+ + e,
    dengo/primordial_rates.py:191) changes the charge, so charge is not an
    invariant of the primordial network as the reference defines it."""
    _, spec = _spec("primordial")
    order = [s.name for s in spec.species]
    want = [[2 if s.startswith("H2") else (1 if s.startswith("H_") else 0) for s in order],
            [1 if s.startswith("He") else 0 for s in order]]
    assert sorted(spec.conservation) == sorted(want)


def test_ion_networks_also_conserve_a_charge_combination():
    _, spec = _spec("oxygen")
    order = [s.name for s in spec.species]
    de = order.index("de")
    assert any(c[de] != 0 for c in spec.conservation)


def _drift(state_in, state_out, spec):
    from dengo_gb300.workloads import MH
    w = np.array([float(s.weight) if not s.is_ge else 1.0 for s in spec.species])
    ige = [s.is_ge for s in spec.species].index(True)

    def num(x):
        n = x.copy()
        for j in range(n.shape[1]):
            if j != ige:
                n[:, j] /= w[j] * MH
        return n
    a, b = num(state_in), num(state_out)
    C = np.array(spec.conservation, float)
    return np.abs(b @ C.T - a @ C.T) / (np.abs(a) @ np.abs(C).T)


def test_fp64_oracle_drift_is_far_below_the_default_tolerance(tables_in_order, oracle):
    """The reference path's own drift on converged config-1 and config-3
    cells stays below 1e-10, a hundredth of the default tolerance.  (Its
    electron consistency at the start changes no nuclei count.)"""
    from dengo_gb300.workloads import primordial_cells
    _, spec = _spec("primordial")
    for cfg in ("config1", "config3"):
        st, dtf = primordial_cells(96, cfg, seed=515)
        r = oracle.evolve_cells(tables_in_order, st, dtf)
        ok = r["status"] == 0
        assert ok.sum() > 30
        assert _drift(st[ok], r["state"][ok], spec).max() < 1e-10


@pytest.fixture(scope="module")
def engines(tmp_path_factory):
    import host_engine as he
    d = tmp_path_factory.mktemp("cons")
    return {"lane": he.compile_engine("primordial", d),
            "split": he.compile_engine("primordial", d, engine="split")}


@pytest.mark.parametrize("engine", ["lane", "split"])
def test_failed_check_resolves_the_cell_in_fp64(tables_in_order, engines, engine):
    """With the check made to fail for every converged cell, each is solved
    again from its input with FP64 linear solves: its state, status and
    counters equal the FP64 path's bit for bit; cells that did not converge
    are not checked and keep the mixed solve's result.  With a sweep budget,
    so re-solved cells also pass through the resume launches."""
    import host_engine as he
    from dengo_gb300.workloads import primordial_cells
    # neutral-gas cells (quick); for the single-lane engine also four
    # config-1 cells, two of which end at the substep cap (in FP64: 1.5e5
    # sweeps each, too slow for the split engine's 128 host threads)
    st, dtf = primordial_cells(40, "cold", seed=808)
    if engine == "lane":
        st2, dtf2 = primordial_cells(4, "config1", seed=27)
        st, dtf = np.concatenate([st, st2]), np.concatenate([dtf, dtf2])
    fp64 = he.evolve_in_subprocess(engines[engine], tables_in_order, st, dtf)
    mixed = he.evolve_in_subprocess(engines[engine], tables_in_order, st, dtf, mixed=True)
    forced = he.evolve_in_subprocess(engines[engine], tables_in_order, st, dtf, mixed=True,
                                     cons_tol=-1.0, sweep_budget=300)
    ok = forced["status"] == 0
    assert ok.sum() > 20 and (engine != "lane" or (~ok).sum() == 2)
    assert np.array_equal(forced["status"], np.where(ok, 0, mixed["status"]))
    assert np.array_equal(forced["state"][ok], fp64["state"][ok])
    for k in ("substeps", "sweeps", "failures"):
        assert np.array_equal(forced[k][ok], fp64[k][ok]), k
    assert np.array_equal(forced["state"][~ok], mixed["state"][~ok])


def test_default_tolerance_leaves_mixed_cells_alone(tables_in_order, engines):
    """At the default 1e-9 no converged config-1/config-3 cell of the mixed
    solve fails the check: the results equal those without it."""
    import host_engine as he
    from dengo_gb300.workloads import primordial_cells
    for cfg in ("cold", "config3"):
        st, dtf = primordial_cells(32, cfg, seed=909)
        a = he.evolve_in_subprocess(engines["lane"], tables_in_order, st, dtf, mixed=True)
        b = he.evolve_in_subprocess(engines["lane"], tables_in_order, st, dtf, mixed=True,
                                    cons_tol=1e-9)
        assert np.array_equal(a["state"], b["state"]) and np.array_equal(a["sweeps"], b["sweeps"])
