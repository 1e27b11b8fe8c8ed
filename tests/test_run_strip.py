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
