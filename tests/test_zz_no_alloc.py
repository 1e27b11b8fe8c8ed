"""The allocation-free entry point, <n>_solve_cells_device_noalloc.

It serves callers that cannot allocate device memory while they run (a host
code that gives all device memory to its own pool at start-up, or one that
must not let a call synchronise the device as cudaMalloc and cudaFree do):
its scratch is a fixed static device array inside the library.  These tests
call it through the C ABI and require the same results as
<n>_solve_cells_device on two calls in a row -- the second call reuses the
scratch the first one left behind, and is the smaller one, so a stale tail
of the cell-order buffer would show -- for every engine variant, with and
without a cost hint, on a network with redshift tables at two redshifts, and
a clear rejection of a batch larger than the array allows.  The file is
named to run last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10            # the parity tolerance of tests/test_gpu_parity.py
MAX_CELLS = 1048448     # (4 MiB - 512 B) / 4 B per cell


def _bind(solver):
    from dengo_gb300.runtime import CellBatch, SolverConfig
    fn = getattr(solver.lib, "%s_solve_cells_device_noalloc" % solver.name)
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(CellBatch), C.c_double, C.POINTER(SolverConfig),
                   C.c_void_p]
    return fn


def _run(solver, state, dtf, hint, noalloc, cfg, z=-1.0):
    import torch
    from dengo_gb300.runtime import CellBatch
    n = len(dtf)
    st = torch.tensor(state.T.copy(), device="cuda")
    at = st * 1e-6
    d_dtf = torch.tensor(dtf, device="cuda")
    status = torch.zeros(n, dtype=torch.int32, device="cuda")
    sweeps = torch.zeros(n, dtype=torch.int32, device="cuda")
    h = None if hint is None else torch.tensor(hint, device="cuda")
    stream = torch.cuda.current_stream()
    if noalloc:
        b = CellBatch(n, 1, n, st.data_ptr(), at.data_ptr(), None, 1e-6, d_dtf.data_ptr(), 0.0,
                      None, None, status.data_ptr(), None, sweeps.data_ptr(), None,
                      None if h is None else h.data_ptr())
        rc = _bind(solver)(solver.data, C.byref(b), float(z), C.byref(cfg),
                           C.c_void_p(stream.cuda_stream))
        assert rc == 0, solver.last_error()
    else:
        solver.solve_device(st, n, 1, n, at, dtf=d_dtf, status=status, sweeps=sweeps, z=z,
                            config=cfg, stream=stream, cost_hint=h)
    torch.cuda.synchronize()
    return st.cpu().numpy(), at.cpu().numpy(), status.cpu().numpy(), sweeps.cpu().numpy()


def _same(got, ref):
    for a, b in zip(got[:2], ref[:2]):
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
        rel[a == b] = 0.0
        assert rel.max() <= RTOL
    assert np.array_equal(got[2], ref[2]) and np.array_equal(got[3], ref[3])


def test_noalloc_matches_allocating_entry_point_twice(solver):
    """Stiff config-3 cells, the default configuration (the allocating entry
    point redistributes stiff cells over three launches, the allocation-free
    one makes one launch: the same results)."""
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import primordial_cells
    cfg = Solver.default_config()
    for call, n in enumerate((700, 257)):
        state, dtf = primordial_cells(n, "config3", seed=900 + call)
        hint = np.random.default_rng(call).integers(0, 10**5, n).astype(np.int32)
        ref = _run(solver, state, dtf, hint, False, cfg)
        got = _run(solver, state, dtf, hint, True, cfg)
        _same(got, ref)


@pytest.mark.parametrize("wpc", [1, 2, 4])
@pytest.mark.parametrize("with_hint", [True, False])
def test_noalloc_every_engine_variant(solver, wpc, with_hint):
    """Neutral-gas cells (a few hundred sweeps each), every engine variant,
    with and without the cost-hint order, a larger call then a smaller one."""
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import primordial_cells
    cfg = Solver.default_config()
    cfg.warps_per_cell = wpc
    for call, n in enumerate((700, 257)):
        state, dtf = primordial_cells(n, "cold", seed=950 + call)
        hint = (np.random.default_rng(call).integers(0, 10**5, n).astype(np.int32)
                if with_hint else None)
        ref = _run(solver, state, dtf, hint, False, cfg)
        got = _run(solver, state, dtf, hint, True, cfg)
        _same(got, ref)


def test_noalloc_redshift_tables_at_two_redshifts():
    """The UV-background ion network: the redshift tables' values at each
    call's z travel with the launch, so consecutive calls at different z
    match the allocating entry point at the same z."""
    import os
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from dengo_gb300.build import build_network, library_path
    from dengo_gb300.runtime import Solver
    from dengo_gb300.workloads import oxygen_cells
    if not os.path.exists(library_path("oxygen_uvb")):
        build_network("oxygen_uvb")
    s = Solver("oxygen_uvb")
    cfg = Solver.default_config()
    state, dtf = oxygen_cells(160, seed=977, dt_range=(1e10, 1e11))
    for z in (0.5, 3.0, 0.5):
        ref = _run(s, state, dtf, None, False, cfg, z=z)
        got = _run(s, state, dtf, None, True, cfg, z=z)
        _same(got, ref)


def test_noalloc_rejects_batches_beyond_its_scratch(solver):
    import torch
    from dengo_gb300.runtime import CellBatch, Solver
    tiny = torch.zeros(16, dtype=torch.float64, device="cuda")
    b = CellBatch(MAX_CELLS + 1, 1, MAX_CELLS + 1, tiny.data_ptr(), tiny.data_ptr(), None, 1e-6,
                  None, 1.0, None, None, None, None, None, None, None)
    cfg = Solver.default_config()
    rc = _bind(solver)(solver.data, C.byref(b), -1.0, C.byref(cfg), None)
    assert rc == -1
    assert "allocation-free maximum" in solver.last_error()
