"""The allocation-free entry point, primordial_solve_cells_device_noalloc.

It serves callers that cannot allocate device memory while they run (a host
code that gives all device memory to its own pool at start-up, or one that
must not let a call synchronise the device as cudaMalloc and cudaFree do):
its scratch is a fixed static device array inside the library.  These tests
call it through the C ABI and require the same results as
primordial_solve_cells_device on two calls in a row -- the second call reuses
the scratch the first one left behind -- and a clear rejection of a batch
larger than the array allows.  The file is named to run last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10            # the parity tolerance of tests/test_gpu_parity.py
MAX_CELLS = 1048448     # (4 MiB - 512 B) / 4 B per cell


def _bind(solver):
    from dengo_gb300.runtime import CellBatch, SolverConfig
    fn = solver.lib.primordial_solve_cells_device_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.POINTER(CellBatch), C.c_double, C.POINTER(SolverConfig),
                   C.c_void_p]
    return fn


def _run(solver, state, dtf, hint, noalloc):
    import torch
    from dengo_gb300.runtime import CellBatch, Solver
    n = len(dtf)
    st = torch.tensor(state.T.copy(), device="cuda")
    at = st * 1e-6
    d_dtf = torch.tensor(dtf, device="cuda")
    status = torch.zeros(n, dtype=torch.int32, device="cuda")
    sweeps = torch.zeros(n, dtype=torch.int32, device="cuda")
    h = torch.tensor(hint, device="cuda")
    cfg = Solver.default_config()
    stream = torch.cuda.current_stream()
    if noalloc:
        b = CellBatch(n, 1, n, st.data_ptr(), at.data_ptr(), None, 1e-6, d_dtf.data_ptr(), 0.0,
                      None, None, status.data_ptr(), None, sweeps.data_ptr(), None, h.data_ptr())
        rc = _bind(solver)(solver.data, C.byref(b), -1.0, C.byref(cfg),
                           C.c_void_p(stream.cuda_stream))
        assert rc == 0, solver.last_error()
    else:
        solver.solve_device(st, n, 1, n, at, dtf=d_dtf, status=status, sweeps=sweeps,
                            config=cfg, stream=stream, cost_hint=h)
    torch.cuda.synchronize()
    return st.cpu().numpy(), at.cpu().numpy(), status.cpu().numpy(), sweeps.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(solver):
    from dengo_gb300.workloads import primordial_cells
    for call, n in enumerate((257, 700)):
        state, dtf = primordial_cells(n, "config3", seed=900 + call)
        hint = np.random.default_rng(call).integers(0, 10**5, n).astype(np.int32)
        ref = _run(solver, state, dtf, hint, noalloc=False)
        got = _run(solver, state, dtf, hint, noalloc=True)
        for a, b in zip(got[:2], ref[:2]):
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
            rel[a == b] = 0.0
            assert rel.max() <= RTOL
        assert np.array_equal(got[2], ref[2]) and np.array_equal(got[3], ref[3])


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
