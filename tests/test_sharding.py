"""Multi-rank path on CPU: two gloo ranks each solve their shard of cells
with the product's own engine -- the default split engine's CUDA source
compiled for the host (tests/host_engine.py), the GPU being absent here --
and the gathered result equals a one-rank run bit for bit.  Cells are
independent, so no rank waits on another's data; the only collectives are
the gather and the barrier."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_range_partitions():
    from dengo_gb300.sharding import shard_range
    for n in (0, 1, 7, 64, 1001):
        for w in (1, 2, 3, 8):
            spans = [shard_range(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1


def _tables():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    return Oracle("primordial").tables_from_bundle(
        os.path.join(ROOT, "dengo_gb300", "generated", "primordial", "primordial_tables.dgt"))


def _cells():
    from dengo_gb300.workloads import primordial_cells
    a, da = primordial_cells(20, "cold", seed=5)
    b, db = primordial_cells(4, "config3", seed=6)
    return np.concatenate([a, b]), np.concatenate([da, db])


def _worker(rank, world, port, so, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import host_engine as he
    from dengo_gb300.sharding import gather_cells, shard_range
    state, dtf = _cells()
    a, b = shard_range(len(dtf), rank, world)
    r = he.evolve_in_subprocess(so, _tables(), state[a:b], dtf[a:b], mixed=True,
                                sweep_budget=500, cons_tol=1e-9)
    full = gather_cells(np.concatenate([r["state"], r["sweeps"][:, None].astype(float)], axis=1),
                        world)
    if rank == 0:
        np.save(out, full)
    dist.barrier()
    dist.destroy_process_group()


@pytest.fixture(scope="module")
def split_so(tmp_path_factory):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import host_engine as he
    return he.compile_engine("primordial", tmp_path_factory.mktemp("shard"), engine="split")


def test_two_rank_gloo_matches_single(tmp_path, split_so):
    import socket
    import torch.multiprocessing as mp
    import host_engine as he
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = str(tmp_path / "full.npy")
    mp.start_processes(_worker, args=(2, port, split_so, out), nprocs=2, join=True,
                       start_method="spawn")
    full = np.load(out)
    state, dtf = _cells()
    single = he.evolve_in_subprocess(split_so, _tables(), state, dtf, mixed=True,
                                     sweep_budget=500, cons_tol=1e-9)
    assert np.array_equal(full[:, :-1], single["state"])
    assert np.array_equal(full[:, -1], single["sweeps"].astype(float))
