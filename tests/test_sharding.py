"""Multi-rank path on CPU: two gloo ranks each solve their shard of cells
(with the oracle standing in for the GPU solver, which needs no rank
coordination), and the gathered result equals the single-process run."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shard_range_partitions():
    from dengo_gb300.sharding import shard_range
    for n in (0, 1, 7, 64, 1001):
        for w in (1, 2, 3, 8):
            spans = [shard_range(n, r, w) for r in range(w)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from dengo_gb300.sharding import gather_cells, shard_range
    from dengo_gb300.workloads import primordial_cells
    from dengo_gb300.tablefile import read_table_file
    from oracle import Oracle
    import json
    state, dtf = primordial_cells(24, "cold", seed=5)
    a, b = shard_range(len(dtf), rank, world)
    with open(os.path.join(ROOT, "tests", "golden", "primordial_expressions.json")) as f:
        order = json.load(f)["tables"]
    tabs = read_table_file(os.path.join(ROOT, "dengo_gb300", "generated", "primordial",
                                        "primordial_tables.dgt"))
    r = Oracle("primordial").evolve_cells([tabs[k] for k in order], state[a:b], dtf[a:b],
                                          nthreads=1)
    full = gather_cells(r["state"], world)
    if rank == 0:
        np.save(out, full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_matches_single(tmp_path):
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = str(tmp_path / "full.npy")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    full = np.load(out)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from dengo_gb300.workloads import primordial_cells
    from dengo_gb300.tablefile import read_table_file
    from oracle import Oracle
    import json
    state, dtf = primordial_cells(24, "cold", seed=5)
    with open(os.path.join(ROOT, "tests", "golden", "primordial_expressions.json")) as f:
        order = json.load(f)["tables"]
    tabs = read_table_file(os.path.join(ROOT, "dengo_gb300", "generated", "primordial",
                                        "primordial_tables.dgt"))
    single = Oracle("primordial").evolve_cells([tabs[k] for k in order], state, dtf)
    assert np.array_equal(full, single["state"])
