"""Partitioning cells across ranks (one process per GPU).

Cells are independent -- no term of the RHS, Jacobian or dt control couples
two cells -- so a multi-GPU run is a set of replicas: rank r solves the
contiguous cell range ``shard_range(n, r, world)`` and nothing is exchanged
on the data path.  The only collectives are the timing barrier and the
max-over-ranks of the elapsed time (and an optional gather of results on
the host).
"""


def shard_range(ncells, rank, world):
    """[start, stop) of rank's cells: contiguous, sizes differ by at most 1."""
    if not 0 <= rank < world:
        raise ValueError("rank %d outside world %d" % (rank, world))
    base, extra = divmod(ncells, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def gather_cells(local, world, group=None):
    """All-gather per-rank numpy arrays (cells first) into one array in rank
    order, through torch.distributed (any backend)."""
    import numpy as np
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(local))
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([t.shape[0]], dtype=torch.int64), group=group)
    m = int(max(s.item() for s in sizes))
    pad = torch.zeros((m,) + tuple(t.shape[1:]), dtype=t.dtype)
    pad[:t.shape[0]] = t
    out = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(out, pad, group=group)
    return np.concatenate([o[:int(s.item())].numpy() for o, s in zip(out, sizes)])
