"""Serving loop: admission/batching logic on the CPU, and on the GPU the
alone-vs-mix equality and the loop's accounting."""
import numpy as np
import pytest

from dengo_gb300.serving import Request, request_bytes, select_group


def _req(net, n, rid, steps=1, nsp=10):
    return Request(net, np.zeros((n, nsp)), 1e10, steps=steps, rid=rid)


def test_group_is_fifo_headed_and_single_network():
    pend = [_req("primordial", 100, 0), _req("oxygen", 50, 1, nsp=16), _req("primordial", 10, 2),
            _req("primordial", 5, 3, steps=2)]
    g = select_group(pend, 0, 1 << 30, 1 << 20)
    assert [r.rid for r in g] == [0, 2]


def test_group_respects_budget_and_size():
    pend = [_req("primordial", 100, 0), _req("primordial", 100, 1), _req("primordial", 10, 2)]
    per = request_bytes(pend[0])
    # room for the head and the small one only
    g = select_group(pend, 0, per + request_bytes(pend[2]), 1 << 20)
    assert [r.rid for r in g] == [0, 2]
    # size cap
    g = select_group(pend, 0, 1 << 30, 150)
    assert [r.rid for r in g] == [0, 2]
    # the head does not fit: nothing is admitted (the head is not overtaken)
    assert select_group(pend, 1 << 30, 1 << 30, 1 << 20) == []
    assert select_group([], 0, 1 << 30, 1 << 20) == []


def test_request_bytes_counts_state_tolerances_and_counters():
    r = _req("oxygen", 7, 0, nsp=16)
    assert request_bytes(r) == 7 * (2 * 16 * 8 + 8 + 4 + 4)


def test_poisson_schedule_is_seeded():
    from dengo_gb300.serving import poisson_requests
    a = poisson_requests(200, 0.05, edge_range=(4, 8), seed=3)
    b = poisson_requests(200, 0.05, edge_range=(4, 8), seed=3)
    assert [(r.network, r.ncells, r.dtf, r.arrival) for r in a] == \
        [(r.network, r.ncells, r.dtf, r.arrival) for r in b]
    assert all(np.all(x.state == y.state) for x, y in zip(a, b))
    assert all(r.state.shape[1] == (10 if r.network == "primordial" else 16) for r in a)


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from dengo_gb300.build import build_network, library_path
    import os
    for n in ("primordial", "oxygen"):
        if not os.path.exists(library_path(n)):
            build_network(n)
    return torch


@pytest.mark.gpu
def test_result_is_the_same_alone_and_in_the_mix(gpu):
    """A request's result, solved alone, equals (bit for bit, FP64 path) its
    result when it shares launch groups and the device with other requests of
    both networks admitted while it runs."""
    from dengo_gb300.serving import ServingLoop, poisson_requests
    reqs = poisson_requests(2000, 0.02, edge_range=(6, 14), seed=11)
    assert len(reqs) >= 20 and {r.network for r in reqs} == {"primordial", "oxygen"}
    loop = ServingLoop(slots=3, hbm_budget=64 << 20, max_group_cells=4096)
    stats = loop.run(reqs, timeout=900)
    assert stats["requests"] == len(reqs) and loop.used == 0
    assert loop.launches < len(reqs)            # some requests shared a launch
    for r in reqs[:: max(1, len(reqs) // 6)]:
        alone = Request(r.network, r.state, r.dtf, steps=r.steps, rid=r.rid)
        solo = ServingLoop(networks=(r.network,), slots=1)
        solo.run([alone], timeout=900)
        assert np.array_equal(alone.result.view(np.int64), r.result.view(np.int64)), r.rid
        assert np.array_equal(alone.status, r.status)


@pytest.mark.gpu
def test_budget_bounds_resident_bytes(gpu):
    from dengo_gb300.serving import ServingLoop, poisson_requests
    reqs = poisson_requests(5000, 0.01, edge_range=(8, 12), seed=12)
    budget = 3 * max(request_bytes(r) for r in reqs)
    loop = ServingLoop(slots=4, hbm_budget=budget, max_group_cells=1 << 20)
    peak = [0]
    orig = loop._launch

    def spy(slot, g):
        orig(slot, g)
        peak[0] = max(peak[0], loop.used)
    loop._launch = spy
    loop.run(reqs, timeout=900)
    assert 0 < peak[0] <= budget and loop.used == 0
    assert all(r.result is not None for r in reqs)


def test_requests_compare_by_identity():
    import collections
    a, b = _req("primordial", 3, 0), _req("primordial", 5, 1)
    q = collections.deque([a, b])
    q.remove(b)
    assert list(q) == [a] and a != _req("primordial", 3, 0)
