"""Admission and scheduling of the PCA server, on the CPU (a stand-in solve).

The scheduling is host logic: first-fit admission under an HBM budget, at most
`slots` solves at once, nothing over budget ever admitted, later small
requests flowing past a large one that waits for memory.
"""
import threading
import time

import numpy as np
import pytest

from brisc_gb300.serve import PCARequest, PCAServer, footprint_bytes, percentile


def _req(n, g=100, k=5, tag=None):
    ip = np.zeros(n + 1, dtype=np.int32)
    return PCARequest(ip, np.zeros(0, np.int32), np.zeros(0, np.uint16), g,
                      np.ones(n, np.float32), num_PCs=k, tag=tag)


class _Fake:
    """Sleeps a little per request and records how much was live at once."""

    def __init__(self):
        self.lock = threading.Lock()
        self.live = 0
        self.max_live = 0

    def __call__(self, req, stream):
        with self.lock:
            self.live += 1
            self.max_live = max(self.max_live, self.live)
        time.sleep(0.3 if req.tag == "long" else 0.02 + req.num_cells * 1e-7)
        with self.lock:
            self.live -= 1
        return req.tag


def test_footprint_grows_with_size():
    a = footprint_bytes(10_000, 2000, 500_000, 100)
    b = footprint_bytes(1_000_000, 2000, 100_000_000, 100)
    assert 0 < a < b
    assert b > 100_000_000 * 8  # at least the two packed copies


def test_slots_and_budget_respected():
    fake = _Fake()
    reqs = [_req(n, tag=i) for i, n in enumerate([5000, 200000, 3000, 80000, 1000,
                                                  150000, 20000, 7000])]
    fps = [footprint_bytes(r.num_cells, r.num_genes, r.nnz, r.shape_params()[1])
           for r in reqs]
    budget = int(max(fps) * 1.5)
    with PCAServer(slots=3, hbm_budget=budget, solve_fn=fake,
                   make_stream=lambda: None) as srv:
        futs = [srv.submit(r) for r in reqs]
        res = [f.result(timeout=30) for f in futs]
    assert [r.result for r in res] == list(range(len(reqs)))
    assert all(r.error is None for r in res)
    assert srv.max_running <= 3 and fake.max_live <= 3
    assert srv.max_committed <= budget
    assert all(r.latency >= 0 for r in res)


def test_first_fit_lets_small_requests_pass():
    fake = _Fake()
    big = _req(300000, tag="big")
    smalls = [_req(2000, tag=f"s{i}") for i in range(4)]
    fp_big = footprint_bytes(big.num_cells, 100, 0, 10)
    fp_first = footprint_bytes(250000, 100, 0, 10)
    fp_small = footprint_bytes(2000, 100, 0, 10)
    # room for the first request and every small one, not for first + big
    budget = fp_first + 4 * fp_small + (1 << 20)
    assert fp_first + fp_big > budget and fp_big <= budget
    with PCAServer(slots=4, hbm_budget=budget, solve_fn=fake,
                   make_stream=lambda: None) as srv:
        first = srv.submit(_req(250000, tag="first"))  # holds most of the budget
        time.sleep(0.005)
        fb = srv.submit(big)
        fs = [srv.submit(s) for s in smalls]
        for f in [first, fb, *fs]:
            assert f.result(timeout=30).error is None
    order = srv.start_order
    # the big request waits for memory; the small ones start before it
    assert order.index("big") > max(order.index(f"s{i}") for i in range(4))


def test_oversize_request_rejected():
    with PCAServer(slots=2, hbm_budget=1 << 20, solve_fn=_Fake(),
                   make_stream=lambda: None) as srv:
        r = srv.submit(_req(100000)).result(timeout=10)
    assert isinstance(r.error, MemoryError)


def test_percentile():
    assert percentile([1, 2, 3, 4], 50) == pytest.approx(2.5)
    assert np.isnan(percentile([], 99))


def test_oldest_request_stops_being_overtaken_after_max_wait():
    """A large request waiting for memory is overtaken by small ones only for
    max_wait seconds; after that nothing else starts until it fits."""
    fake = _Fake()
    big = _req(300000, tag="big")
    fp_big = footprint_bytes(big.num_cells, 100, 0, 10)
    fp_first = footprint_bytes(250000, 100, 0, 10)
    fp_small = footprint_bytes(2000, 100, 0, 10)
    budget = fp_first + 4 * fp_small + (1 << 20)
    assert fp_first + fp_big > budget and fp_big <= budget
    with PCAServer(slots=4, hbm_budget=budget, solve_fn=fake,
                   make_stream=lambda: None, max_wait=0.05) as srv:
        first = srv.submit(_req(250000, tag="long"))  # holds memory for 0.3 s
        time.sleep(0.005)
        fb = srv.submit(big)
        early = [srv.submit(_req(2000, tag=f"e{i}")) for i in range(2)]
        time.sleep(0.1)  # past max_wait: the big request is now the oldest waiting
        late = [srv.submit(_req(2000, tag=f"l{i}")) for i in range(3)]
        for f in [first, fb, *early, *late]:
            assert f.result(timeout=30).error is None
    order = srv.start_order
    # the early small requests overtook the waiting big one; the late ones,
    # which would fit beside the long request, did not
    assert max(order.index(f"e{i}") for i in range(2)) < order.index("big")
    assert order.index("big") < min(order.index(f"l{i}") for i in range(3))


def test_requeue_after_allocation_failure():
    """A solve that runs out of device memory goes back to the queue with a
    larger footprint and succeeds on the retry; one that keeps failing is
    returned as an error after max_retries."""
    from brisc_gb300._lib import ERR_ALLOC, BriscGPUError
    attempts = {}

    def flaky(req, stream):
        attempts[req.tag] = attempts.get(req.tag, 0) + 1
        if req.tag == "always" or (req.tag == "once" and attempts[req.tag] == 1):
            raise BriscGPUError(ERR_ALLOC, "bgpu_irlba", "cudaMalloc failed")
        return req.tag

    with PCAServer(slots=2, hbm_budget=1 << 40, solve_fn=flaky,
                   make_stream=lambda: None, max_retries=2) as srv:
        ok = srv.submit(_req(5000, tag="once")).result(timeout=30)
        bad = srv.submit(_req(5000, tag="always")).result(timeout=30)
    assert ok.error is None and ok.result == "once" and attempts["once"] == 2
    assert isinstance(bad.error, BriscGPUError) and attempts["always"] == 3
    assert srv.requeued == 1 + 2
