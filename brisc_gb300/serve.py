"""A PCA request server: continuous batching of IRLBA solves on one GPU.

Requests (a count matrix on the host plus solve parameters) arrive at any
time. A dispatcher admits them in arrival order, first fit: the first waiting
request whose estimated device footprint fits in the HBM budget left by the
running ones starts as soon as a slot is free, so small requests flow past a
large one that is waiting for memory. Past `max_wait` seconds of waiting the
oldest request stops being overtaken: nothing else starts until it fits, so a
steady stream of small requests cannot starve a large one. Each slot is a
host thread with its own CUDA stream; it uploads the request, builds its
device layout, solves and returns the PCs. Requests that arrive while others
run overlap with them on the device. A solve that fails to allocate device
memory (the footprint model under-estimated it, or memory outside the server
is in use) goes back to the head of the queue with a larger footprint, up to
`max_retries` times.

Every solve is deterministic and independent of what else runs, so a
request's result is bit-identical alone and in the mix (the tests check this).
"""
from __future__ import annotations

import threading
import time
from concurrent.futures import Future, ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from .pca import DeviceMatrix, SolveResult


@dataclass
class PCARequest:
    indptr: np.ndarray           # int32/int64, num_cells + 1
    indices: np.ndarray          # same type, nnz gene indices
    counts: np.ndarray           # uint16 counts, nnz
    num_genes: int
    inv_size_factors: np.ndarray  # float32, num_cells
    num_PCs: int = 50
    subspace_size: int | None = None
    tolerance: float = 1e-6
    max_iterations: int = 100
    seed: int = 0
    method: str = "logCP10k"
    post_factors: np.ndarray | None = None
    tag: object = None

    @property
    def num_cells(self) -> int:
        return int(self.indptr.shape[0]) - 1

    @property
    def nnz(self) -> int:
        return int(self.counts.shape[0])

    def shape_params(self) -> tuple[int, int]:
        m = 2 * self.num_PCs if self.subspace_size is None else int(self.subspace_size)
        m = min(m, self.num_cells, self.num_genes)
        return min(self.num_PCs, m), m


def footprint_bytes(num_cells: int, num_genes: int, nnz: int, m: int) -> int:
    """Device bytes one request holds at its peak (with 10 % margin): the
    staged inputs and build temporaries of the sliced-ELL layout (packed CSR
    words, per-panel segment tables), the resident layout (2-byte entries of
    both copies with their padding, per-row and per-segment descriptors) and
    the solver state (two n x m and two g x m bases, partials)."""
    n, g = int(num_cells), int(num_genes)
    panels = (n + 511) // 512 + 1
    ld_n = (n + 63) // 64 * 64
    build = nnz * (6 + 4) + (n + 1) * 8 + n * 8 + panels * g * 12
    layout = int(nnz * 2 * 2.4) + n * 30 + panels * g * 4 + (n + 5) * 8
    solver = 2 * ld_n * m * 4 + 2 * g * m * 4 + 2 * ld_n * 4 \
        + ((n + 255) // 256) * (m + 2) * 4 + panels * g * 4 * 5 + n * m * 4 \
        + m * m * 64
    return int((build + layout + solver) * 1.1) + (16 << 20)


@dataclass
class PCAResponse:
    result: SolveResult | None
    error: BaseException | None
    arrival: float
    start: float
    finish: float
    footprint: int

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


@dataclass
class _Pending:
    req: PCARequest
    fut: Future
    arrival: float
    footprint: int
    retries: int = 0


def _out_of_memory(e: BaseException) -> bool:
    """A device allocation failure of the library (BGPU_ERR_ALLOC) or of torch."""
    from ._lib import ERR_ALLOC, BriscGPUError
    if isinstance(e, BriscGPUError) and e.code == ERR_ALLOC:
        return True
    try:
        import torch
        return isinstance(e, torch.cuda.OutOfMemoryError)
    except (ImportError, AttributeError):  # pragma: no cover
        return False


def gpu_solve(req: PCARequest, stream) -> SolveResult:
    """Upload, lay out and solve one request on `stream` (the default slot work)."""
    import torch
    k, m = req.shape_params()
    with torch.cuda.stream(stream):
        M = DeviceMatrix(req.indptr, req.indices, req.counts, req.num_cells,
                         req.num_genes, norm=req.method,
                         inv_size_factors=req.inv_size_factors,
                         post_factors=req.post_factors, stream=stream)
        try:
            return M.solve(k, m, req.tolerance, req.max_iterations, req.seed,
                           stream=stream)
        finally:
            M.close()


class PCAServer:
    """Continuous-batching PCA server.

    slots: solves that may run at once. hbm_budget: device bytes the running
    solves may hold together (default: 80 % of the free memory at start).
    max_wait: seconds after which the oldest waiting request is no longer
    overtaken (None: pure first fit). max_retries: how often a request whose
    solve ran out of device memory is queued again. solve_fn(request,
    stream) -> SolveResult does the work (default: the GPU solve);
    make_stream() gives each slot its stream.
    """

    def __init__(self, slots: int = 8, hbm_budget: int | None = None,
                 solve_fn: Callable | None = None,
                 make_stream: Callable | None = None,
                 max_wait: float | None = 10.0, max_retries: int = 3):
        if slots < 1:
            raise ValueError("slots must be >= 1")
        self.max_wait = max_wait
        self.max_retries = int(max_retries)
        self.requeued = 0
        if hbm_budget is None:
            import torch
            hbm_budget = int(torch.cuda.mem_get_info()[0] * 0.8)
        self.slots = slots
        self.budget = int(hbm_budget)
        self._solve = solve_fn or gpu_solve
        if make_stream is None:
            def make_stream():
                import torch
                return torch.cuda.Stream()
        self._make_stream = make_stream
        self._pending: list[_Pending] = []
        self._cv = threading.Condition()
        self._committed = 0
        self._running = 0
        self._closing = False
        self.max_committed = 0
        self.max_running = 0
        self.start_order: list[object] = []
        self._local = threading.local()
        self._pool = ThreadPoolExecutor(max_workers=slots)
        self._dispatcher = threading.Thread(target=self._dispatch, daemon=True)
        self._dispatcher.start()

    def submit(self, req: PCARequest, arrival: float | None = None) -> Future:
        """Queue a request; the future resolves to a PCAResponse."""
        k, m = req.shape_params()
        fp = footprint_bytes(req.num_cells, req.num_genes, req.nnz, m)
        fut: Future = Future()
        arrival = time.perf_counter() if arrival is None else arrival
        if fp > self.budget:
            fut.set_result(PCAResponse(None, MemoryError(
                f"request needs ~{fp:,} device bytes, over the budget of "
                f"{self.budget:,}"), arrival, arrival, arrival, fp))
            return fut
        with self._cv:
            if self._closing:
                raise RuntimeError("server is closed")
            self._pending.append(_Pending(req, fut, arrival, fp))
            self._cv.notify_all()
        return fut

    def close(self, wait: bool = True) -> None:
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        if wait:
            self._dispatcher.join()
            self._pool.shutdown(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- internals ---------------------------------------------------------
    def _pick(self) -> _Pending | None:
        if self._running >= self.slots or not self._pending:
            return None
        room = self.budget - self._committed
        head = min(self._pending, key=lambda p: p.arrival)
        if self.max_wait is not None and \
                time.perf_counter() - head.arrival > self.max_wait:
            # the oldest request has waited long enough: it goes next
            if head.footprint <= room:
                self._pending.remove(head)
                return head
            return None
        for i, p in enumerate(self._pending):
            if p.footprint <= room:
                return self._pending.pop(i)
        return None

    def _dispatch(self) -> None:
        while True:
            with self._cv:
                while True:
                    p = self._pick()
                    if p is not None:
                        break
                    if self._closing and not self._pending and self._running == 0:
                        return
                    # wake up to re-check the waiting time of the oldest request
                    self._cv.wait(timeout=0.05 if self._pending else None)
                self._committed += p.footprint
                self._running += 1
                self.max_committed = max(self.max_committed, self._committed)
                self.max_running = max(self.max_running, self._running)
                self.start_order.append(p.req.tag)
            self._pool.submit(self._work, p)

    def _work(self, p: _Pending) -> None:
        if not hasattr(self._local, "stream"):
            self._local.stream = self._make_stream()
        start = time.perf_counter()
        res, err = None, None
        try:
            res = self._solve(p.req, self._local.stream)
        except BaseException as e:  # noqa: BLE001 - returned to the caller
            err = e
        finish = time.perf_counter()
        retry = (err is not None and _out_of_memory(err)
                 and p.retries < self.max_retries)
        with self._cv:
            self._committed -= p.footprint
            self._running -= 1
            if retry:  # back to the queue, oldest first, with a larger estimate
                p.retries += 1
                p.footprint = min(int(p.footprint * 1.5), self.budget)
                self._pending.insert(0, p)
                self.requeued += 1
            self._cv.notify_all()
        if not retry:
            p.fut.set_result(PCAResponse(res, err, p.arrival, start, finish,
                                         p.footprint))


def percentile(xs, q: float) -> float:
    a = np.sort(np.asarray(xs, dtype=np.float64))
    if a.size == 0:
        return float("nan")
    return float(np.percentile(a, q))
