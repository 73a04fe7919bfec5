"""Batched per-subset PCAs over one shared count matrix.

The common single-cell pattern is to PCA each cell type again on its own
(subclustering): one shared cells x genes matrix, a partition of its cells,
and one IRLBA solve per part, each with its own gene centring and scaling
(``SingleCell.pca()`` run on a subset, brisc/single_cell.py:11800-11808).

Here the shared matrix stays resident on the GPU. Each subset's layout is
gathered from it on the device (``bgpu_matrix_create_rows``, by worker
threads on streams of their own). Then, by default, all the solves run in
lock step (``bgpu_irlba_batch``): each kernel of a Lanczos step is one launch
over every subset that is stepping, and each subset restarts on a stream of
its own meanwhile, so a step costs ten launches whatever the number of
subsets. ``mode="streams"`` instead runs independent solves, ``concurrency``
at a time on their own streams. Every solve's kernels compute the same
arithmetic in either mode, so a subset's PCs are bit-identical whether it
runs alone, sequentially or in the batch (the tests check this).
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .pca import DeviceMatrix, SolveResult, reorth_code

_METHODS = ("logCP10k", "log1pPF", "PFlog1pPF")
# X^T.u panel rows of the subsets' layouts: the longest the sliced-ELL layout
# takes. A batch's CTAs come from every subset at once, so it needs no wave of
# CTAs per subset; longer panels give fewer, longer per-gene sums and fewer
# partials. A subset solved alone on a layout with these panel rows gives
# the same bits.
SUBSET_PANEL_ROWS = 512


@dataclass
class SubsetResult:
    rows: int
    result: SolveResult
    seconds: float


def subset_solve_params(num_rows: int, num_genes: int, num_PCs: int,
                        subspace_size: int | None) -> tuple[int, int]:
    """(k, m) for one subset: m = 2k by default, both clipped to the subset's
    shape as pca() clips them (brisc/single_cell.py:11958)."""
    m = 2 * num_PCs if subspace_size is None else int(subspace_size)
    m = min(m, num_rows, num_genes)
    k = min(num_PCs, m)
    return k, m


class SharedMatrix:
    """A count matrix resident on the GPU, from which subsets are solved."""

    def __init__(self, indptr, indices, counts, num_cells: int, num_genes: int,
                 *, inv_size_factors, post_factors=None, method: str = "logCP10k",
                 device=None):
        import torch
        if method not in _METHODS:
            raise ValueError(f"method must be one of {_METHODS}")
        if (method == "PFlog1pPF") != (post_factors is not None):
            raise ValueError("post_factors are required for (and only for) PFlog1pPF")
        self.device = torch.device("cuda") if device is None else torch.device(device)

        def up(a, dt):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(self.device)

        itype = np.int64 if np.asarray(indptr)[-1] >= 2 ** 31 else np.int32
        self.indptr = up(indptr, itype)
        self.indices = up(indices, itype)
        c = np.ascontiguousarray(counts)
        self.counts = up(c.view(np.int16) if c.dtype == np.uint16 else c, c.dtype
                         if c.dtype != np.uint16 else np.int16)
        self._value_view = np.uint16 if c.dtype == np.uint16 else c.dtype
        self.isf = up(inv_size_factors, np.float32)
        self.post = up(post_factors, np.float32) if post_factors is not None else None
        self.num_cells, self.num_genes = int(num_cells), int(num_genes)
        self.method = method
        torch.cuda.synchronize(self.device)

    def subset(self, rows, stream=None) -> DeviceMatrix:
        import torch
        r = torch.as_tensor(np.ascontiguousarray(rows, dtype=np.int64)).to(
            self.device, non_blocking=False)
        vals = self.counts if self._value_view != np.uint16 else _U16View(self.counts)
        return DeviceMatrix(self.indptr, self.indices, vals, self.num_cells,
                            self.num_genes, norm=self.method,
                            inv_size_factors=self.isf, post_factors=self.post,
                            stream=stream, rows=r, sell_panel_rows=SUBSET_PANEL_ROWS)


class _U16View:
    """A CUDA int16 tensor presented to DeviceMatrix as uint16 counts."""

    def __init__(self, t):
        self._t = t
        self.shape = t.shape
        self.dtype = "torch.uint16"

    def data_ptr(self) -> int:
        return self._t.data_ptr()


def pca_subsets(shared: SharedMatrix, subsets, *, num_PCs: int = 30,
                subspace_size: int | None = None, tolerance: float = 1e-6,
                max_iterations: int = 100, seed: int = 0, concurrency: int = 8,
                reorth_passes: int | str = "auto", mode: str = "auto",
                info: dict | None = None) -> list[SubsetResult]:
    """One IRLBA PCA per row subset of `shared`.

    `subsets` is a sequence of int64 row-index arrays. Returns one
    SubsetResult per subset, in the input order. ``mode``: "fused" (all
    solves in lock step, one launch per step kernel over all subsets),
    "streams" (independent solves, `concurrency` at a time) or "auto" (fused
    where every subset's layout and options allow it: sliced-ELL layout,
    adaptive `reorth_passes`). `concurrency` threads build the subsets'
    layouts in either mode. `info`, if given, receives the mode run and, for
    a fused batch, its kernel launches.
    """
    if mode not in ("auto", "fused", "streams"):
        raise ValueError("mode must be 'auto', 'fused' or 'streams'")
    if mode != "streams":
        out = _pca_fused(shared, subsets, num_PCs=num_PCs, subspace_size=subspace_size,
                         tolerance=tolerance, max_iterations=max_iterations, seed=seed,
                         concurrency=concurrency, reorth_passes=reorth_passes,
                         required=mode == "fused", info=info)
        if out is not None:
            return out
    if info is not None:
        info["mode"] = "streams"
    return _pca_streams(shared, subsets, num_PCs=num_PCs, subspace_size=subspace_size,
                        tolerance=tolerance, max_iterations=max_iterations, seed=seed,
                        concurrency=concurrency, reorth_passes=reorth_passes)


def _pca_fused(shared: SharedMatrix, subsets, *, num_PCs, subspace_size, tolerance,
               max_iterations, seed, concurrency, reorth_passes, required,
               info) -> list[SubsetResult] | None:
    """The lock-step batch; None (nothing solved) when a subset cannot take
    part and the caller allowed the streams mode instead."""
    import torch
    t0 = time.perf_counter()
    count = len(subsets)
    rows = [np.asarray(r, dtype=np.int64) for r in subsets]
    params = [subset_solve_params(r.shape[0], shared.num_genes, num_PCs, subspace_size)
              for r in rows]
    mats: list[DeviceMatrix | None] = [None] * count
    local = threading.local()

    def build(i: int) -> None:
        if not hasattr(local, "stream"):
            local.stream = torch.cuda.Stream(device=shared.device)
        with torch.cuda.stream(local.stream):
            mats[i] = shared.subset(rows[i], stream=local.stream)
        local.stream.synchronize()

    order = sorted(range(count), key=lambda i: -len(rows[i]))
    try:
        if concurrency <= 1:
            for i in order:
                build(i)
        else:
            with ThreadPoolExecutor(max_workers=concurrency) as ex:
                for f in [ex.submit(build, i) for i in order]:
                    f.result()
        t_build = time.perf_counter() - t0
        opts = (L.SolveOpts * count)()
        pcs, svs = [], []
        for i, (k, m) in enumerate(params):
            o = opts[i]
            L.lib().bgpu_solve_opts_default(C.byref(o))
            o.k, o.subspace_size = k, m
            o.tolerance, o.max_iterations = float(tolerance), int(max_iterations)
            o.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
            o.reorth_passes = reorth_code(reorth_passes)
            pcs.append(np.empty((rows[i].shape[0], k), dtype=np.float32))
            svs.append(np.empty(k, dtype=np.float32))
        handles = (C.c_void_p * count)(*[M.handle for M in mats])
        pptr = (C.c_void_p * count)(*[p.ctypes.data for p in pcs])
        sptr = (C.c_void_p * count)(*[v.ctypes.data for v in svs])
        infos = (L.SolveInfo * count)()
        launches = C.c_uint64(0)
        stream = torch.cuda.current_stream(shared.device)
        code = L.lib().bgpu_irlba_batch(handles, opts, count, pptr, 0, sptr, infos,
                                        C.byref(launches), C.c_void_p(stream.cuda_stream))
        if code == L.ERR_UNSUPPORTED and not required:
            return None
        L.check(code, "bgpu_irlba_batch")
    finally:
        for M in mats:
            if M is not None:
                M.close()
    if info is not None:
        info.update(mode="fused", kernel_launches=int(launches.value),
                    build_seconds=t_build)
    out = []
    for i in range(count):
        d = infos[i].as_dict()
        out.append(SubsetResult(rows[i].shape[0],
                                SolveResult(pcs[i], svs[i], None, bool(d["converged"]), d),
                                d["seconds"]))
    return out


def _pca_streams(shared: SharedMatrix, subsets, *, num_PCs, subspace_size, tolerance,
                 max_iterations, seed, concurrency, reorth_passes) -> list[SubsetResult]:
    import torch
    order = sorted(range(len(subsets)), key=lambda i: -len(subsets[i]))
    out: list[SubsetResult | None] = [None] * len(subsets)
    local = threading.local()

    def run(i: int) -> None:
        if not hasattr(local, "stream"):
            local.stream = torch.cuda.Stream(device=shared.device)
        rows = np.asarray(subsets[i], dtype=np.int64)
        k, m = subset_solve_params(rows.shape[0], shared.num_genes, num_PCs,
                                   subspace_size)
        t0 = time.perf_counter()
        with torch.cuda.stream(local.stream):
            M = shared.subset(rows, stream=local.stream)
            try:
                r = M.solve(k, m, tolerance, max_iterations, seed,
                            reorth_passes=reorth_passes, stream=local.stream)
            finally:
                M.close()
        out[i] = SubsetResult(rows.shape[0], r, time.perf_counter() - t0)

    if concurrency <= 1:
        for i in order:
            run(i)
    else:
        with ThreadPoolExecutor(max_workers=concurrency) as ex:
            for f in [ex.submit(run, i) for i in order]:
                f.result()
    return out  # type: ignore[return-value]
