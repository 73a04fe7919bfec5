"""Batched per-subset PCAs over one shared count matrix.

The common single-cell pattern is to PCA each cell type again on its own
(subclustering): one shared cells x genes matrix, a partition of its cells,
and one IRLBA solve per part, each with its own gene centring and scaling
(``SingleCell.pca()`` run on a subset, brisc/single_cell.py:11800-11808).

Here the shared matrix stays resident on the GPU. Each subset's layout is
gathered from it on the device (``bgpu_matrix_create_rows``). The solves run
concurrently: worker threads each own a CUDA stream and take the next subset,
largest first. Every solve's kernels are deterministic and independent of
what else runs, so a subset's PCs are bit-identical whether it runs alone,
sequentially or in the batch (the tests check this).
"""
from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

from .pca import DeviceMatrix, SolveResult

_METHODS = ("logCP10k", "log1pPF", "PFlog1pPF")


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
                            stream=stream, rows=r)


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
                reorth_passes: int | str = "auto") -> list[SubsetResult]:
    """One IRLBA PCA per row subset of `shared`, `concurrency` at a time.

    `subsets` is a sequence of int64 row-index arrays. Returns one
    SubsetResult per subset, in the input order.
    """
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
