"""Host-side mirror of brisc's PCA interface, running on the GPU.

* :func:`irlba` has exactly the keyword signature and meaning of the
  reference's Cython ``irlba`` (brisc/pca.pyx:661-678): it can be bound in
  place of ``brisc.single_cell.irlba`` (see :func:`install`) so that an
  installed brisc's ``SingleCell.pca()`` runs on the GPU unchanged.
* :func:`pca` restates ``SingleCell.pca()`` (brisc/single_cell.py:11625-12137)
  for plain scipy sparse matrices and boolean masks: the same arguments,
  validation messages, QC/HVG subsetting, joint PCA over several datasets,
  subspace clipping and NaN back-fill of cells that failed QC.
* :func:`pca_counts` is the fused form: raw integer counts plus the
  normalisation method of ``SingleCell.normalize()``
  (brisc/single_cell.py:11450-11623); the normalisation is never
  materialised, it is applied inside every sparse product.
* :class:`DeviceMatrix` keeps one matrix resident on the GPU for repeated
  solves.

There is no CPU path: every call goes through ``libbriscgpu.so``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib as L

_INDEX_TYPES = {np.dtype(np.int32): L.INDEX_I32, np.dtype(np.int64): L.INDEX_I64}
_VALUE_TYPES = {np.dtype(np.uint16): L.VALUE_U16, np.dtype(np.uint32): L.VALUE_U32,
                np.dtype(np.int32): L.VALUE_I32, np.dtype(np.float32): L.VALUE_F32}
_METHODS = {"logCP10k": 0, "log1pPF": 1, "PFlog1pPF": 2}


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())  # torch tensor


def _stream(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available() and torch.cuda.is_initialized():
                return int(torch.cuda.current_stream().cuda_stream)
        except ImportError:  # pragma: no cover - torch is optional here
            pass
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def _check_vec(a, name: str, dtype, length=None, writeable=False):
    if not isinstance(a, np.ndarray):
        raise TypeError(f"{name} must be a NumPy array, but has type "
                        f"{type(a).__name__!r}")
    if a.dtype != dtype:
        raise TypeError(f"{name} must have data type {np.dtype(dtype).name!r}, "
                        f"but has data type {a.dtype.name!r}")
    if not a.flags.c_contiguous:
        raise ValueError(f"{name} must be C-contiguous")
    if length is not None and a.shape[0] != length:
        raise ValueError(f"{name} has length {a.shape[0]:,}, expected {length:,}")
    if writeable and not a.flags.writeable:
        raise ValueError(f"{name} must be writeable")


# ---------------------------------------------------------------------------
def irlba(data_matvec, indices_matvec, indptr_matvec, data_rmatvec,
          indices_rmatvec, indptr_rmatvec, num_cells, num_genes, k,
          subspace_size, tolerance, max_iterations, seed, match_parallel,
          is_csr, num_threads, chunk_size, PCs) -> bool:
    """GPU drop-in for ``brisc.pca.irlba`` (brisc/pca.pyx:661-678).

    Arguments and their meaning are the reference's: ``data_*`` float32
    normalised values, ``indices_*``/``indptr_*`` one shared signed integer
    type (int32 or int64), CSR arrays for the matvec and CSC arrays for the
    rmatvec, ``PCs`` a preallocated C-contiguous float32 (num_cells, k) array
    filled in place. Returns whether IRLBA converged. The CSC arrays are
    accepted for compatibility; the GPU builds its own transposed copy.
    ``chunk_size`` sets the reference's reduction blocks (pca.pyx:1006-1010),
    which change only the rounding of its sums; the GPU sums over fixed
    1024-row blocks whatever it is, and warns when it is not 1024.
    """
    num_cells, num_genes, k = int(num_cells), int(num_genes), int(k)
    if int(chunk_size) != 1024:
        import warnings
        warnings.warn(f"chunk_size={int(chunk_size)}: the GPU solve reduces over fixed "
                      "1024-row blocks (the value only changes the reference's "
                      "rounding)", RuntimeWarning, stacklevel=2)
    _check_vec(data_matvec, "data_matvec", np.float32)
    idx_t = indices_matvec.dtype
    if idx_t not in _INDEX_TYPES:
        raise TypeError("indices must be int32 or int64 (signed_integer)")
    for name, a in (("indices_matvec", indices_matvec),
                    ("indptr_matvec", indptr_matvec)):
        _check_vec(a, name, idx_t)
    if not isinstance(PCs, np.ndarray) or PCs.dtype != np.float32 or \
            not PCs.flags.c_contiguous or PCs.shape != (num_cells, k):
        raise ValueError(f"PCs must be a C-contiguous float32 array of shape "
                         f"({num_cells}, {k})")
    conv = C.c_int(0)
    L.call("bgpu_irlba_f32", _ptr(data_matvec), _ptr(indices_matvec),
           _ptr(indptr_matvec), _ptr(data_rmatvec), _ptr(indices_rmatvec),
           _ptr(indptr_rmatvec), _INDEX_TYPES[idx_t], num_cells, num_genes,
           k, int(subspace_size), float(tolerance), int(max_iterations),
           int(seed) & 0xFFFFFFFFFFFFFFFF, int(bool(match_parallel)),
           int(bool(is_csr)), int(num_threads), int(chunk_size),
           _ptr(PCs), C.byref(conv))
    return bool(conv.value)


def install(module=None):
    """Bind :func:`irlba` into brisc's ``single_cell`` module (the name its
    ``pca()`` calls, brisc/single_cell.py:12082). Returns the previous binding."""
    if module is None:
        import brisc.single_cell as module  # pragma: no cover
    previous = getattr(module, "irlba", None)
    module.irlba = irlba
    return previous


# ---------------------------------------------------------------------------
@dataclass
class SolveResult:
    PCs: np.ndarray
    singular_values: np.ndarray
    loadings: np.ndarray | None
    converged: bool
    info: dict


class DeviceMatrix:
    """A cells x genes matrix resident on the GPU in the solver's layout.

    ``indptr``/``indices``/``values`` are NumPy arrays (copied to the device)
    or CUDA torch tensors (used in place). ``norm`` is None for already
    normalised float32 values, or one of ``'logCP10k'``, ``'log1pPF'``,
    ``'PFlog1pPF'`` for raw counts with per-cell factors.
    """

    def __init__(self, indptr, indices, values, num_cells: int,
                 num_genes: int, *, norm: str | None = None,
                 inv_size_factors=None, post_factors=None,
                 panel_rows: int = 0, stream=None, rows=None, kernels=(),
                 sell_panel_rows: int = 0):
        """``rows`` (int64 cell indices, NumPy for host inputs or a CUDA
        tensor for device inputs) selects the row subset X[rows, :]: the
        matrix is then that subset, with its own gene centring and scaling.
        ``kernels`` (names of _lib.KERNELS) forces product-kernel choices,
        for comparing layouts; the default picks them automatically.
        ``sell_panel_rows`` fixes the rows of the sliced-ELL layout's X^T.u
        panels (0 = automatic; the batched subsets use 512)."""
        on_dev = not isinstance(indptr, np.ndarray)
        idx_dt = _np_dtype(indices)
        if idx_dt != _np_dtype(indptr) or idx_dt not in _INDEX_TYPES:
            raise TypeError("indptr and indices must share int32 or int64")
        val_dt = _np_dtype(values)
        if val_dt not in _VALUE_TYPES:
            raise TypeError(f"unsupported value dtype {val_dt}")
        d = L.MatrixDesc()
        d.indptr, d.indices, d.values = _ptr(indptr), _ptr(indices), _ptr(values)
        d.index_type = _INDEX_TYPES[idx_dt]
        d.value_type = _VALUE_TYPES[val_dt]
        d.on_device = int(on_dev)
        d.num_cells, d.num_genes = int(num_cells), int(num_genes)
        d.nnz = int(values.shape[0])
        d.norm_method = L.NORM_NONE if norm is None else _METHODS[norm]
        d.inv_size_factors = _ptr(inv_size_factors)
        d.post_factors = _ptr(post_factors)
        d.panel_rows = int(panel_rows)
        d.sell_panel_rows = int(sell_panel_rows)
        d.kernels = 0
        for name in kernels:
            d.kernels |= L.KERNELS[name]
        self._keep = (indptr, indices, values, inv_size_factors, post_factors)
        h = C.c_void_p()
        if rows is None:
            L.call("bgpu_matrix_create", C.byref(h), C.byref(d), _stream(stream))
            num_cells = int(num_cells)
        else:
            if isinstance(rows, np.ndarray):
                if on_dev:
                    raise TypeError("rows must be a CUDA tensor when the arrays are")
                rows = np.ascontiguousarray(rows, dtype=np.int64)
            elif str(rows.dtype) != "torch.int64" or not on_dev:
                raise TypeError("rows must be int64, in the arrays' memory space")
            L.call("bgpu_matrix_create_rows", C.byref(h), C.byref(d), _ptr(rows),
                   int(rows.shape[0]), _stream(stream))
            num_cells = int(rows.shape[0])
        self._h = h
        self._keep = None  # the library copied what it needs
        self._stream = stream  # device memory is released on the creation stream
        self.num_cells, self.num_genes = num_cells, int(num_genes)
        self.nnz = int(d.nnz) if rows is None else None
        self.norm = norm

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise RuntimeError("DeviceMatrix was closed")
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            L.lib().bgpu_matrix_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def layout(self) -> str:
        """'sell' (sliced-ELL products), 'panels' or 'float'."""
        v = C.c_int()
        L.call("bgpu_matrix_layout", self.handle, C.byref(v))
        return {0: "panels", 1: "sell", 2: "float"}[v.value]

    def device_bytes(self) -> int:
        b = C.c_uint64()
        L.call("bgpu_matrix_bytes", self.handle, C.byref(b))
        return int(b.value)

    # raw products (device tensors; used by the parity tests)
    def matvec(self, v, sd, y, stream=None) -> None:
        L.call("bgpu_matrix_matvec", self.handle, _ptr(v), _ptr(sd), _ptr(y),
               _stream(stream))

    def rmatvec(self, u, sd, z, stream=None) -> None:
        L.call("bgpu_matrix_rmatvec", self.handle, _ptr(u), _ptr(sd), _ptr(z),
               _stream(stream))

    def gene_stddev(self, sd, stream=None) -> None:
        L.call("bgpu_matrix_gene_stddev", self.handle, _ptr(sd), _stream(stream))

    def solve(self, num_PCs: int = 50, subspace_size: int = 100,
              tolerance: float = 1e-6, max_iterations: int = 100,
              seed: int = 0, chunk_size: int = 1024, *,
              reorth_passes: int | str = "auto",
              rotation_mode: int = 0, loadings: bool = False, PCs=None,
              use_graphs: bool = False, profile: bool = False,
              svd_mode: int = 0, stream=None) -> SolveResult:
        o = L.SolveOpts()
        L.lib().bgpu_solve_opts_default(C.byref(o))
        o.k, o.subspace_size = int(num_PCs), int(subspace_size)
        o.tolerance, o.max_iterations = float(tolerance), int(max_iterations)
        o.seed, o.chunk_size = int(seed) & 0xFFFFFFFFFFFFFFFF, int(chunk_size)
        o.reorth_passes = reorth_code(reorth_passes)
        o.rotation_mode = int(rotation_mode)
        o.use_graphs, o.profile = int(use_graphs), int(profile)
        o.svd_mode = int(svd_mode)
        on_dev = PCs is not None and not isinstance(PCs, np.ndarray)
        if PCs is None:
            PCs = np.empty((self.num_cells, num_PCs), dtype=np.float32)
        sv = np.empty(num_PCs, dtype=np.float32)
        ld = np.empty((self.num_genes, num_PCs), dtype=np.float32) if loadings else None
        info = L.SolveInfo()
        L.call("bgpu_irlba", self.handle, C.byref(o), _ptr(PCs), int(on_dev),
               sv.ctypes.data, _ptr(ld), C.byref(info), _stream(stream))
        return SolveResult(PCs, sv, ld, bool(info.converged), info.as_dict())


def reorth_code(reorth_passes) -> int:
    """U-side Gram-Schmidt passes per Lanczos step: "auto" (one pass as the
    reference, a second only where the first cancelled more than half of the
    squared norm), 1 or 2."""
    if isinstance(reorth_passes, str):
        if reorth_passes == "auto":
            return 0
    elif reorth_passes in (1, 2):
        return int(reorth_passes)
    raise ValueError(f"reorth_passes must be 'auto', 1 or 2, got {reorth_passes!r}")


def _np_dtype(a) -> np.dtype:
    if isinstance(a, np.ndarray):
        return a.dtype
    import torch
    return np.dtype(str(a.dtype).replace("torch.", ""))


# ---------------------------------------------------------------------------
def _as_mask(col, n: int, name: str):
    if col is None:
        return None
    m = np.asarray(col)
    if m.dtype != bool or m.ndim != 1 or m.shape[0] != n:
        raise TypeError(f"{name} must be a 1D Boolean array of length {n:,}")
    return m


def _validate(num_PCs, subspace_size, tolerance, max_iterations, chunk_size,
              seed, match_parallel, num_threads):
    """Argument checks of brisc/single_cell.py:11790-11840."""
    def is_int(x):
        return isinstance(x, (int, np.integer)) and not isinstance(x, bool)
    if not is_int(num_PCs):
        raise TypeError("num_PCs must be a positive integer")
    if num_PCs < 1:
        raise ValueError(f"num_PCs is {num_PCs:,}, but must be ≥ 1")
    if not is_int(subspace_size):
        raise TypeError("subspace_size must be a positive integer")
    if subspace_size < num_PCs:
        raise ValueError(f"subspace_size is {subspace_size:,}, but must be ≥ "
                         f"num_PCs ({num_PCs:,})")
    if not isinstance(tolerance, (int, float, np.integer, np.floating)) or \
            isinstance(tolerance, bool):
        raise TypeError("tolerance must be a positive number")
    if tolerance <= 0:
        raise ValueError(f"tolerance is {tolerance}, but must be > 0")
    if not is_int(max_iterations):
        raise TypeError("max_iterations must be a positive integer")
    if max_iterations < 1:
        raise ValueError(f"max_iterations is {max_iterations:,}, but must be ≥ 1")
    if not is_int(chunk_size):
        raise TypeError("chunk_size must be a positive integer")
    if chunk_size < 1:
        raise ValueError(f"chunk_size is {chunk_size:,}, but must be ≥ 1")
    if not is_int(seed):
        raise TypeError("seed must be an integer")
    if num_threads is None:
        num_threads = 1
    elif num_threads == -1:
        num_threads = os.cpu_count()
    elif not is_int(num_threads) or num_threads < 1:
        raise ValueError("num_threads must be a positive integer or -1")
    if not isinstance(match_parallel, bool):
        raise TypeError("match_parallel must be Boolean")
    if match_parallel and num_threads != 1:
        raise ValueError("match_parallel must be False unless num_threads is 1")
    return num_threads


def _subset(X, qc, hvg):
    import scipy.sparse as sp
    X = X.tocsr() if not sp.isspmatrix_csr(X) and not isinstance(X, sp.csr_array) else X
    if qc is not None:
        X = X[np.flatnonzero(qc)]
    if hvg is not None:
        X = X[:, np.flatnonzero(hvg)]
    X = sp.csr_matrix(X)
    X.sort_indices()
    return X


def _full_loadings(ld, hvg, num_all_genes: int):
    """Loadings over every gene (the varm layout): NaN rows for genes outside
    the HVG mask."""
    if hvg is None:
        return ld
    full = np.full((num_all_genes, ld.shape[1]), np.nan, dtype=np.float32)
    full[hvg] = ld
    return full


def pca(X, *others, QC_column=None, hvg_column=None, num_PCs: int = 50,
        subspace_size: int = 100, tolerance: float = 1e-6,
        max_iterations: int = 100, chunk_size: int = 1024, seed: int = 0,
        match_parallel: bool = False, verbose: bool = False,
        num_threads=None, loadings: bool = False, return_result: bool = False):
    """``SingleCell.pca()`` for scipy sparse matrices of normalised counts.

    ``X`` (and each of ``others``) is a float32 cells x genes CSR/CSC matrix,
    as ``SingleCell.normalize()`` leaves it. ``QC_column`` / ``hvg_column``
    are Boolean masks (or sequences of masks, one per dataset, or None).
    Returns the PCs array (cells x num_PCs, float32, NaN rows for cells that
    failed QC), or a tuple of arrays when ``others`` are given. With
    ``loadings=True`` returns ``(PCs, loadings)``: the right singular vectors,
    genes x num_PCs float32 over every gene of ``X`` (a varm-shaped array),
    NaN for genes outside ``hvg_column``; one array shared by all datasets.
    """
    import scipy.sparse as sp
    datasets = [X, *others]
    for d in datasets:
        if not sp.issparse(d):
            raise TypeError("X must be a scipy sparse matrix")
        if d.dtype != np.float32:
            raise TypeError(
                f"PCA() requires normalized counts with data type float32, but "
                f"X has data type {str(d.dtype)!r}; did you forget to run "
                f"normalize() before PCA()?")
    nd = len(datasets)
    qcs = QC_column if isinstance(QC_column, (list, tuple)) else [QC_column] * nd
    hvgs = hvg_column if isinstance(hvg_column, (list, tuple)) else [hvg_column] * nd
    if len(qcs) != nd or len(hvgs) != nd:
        raise ValueError("QC_column/hvg_column sequences need one entry per dataset")
    qcs = [_as_mask(q, d.shape[0], "QC_column") for q, d in zip(qcs, datasets)]
    hvgs = [_as_mask(h, d.shape[1], "hvg_column") for h, d in zip(hvgs, datasets)]
    suffix = " for at least one dataset" if others else ""
    if any(q is not None and not q.any() for q in qcs):
        raise ValueError(f"no cells pass QC{suffix}: QC_column is all-False")
    _validate(num_PCs, subspace_size, tolerance, max_iterations, chunk_size,
              seed, match_parallel, num_threads)
    Xs = [_subset(d, q, h) for d, q, h in zip(datasets, qcs, hvgs)]
    g = {x.shape[1] for x in Xs}
    if len(g) != 1:
        raise ValueError("datasets have different numbers of selected genes")
    Xall = Xs[0] if nd == 1 else sp.vstack(Xs, format="csr")
    num_cells, num_genes = Xall.shape
    if num_cells < num_PCs:
        raise ValueError(f"num_PCs is {num_PCs:,}, but must be ≤ the number of "
                         f"cells ({num_cells:,})")
    if num_genes < num_PCs:
        raise ValueError(f"num_PCs is {num_PCs:,}, but must be ≤ the number of "
                         f"genes ({num_genes:,})")
    if num_cells == 1:
        raise ValueError("there is only one cell, so principal components "
                         "cannot be calculated")
    if num_genes == 1:
        raise ValueError("there is only one gene, so principal components "
                         "cannot be calculated")
    subspace_size = min(subspace_size, num_cells, num_genes)
    M = DeviceMatrix(Xall.indptr, Xall.indices, Xall.data, num_cells, num_genes)
    try:
        res = M.solve(num_PCs, subspace_size, tolerance, max_iterations, seed,
                      chunk_size, loadings=loadings)
    finally:
        M.close()
    if not res.converged and verbose:
        print(f"PCA did not converge to a tolerance of {tolerance:.2g} after "
              f"{max_iterations:,} iterations; consider increasing "
              f"max_iterations or tolerance")
    outs, start = [], 0
    for d, q, x in zip(datasets, qcs, Xs):
        part = res.PCs[start:start + x.shape[0]]
        start += x.shape[0]
        if q is not None:
            full = np.full((d.shape[0], num_PCs), np.nan, dtype=np.float32)
            full[q] = part
            part = full
        outs.append(part)
    out = outs[0] if nd == 1 else tuple(outs)
    if loadings:
        out = (out, _full_loadings(res.loadings, hvgs[0], datasets[0].shape[1]))
    return (out, res) if return_result else out


def pca_counts(counts, *, method: str = "logCP10k", QC_column=None,
               hvg_column=None, num_PCs: int = 50, subspace_size: int = 100,
               tolerance: float = 1e-6, max_iterations: int = 100,
               seed: int = 0, chunk_size: int = 1024, loadings: bool = False,
               return_result: bool = False):
    """PCA straight from raw counts, normalisation fused into the products.

    ``counts`` is a cells x ALL-genes integer CSR matrix (uint16, uint32,
    int32, or float32 holding integers). Per-cell size factors are computed
    on the GPU over all genes (as ``normalize()`` does, brisc/normalize.pyx:
    36-81, with the QC mask for log1pPF's mean), then the QC cells and HVG
    genes are selected and PCA runs on log1p(count * factor) without ever
    storing the normalised values. ``loadings=True`` returns ``(PCs,
    loadings)`` as :func:`pca` does.
    """
    import scipy.sparse as sp
    import torch
    if method not in _METHODS:
        raise ValueError("method must be one of 'PFlog1pPF', 'log1pPF', or "
                         "'logCP10k'")
    X = sp.csr_matrix(counts)
    n, G = X.shape
    qc = _as_mask(QC_column, n, "QC_column")
    hvg = _as_mask(hvg_column, G, "hvg_column")
    if qc is not None and not qc.any():
        raise ValueError("no cells pass QC: QC_column is all-False")
    _validate(num_PCs, subspace_size, tolerance, max_iterations, chunk_size,
              seed, False, None)
    if X.dtype not in _VALUE_TYPES:
        X = X.astype(np.float32)
    isf, post = size_factors(X, method, qc)
    if qc is not None:
        keep = np.flatnonzero(qc)
        isf = isf[keep]
        post = post[keep] if post is not None else None
    Xs = _subset(X, qc, hvg)
    num_cells, num_genes = Xs.shape
    subspace_size = min(subspace_size, num_cells, num_genes)
    M = DeviceMatrix(Xs.indptr, Xs.indices.astype(Xs.indptr.dtype, copy=False),
                     Xs.data, num_cells, num_genes, norm=method,
                     inv_size_factors=isf, post_factors=post)
    try:
        res = M.solve(num_PCs, subspace_size, tolerance, max_iterations, seed,
                      chunk_size, loadings=loadings)
    finally:
        M.close()
    out = res.PCs
    if qc is not None:
        full = np.full((n, num_PCs), np.nan, dtype=np.float32)
        full[qc] = out
        out = full
    if loadings:
        out = (out, _full_loadings(res.loadings, hvg, G))
    return (out, res) if return_result else out


def size_factors(counts, method: str = "logCP10k", qc=None, stream=None):
    """Per-cell inverse size factors (and method-2 post factors) on the GPU,
    over all genes (brisc/normalize.pyx:9-268). Returns host float32 arrays."""
    import scipy.sparse as sp
    import torch
    X = sp.csr_matrix(counts)
    if X.dtype not in _VALUE_TYPES:
        X = X.astype(np.float32)
    n = X.shape[0]
    dev = torch.device("cuda")
    ip = torch.from_numpy(np.ascontiguousarray(X.indptr)).to(dev)
    vals = torch.from_numpy(np.ascontiguousarray(X.data).view(
        np.int16 if X.dtype == np.uint16 else X.dtype)).to(dev)
    isf = torch.empty(n, dtype=torch.float32, device=dev)
    post = torch.empty(n, dtype=torch.float32, device=dev) if method == "PFlog1pPF" else None
    q = torch.from_numpy(qc.astype(np.uint8)).to(dev) if qc is not None else None
    L.call("bgpu_size_factors", _ptr(ip), _INDEX_TYPES[X.indptr.dtype],
           _ptr(vals), _VALUE_TYPES[X.dtype], n, _METHODS[method], _ptr(q),
           _ptr(isf), _ptr(post), None, _stream(stream))
    torch.cuda.synchronize()
    return isf.cpu().numpy(), (post.cpu().numpy() if post is not None else None)
