"""Harmony batch correction of the PCs, on the GPU.

``normalize_rows`` and ``harmony`` keep the reference's names, keyword
arguments and in-place outputs (brisc/harmonize.pyx:244 and :269):
``SingleCell.harmonize()`` normalises the PCs' rows, runs k-means on them for
the initial centroids and calls harmony (brisc/single_cell.py:13812-13875).
``install_harmony()`` binds both into brisc's ``single_cell`` module in place
of the reference's, so an installed brisc's ``harmonize()`` runs them on the
GPU (its k-means too, after ``install_knn()``); ``harmonize()`` here restates
that method's core for a PCs array, entirely on the device.

The algorithm is the reference's: the same PCG32 cell order, the same blocks
and chunks, each chunk's assignments recomputed from the cluster-batch sums as
the block found them and the sums updated block by block in chunk order, the
same ridge correction and stopping rule. Products and sums run in FP32 in a
fixed order of their own (the reference's are sgemm calls and per-thread
sums), so results agree to float rounding, which Harmony's iterations amplify
a little; the tests state the tolerance. ``verbose`` and ``num_threads`` are
accepted and have no effect.

Arrays are NumPy arrays (copied to the device and back) or CUDA tensors (used
in place; then every array must be one).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .knn import _is_cuda, _need, kmeans


def _stream(dev):
    import torch
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def normalize_rows(arr, out, num_threads=1) -> None:
    """brisc/harmonize.pyx:244-266 on the GPU: ``out`` = ``arr`` with every
    row scaled to unit norm."""
    n, d = int(arr.shape[0]), int(arr.shape[1])
    _need(arr, "arr", np.float32, (n, d))
    _need(out, "out", np.float32, (n, d))
    if _is_cuda(arr) != _is_cuda(out):
        raise TypeError("arr and out must both be NumPy arrays or both CUDA tensors")
    import torch
    if _is_cuda(arr):
        L.call("bgpu_normalize_rows", arr.data_ptr(), out.data_ptr(), n, d,
               _stream(arr.device))
        return
    dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.from_numpy(np.ascontiguousarray(arr)).to(dev)
    L.call("bgpu_normalize_rows", t.data_ptr(), t.data_ptr(), n, d, _stream(dev))
    out[...] = t.cpu().numpy()


def harmony(PCs, Z, Y, R, batch_labels, num_batches, max_iterations=10,
            max_clustering_iterations=5, block_proportion=0.05, tolerance=0.01,
            early_stopping=False, clustering_tolerance=1e-3, theta=2, tau=0,
            alpha=0.2, sigma=0.1, chunk_size=256, seed=0, verbose=False,
            num_threads=1) -> int:
    """brisc/harmonize.pyx:269-871 on the GPU. Updates ``Z`` (to the Harmony
    embedding), ``Y`` and ``R`` in place; returns the number of correction
    rounds run."""
    n, d = int(PCs.shape[0]), int(PCs.shape[1])
    nc = int(Y.shape[0])
    _need(PCs, "PCs", np.float32, (n, d))
    _need(Z, "Z", np.float32, (n, d))
    _need(Y, "Y", np.float32, (nc, d))
    _need(R, "R", np.float32, (n, nc))
    _need(batch_labels, "batch_labels", np.uint32, (n,))
    arrays = (PCs, Z, Y, R, batch_labels)
    on_dev = _is_cuda(PCs)
    if any(_is_cuda(a) != on_dev for a in arrays):
        raise TypeError("all arrays must be NumPy arrays, or all CUDA tensors")
    import torch
    it = C.c_uint32(0)
    args = (int(num_batches), int(max_iterations), int(max_clustering_iterations),
            float(block_proportion), float(tolerance), int(bool(early_stopping)),
            float(clustering_tolerance), float(theta), float(tau), float(alpha),
            float(sigma), int(chunk_size), int(seed) & 0xFFFFFFFFFFFFFFFF, n, d, nc,
            C.byref(it))
    if on_dev:
        L.call("bgpu_harmony", *[a.data_ptr() for a in arrays], *args, _stream(PCs.device))
        return int(it.value)
    dev = torch.device("cuda", torch.cuda.current_device())
    t = [torch.from_numpy(a.view(np.uint8).reshape(-1)).to(dev) for a in arrays]
    L.call("bgpu_harmony", *[x.data_ptr() for x in t], *args, _stream(dev))
    for i in (1, 2, 3):
        arrays[i].view(np.uint8).reshape(-1)[:] = t[i].cpu().numpy()
    return int(it.value)


def harmonize(PCs, batch_labels, num_batches=None, num_clusters=None,
              max_iterations: int = 10, num_kmeans_iterations: int = 25,
              kmeans_tolerance: float = 1e-2, chunk_size_kmeans=None,
              max_clustering_iterations: int = 5, block_proportion: float = 0.05,
              tolerance: float = 0.01, early_stopping: bool = False,
              clustering_tolerance: float = 1e-3, theta: float = 2, tau: float = 0,
              alpha: float = 0.2, sigma: float = 0.1, chunk_size_Harmony=None,
              seed: int = 0, return_info: bool = False):
    """The core of SingleCell.harmonize() (brisc/single_cell.py:13776-13875)
    for the float32 PCs of the cells passing QC and their uint32 batch labels:
    default cluster count and chunk sizes with the reference's checks, Z =
    normalize_rows(PCs), k-means on Z (random initialisation), harmony.
    NumPy inputs give a NumPy result; CUDA tensors stay on their device.
    Returns the Harmony embedding (num_cells x num_PCs, float32); with
    return_info, also a dict of the k-means and Harmony iteration counts and
    the cluster count."""
    import torch
    on_dev = _is_cuda(PCs)
    if on_dev:
        dev = PCs.device
        P = PCs.contiguous()
        b = batch_labels.to(device=dev, dtype=torch.int32).contiguous()
    else:
        dev = torch.device("cuda", torch.cuda.current_device())
        P = torch.from_numpy(np.ascontiguousarray(PCs, dtype=np.float32)).to(dev)
        b = torch.from_numpy(np.ascontiguousarray(batch_labels, dtype=np.uint32)
                             .view(np.int32)).to(dev)
    if P.dtype != torch.float32:
        raise TypeError(f"PCs.dtype is {P.dtype}, but must be float32")
    n, d = P.shape
    if num_batches is None:
        num_batches = int(b.max().item()) + 1 if n else 0
    if num_clusters is None:
        num_clusters = max(min(100, int(round(n / 30))), 1)
    elif num_clusters >= n:
        raise ValueError(f"num_clusters is {num_clusters:,}, but must be less than the "
                         f"total number of cells across all datasets ({n:,})")
    if chunk_size_kmeans is None:
        chunk_size_kmeans = min(4096, n)
    elif chunk_size_kmeans >= n:
        raise ValueError(f"chunk_size_kmeans is {chunk_size_kmeans:,}, but must be less "
                         f"than the total number of cells across all datasets ({n:,})")
    if chunk_size_Harmony is None:
        chunk_size_Harmony = min(256, n)
    elif chunk_size_Harmony >= n:
        raise ValueError(f"chunk_size_Harmony is {chunk_size_Harmony:,}, but must be less "
                         f"than the total number of cells across all datasets ({n:,})")
    Z = torch.empty_like(P)
    normalize_rows(P, Z)
    f32 = dict(dtype=torch.float32, device=dev)
    i32 = dict(dtype=torch.int32, device=dev)
    Y = torch.empty((num_clusters, d), **f32)
    Y_new = torch.empty((num_clusters, d), **f32)
    it = kmeans(X=Z, cluster_labels=torch.empty(n, **i32), centroids=Y,
                centroids_new=Y_new, num_cells_per_cluster=torch.empty(num_clusters, **i32),
                min_distances=torch.empty(n, **f32), cell_norms=torch.empty(0, **f32),
                num_kmeans_iterations=num_kmeans_iterations, tolerance=kmeans_tolerance,
                chunk_size=chunk_size_kmeans, seed=seed)
    if it & 1:
        Y = Y_new
    R = torch.empty((n, num_clusters), **f32)
    h_it = harmony(PCs=P, Z=Z, Y=Y, R=R, batch_labels=b, num_batches=num_batches,
            max_iterations=max_iterations,
            max_clustering_iterations=max_clustering_iterations,
            block_proportion=block_proportion, tolerance=tolerance,
            early_stopping=early_stopping, clustering_tolerance=clustering_tolerance,
            theta=theta, tau=tau, alpha=alpha, sigma=sigma,
            chunk_size=chunk_size_Harmony, seed=seed)
    out = Z if on_dev else Z.cpu().numpy()
    if return_info:
        return out, {"kmeans_iterations": it, "iterations": h_it,
                     "num_clusters": num_clusters}
    return out


NAMES = ("harmony", "normalize_rows")


def install_harmony(module=None) -> dict:
    """Bind ``harmony`` and ``normalize_rows`` into brisc's ``single_cell``
    module, where ``import_cython`` puts the reference's (brisc/
    single_cell.py:34-40) and ``harmonize()`` calls them (single_cell.py:13819,
    13864). Returns the previous bindings (name -> function)."""
    if module is None:
        import brisc.single_cell as module  # pragma: no cover
    previous = {name: getattr(module, name, None) for name in NAMES}
    here = globals()
    for name in NAMES:
        setattr(module, name, here[name])
    return previous
