"""k-nearest neighbours on the principal components, on the GPU.

``knn_self`` keeps the reference's name, keyword arguments and in-place
outputs (brisc/knn.pyx:13-31): ``SingleCell.neighbors()`` runs k-means, sorts
the cells by cluster and calls it (brisc/single_cell.py:12532-12626).
``install_knn()`` binds this version into brisc's ``single_cell`` module in
place of the reference's, so an installed brisc's ``neighbors()`` searches on
the GPU.

The search is the reference's: the same candidate clusters and the same
candidates in the same order, each kept when strictly closer than the
current worst; the dot products are FP32 fused multiply-adds instead of
sgemm, so distances agree to FP32 rounding and the neighbour lists differ
only where two candidates' distances do. ``chunk_size_kmeans``,
``chunk_size_search``, ``is_mac`` and ``num_threads`` are CPU scheduling
arguments; they are checked as the reference's caller checks them and have
no effect here.

Arrays are NumPy arrays (copied to the device and back) or CUDA tensors (used
in place; then every array must be one).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _is_cuda(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _dt(a):
    return a.dtype if isinstance(a, np.ndarray) else np.dtype(str(a.dtype).replace("torch.", ""))


def _need(a, name, dtype, shape):
    ok = (np.dtype(dtype),)
    if np.dtype(dtype) == np.uint32 and _is_cuda(a):
        ok += (np.dtype(np.int32),)  # torch keeps few uint32 operations
    if _dt(a) not in ok:
        raise TypeError(f"{name} has dtype {_dt(a)}; expected {np.dtype(dtype)}")
    if tuple(a.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(a.shape)}; expected {tuple(shape)}")
    contig = a.flags.c_contiguous if isinstance(a, np.ndarray) else a.is_contiguous()
    if not contig:
        raise ValueError(f"{name} must be C-contiguous")


def knn_self(X, sorted_order, centroids, num_cells_per_cluster, neighbors,
             distances, cell_norms, centroid_distances, nearest_clusters,
             num_neighbors, num_clusters_searched, chunk_size_kmeans=None,
             chunk_size_search=None, is_mac=False, num_threads=1) -> None:
    """brisc/knn.pyx:13-515 on the GPU. Fills ``neighbors``, ``distances``,
    ``centroid_distances`` and ``nearest_clusters`` in place."""
    n, d = int(X.shape[0]), int(X.shape[1])
    nc = int(centroids.shape[0])
    k, cs = int(num_neighbors), int(num_clusters_searched)
    _need(X, "X", np.float32, (n, d))
    _need(sorted_order, "sorted_order", np.uint32, (n,))
    _need(centroids, "centroids", np.float32, (nc, d))
    _need(num_cells_per_cluster, "num_cells_per_cluster", np.uint32, (nc,))
    _need(neighbors, "neighbors", np.uint32, (n, k))
    _need(distances, "distances", np.float32, (n, k))
    _need(cell_norms, "cell_norms", np.float32, (n,))
    _need(centroid_distances, "centroid_distances", np.float32, (n, cs))
    _need(nearest_clusters, "nearest_clusters", np.uint32, (n, cs))
    if chunk_size_kmeans is None:  # neighbors()'s defaults, single_cell.py:12487-12510
        chunk_size_kmeans = min(4096, n)
    if chunk_size_search is None:
        chunk_size_search = min(256, n)
    for v, name in ((chunk_size_kmeans, "chunk_size_kmeans"),
                    (chunk_size_search, "chunk_size_search")):
        if not 1 <= int(v) <= n:
            raise ValueError(f"{name} is {int(v):,}, but must be ≥ 1 and ≤ the "
                             f"number of cells ({n:,})")
    arrays = (X, sorted_order, centroids, num_cells_per_cluster, neighbors, distances,
              cell_norms, centroid_distances, nearest_clusters)
    on_dev = _is_cuda(X)
    if any(_is_cuda(a) != on_dev for a in arrays):
        raise TypeError("all arrays must be NumPy arrays, or all CUDA tensors")
    import torch
    if on_dev:
        dev = X.device
        ptrs = [a.data_ptr() for a in arrays]
        stream = torch.cuda.current_stream(dev).cuda_stream
        L.call("bgpu_knn_self", *ptrs, n, d, nc, k, cs, C.c_void_p(stream))
        return
    # host arrays: byte copies to device buffers and back
    dev = torch.device("cuda", torch.cuda.current_device())
    outputs = (4, 5, 7, 8)
    t = [torch.empty(a.nbytes, dtype=torch.uint8, device=dev) if i in outputs
         else torch.from_numpy(a.view(np.uint8).reshape(-1)).to(dev)
         for i, a in enumerate(arrays)]
    stream = torch.cuda.current_stream(dev).cuda_stream
    L.call("bgpu_knn_self", *[x.data_ptr() for x in t], n, d, nc, k, cs,
           C.c_void_p(stream))
    for i in outputs:
        arrays[i].view(np.uint8).reshape(-1)[:] = t[i].cpu().numpy()


NAMES = ("knn_self",)


def install_knn(module=None) -> dict:
    """Bind ``knn_self`` into brisc's ``single_cell`` module, where
    ``import_cython`` puts the reference's (brisc/single_cell.py:34-61) and
    ``neighbors()`` calls it (single_cell.py:12613). Returns the previous
    binding, for restoring it."""
    if module is None:
        import brisc.single_cell as module  # pragma: no cover
    previous = {name: getattr(module, name, None) for name in NAMES}
    module.knn_self = knn_self
    return previous
