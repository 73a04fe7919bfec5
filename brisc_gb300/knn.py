"""k-nearest neighbours on the principal components, on the GPU.

``kmeans`` and ``knn_self`` keep the reference's names, keyword arguments and
in-place outputs (brisc/kmeans.pyx:889-904, brisc/knn.pyx:13-31):
``SingleCell.neighbors()`` runs k-means, sorts the cells by cluster and calls
knn_self (brisc/single_cell.py:12532-12626). ``install_knn()`` binds both into
brisc's ``single_cell`` module in place of the reference's, so an installed
brisc's ``neighbors()`` runs on the GPU; ``neighbors()`` here restates that
method for a PCs array.

k-means uses the reference's random initialisation (its default) and its
M-step summation order; the E step's distances are FP32 fused multiply-adds
instead of sgemm, so assignments can differ only where two centroids are
equally near to FP32 rounding.

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


def kmeans(X, cluster_labels, centroids, centroids_new, num_cells_per_cluster,
           min_distances, cell_norms, kmeans_barbar=False, num_init_iterations=5,
           num_kmeans_iterations=2, tolerance=1e-2, oversampling_factor=1,
           chunk_size=None, seed=0, is_mac=False, num_threads=1) -> int:
    """brisc/kmeans.pyx:889-1433 on the GPU (random initialisation). Fills
    the outputs in place and returns the number of iterations run; the final
    centroids are in ``centroids_new`` when it is odd, as the reference's.
    An empty ``cell_norms`` skips the norms, as there."""
    n, d = int(X.shape[0]), int(X.shape[1])
    nc = int(centroids.shape[0])
    if kmeans_barbar:
        raise NotImplementedError("kmeans_barbar=True (k-means|| initialisation) is not "
                                  "on the GPU path; the default random initialisation is")
    _need(X, "X", np.float32, (n, d))
    _need(cluster_labels, "cluster_labels", np.uint32, (n,))
    _need(centroids, "centroids", np.float32, (nc, d))
    _need(centroids_new, "centroids_new", np.float32, (nc, d))
    _need(num_cells_per_cluster, "num_cells_per_cluster", np.uint32, (nc,))
    _need(min_distances, "min_distances", np.float32, (n,))
    with_norms = int(cell_norms.shape[0]) != 0
    if with_norms:
        _need(cell_norms, "cell_norms", np.float32, (n,))
    chunk_size = min(4096, n) if chunk_size is None else int(chunk_size)
    arrays = [X, cluster_labels, centroids, centroids_new, num_cells_per_cluster,
              min_distances] + ([cell_norms] if with_norms else [])
    on_dev = _is_cuda(X)
    if any(_is_cuda(a) != on_dev for a in arrays):
        raise TypeError("all arrays must be NumPy arrays, or all CUDA tensors")
    import torch
    it = C.c_uint32(0)
    if on_dev:
        ptrs = [a.data_ptr() for a in arrays] + ([] if with_norms else [None])
        stream = torch.cuda.current_stream(X.device).cuda_stream
    else:
        dev = torch.device("cuda", torch.cuda.current_device())
        outputs = range(1, len(arrays))
        t = [torch.empty(a.nbytes, dtype=torch.uint8, device=dev) if i in outputs
             else torch.from_numpy(a.view(np.uint8).reshape(-1)).to(dev)
             for i, a in enumerate(arrays)]
        ptrs = [x.data_ptr() for x in t] + ([] if with_norms else [None])
        stream = torch.cuda.current_stream(dev).cuda_stream
    L.call("bgpu_kmeans", *ptrs, 0, int(num_kmeans_iterations), float(tolerance),
           chunk_size, int(seed) & 0xFFFFFFFFFFFFFFFF, n, d, nc, C.byref(it),
           C.c_void_p(stream))
    if not on_dev:
        for i in outputs:
            arrays[i].view(np.uint8).reshape(-1)[:] = t[i].cpu().numpy()
    return int(it.value)


def neighbors(PCs, num_neighbors: int = 20, num_clusters=None,
              num_clusters_searched=None, num_kmeans_iterations: int = 2,
              kmeans_tolerance: float = 1e-2, chunk_size_kmeans=None,
              chunk_size_search=None, seed: int = 0):
    """SingleCell.neighbors() (brisc/single_cell.py:12139-12665) for a
    float32 PCs array of the cells passing QC: k-means, the argument
    preparation of single_cell.py:12451-12611 (default cluster counts and
    chunk sizes, empty clusters removed, enough clusters searched for
    num_neighbors + 1 candidates, centroids ordered by PC 1, cells sorted by
    cluster), knn_self, and the un-sorting of single_cell.py:12628-12646.
    Returns (neighbors uint32, distances float32), num_cells x
    num_neighbors, in the cells' original order. Checks and messages are
    the reference's."""
    X = np.ascontiguousarray(PCs, dtype=np.float32)
    n, d = X.shape
    if n == 1:
        raise ValueError("there is only one cell, so nearest neighbors cannot be "
                         "calculated")
    if not 1 <= num_neighbors < n:
        raise ValueError(f"num_neighbors is {num_neighbors:,}, but must be ≥ 1 and less "
                         f"than the number of cells ({n:,})")
    if num_clusters is None:
        num_clusters = max(1, int(np.ceil(min(4 * np.sqrt(n), n / 100))))
    elif not 1 <= num_clusters <= n:
        raise ValueError(f"num_clusters is {num_clusters:,}, but must be ≥ 1 and ≤ the "
                         f"number of cells ({n:,})")
    if num_clusters_searched is None:
        num_clusters_searched = min(64, num_clusters)
    elif not 1 <= num_clusters_searched <= num_clusters:
        raise ValueError(f"num_clusters_searched is {num_clusters_searched:,}, but must be "
                         f"≥ 1 and ≤ num_clusters ({num_clusters:,})")
    chunk_size_kmeans = min(4096, n) if chunk_size_kmeans is None else chunk_size_kmeans
    chunk_size_search = min(256, n) if chunk_size_search is None else chunk_size_search
    labels = np.empty(n, dtype=np.uint32)
    mind = np.empty(n, dtype=np.float32)
    norms = np.empty(n, dtype=np.float32)
    cent = np.empty((num_clusters, d), dtype=np.float32)
    cent_new = np.empty((num_clusters, d), dtype=np.float32)
    counts = np.empty(num_clusters, dtype=np.uint32)
    it = kmeans(X=X, cluster_labels=labels, centroids=cent, centroids_new=cent_new,
                num_cells_per_cluster=counts, min_distances=mind, cell_norms=norms,
                num_kmeans_iterations=num_kmeans_iterations, tolerance=kmeans_tolerance,
                chunk_size=chunk_size_kmeans, seed=seed)
    if it & 1:
        cent = cent_new
    keep = counts > 0
    if not keep.all():
        cent, counts = cent[keep], counts[keep]
        remap = np.zeros(len(keep), dtype=np.uint32)
        remap[keep] = np.arange(len(cent), dtype=np.uint32)
        labels = remap[labels]
    nc = len(cent)
    cumsum = np.sort(counts).cumsum(dtype=np.uint64)
    min_searched = int(np.searchsorted(cumsum, num_neighbors + 1)) + 1
    cs = min(max(num_clusters_searched, min_searched), nc)
    order = np.argsort(cent[:, 0]).astype(np.uint32)
    cent = np.ascontiguousarray(cent[order])
    counts = np.ascontiguousarray(counts[order])
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order), dtype=np.uint32)
    labels = inv[labels]
    so = np.argsort(labels).astype(np.uint32)
    nbr = np.empty((n, num_neighbors), dtype=np.uint32)
    dist = np.empty((n, num_neighbors), dtype=np.float32)
    knn_self(X=np.ascontiguousarray(X[so]), sorted_order=so, centroids=cent,
             num_cells_per_cluster=counts, neighbors=nbr, distances=dist,
             cell_norms=np.ascontiguousarray(norms[so]),
             centroid_distances=np.empty((n, cs), dtype=np.float32),
             nearest_clusters=np.empty((n, cs), dtype=np.uint32),
             num_neighbors=num_neighbors, num_clusters_searched=cs,
             chunk_size_kmeans=chunk_size_kmeans, chunk_size_search=chunk_size_search)
    out_n = np.empty_like(nbr)
    out_d = np.empty_like(dist)
    out_n[so], out_d[so] = nbr, dist
    return out_n, out_d


NAMES = ("kmeans", "knn_self")


def install_knn(module=None) -> dict:
    """Bind ``kmeans`` and ``knn_self`` into brisc's ``single_cell`` module,
    where ``import_cython`` puts the reference's (brisc/single_cell.py:34-61)
    and ``neighbors()`` calls them (single_cell.py:12532, 12613). Returns the
    previous bindings (name -> function), for restoring them."""
    if module is None:
        import brisc.single_cell as module  # pragma: no cover
    previous = {name: getattr(module, name, None) for name in NAMES}
    here = globals()
    for name in NAMES:
        setattr(module, name, here[name])
    return previous
