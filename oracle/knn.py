"""NumPy restatement of the reference's knn_self (brisc/knn.pyx:13-515).

Test infrastructure: the checker for brisc_gb300's GPU knn_self, pinned
against the compiled reference's outputs in tests/golden/knn.npz. Never
imported by the product.

The search, as knn.pyx does it (single-threaded branch, :113-290; the
parallel branch computes the same lists):
- centroid norms |c|^2, a float sum over dimensions in order (:117-121);
- per cell, the num_clusters_searched centroids with the smallest partial
  distance |c|^2 - 2 x.c, visited in ascending centroid order, a candidate
  kept when strictly smaller than the current worst (:131-175), output in
  ascending order (:178-182);
- per cell, every cell of those clusters except itself, visited by ascending
  cluster label (the pair sort of :198-210) and ascending position, distance
  |x|^2 + (|c|^2 - 2 x.c), kept when strictly smaller than the current worst
  (:232-275), output ascending (:279-283), ids mapped through sorted_order.
Distances here are computed in FP64 from the float32 inputs (the reference's
come from sgemm in FP32), so comparisons against either allow for FP32
rounding: see ``compare``.
"""
from __future__ import annotations

import numpy as np


def _select(dist: np.ndarray, ids: np.ndarray, k: int):
    """The k entries a strict-improvement max-heap keeps when fed (dist, id)
    in order: the k smallest, an earlier entry winning a tie. Returned in
    ascending (distance, visiting order)."""
    order = np.argsort(dist, kind="stable")[:k]
    return dist[order], ids[order]


def knn_self(X, sorted_order, centroids, num_cells_per_cluster, cell_norms,
             num_neighbors: int, num_clusters_searched: int):
    X = np.asarray(X, dtype=np.float32)
    C = np.asarray(centroids, dtype=np.float32)
    n = X.shape[0]
    k, cs = int(num_neighbors), int(num_clusters_searched)
    X64, C64 = X.astype(np.float64), C.astype(np.float64)
    cn = np.einsum("ij,ij->i", C64, C64)
    pd = cn[None, :] - 2.0 * (X64 @ C64.T)
    nearest = np.empty((n, cs), dtype=np.uint32)
    cdist = np.empty((n, cs), dtype=np.float64)
    labels = np.arange(C.shape[0], dtype=np.uint32)
    for i in range(n):
        d, ids = _select(pd[i], labels, cs)
        nearest[i], cdist[i] = ids, d
    off = np.concatenate([[0], np.cumsum(num_cells_per_cluster, dtype=np.int64)])
    norms = np.asarray(cell_norms, dtype=np.float64)
    nbr = np.empty((n, k), dtype=np.uint32)
    dist = np.empty((n, k), dtype=np.float64)
    for i in range(n):
        cand = np.concatenate([np.arange(off[c], off[c + 1])
                               for c in np.sort(nearest[i])])
        cand = cand[cand != i]
        dd = norms[i] + (norms[cand] - 2.0 * (X64[cand] @ X64[i]))
        d, ids = _select(dd, cand, k)
        nbr[i] = np.asarray(sorted_order)[ids]
        dist[i] = d
    return nbr, dist, nearest, cdist


def exact_distances(X, sorted_order, nbr):
    """FP64 squared distances sum (x - y)^2 between each row of X (cluster
    order) and the listed neighbours (original ids)."""
    X64 = np.asarray(X, dtype=np.float64)
    inv = np.empty_like(sorted_order)
    inv[sorted_order] = np.arange(len(sorted_order), dtype=sorted_order.dtype)
    rows = inv[nbr.astype(np.int64)]
    diff = X64[rows] - X64[:, None, :]
    return np.einsum("ijk,ijk->ij", diff, diff)


def compare(X, sorted_order, cell_norms, nbr_a, nbr_b, rtol: float = 2e-6, rows=None):
    """Two neighbour lists of the same search agree when, row by row, they
    hold the same ids except where the ids that differ sit at distances
    within FP32 rounding of the other list's k-th distance (a near-tie that
    either side may break). Rounding scale: rtol * (|x|^2 + max |y|^2).
    Returns (fraction of rows identical as sets, worst excess of a differing
    id's distance beyond the tie band, in units of the band), over ``rows``
    (default: all)."""
    da = exact_distances(X, sorted_order, nbr_a)
    db = exact_distances(X, sorted_order, nbr_b)
    norms = np.asarray(cell_norms, dtype=np.float64)
    band = rtol * (norms + norms.max()) + 1e-30
    same = 0
    worst = 0.0
    rows = range(nbr_a.shape[0]) if rows is None else rows
    for i in rows:
        sa, sb = set(nbr_a[i].tolist()), set(nbr_b[i].tolist())
        if sa == sb:
            same += 1
            continue
        kth = max(da[i].max(), db[i].max())
        for j, v in enumerate(nbr_a[i]):
            if v not in sb:
                worst = max(worst, (kth - da[i, j]) / band[i])
        for j, v in enumerate(nbr_b[i]):
            if v not in sa:
                worst = max(worst, (kth - db[i, j]) / band[i])
    return same / max(1, len(rows)), worst
