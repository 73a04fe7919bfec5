"""Shared helpers of the knn tests: the fixture cases of tests/golden/knn.npz
with their regenerated inputs."""
from __future__ import annotations

import hashlib

import numpy as np


def knn_pcs(n: int, d: int, comps: int, seed: int) -> np.ndarray:
    """The seeded Gaussian-mixture stand-in for principal components that
    tests/golden/make_golden.py fed the reference (synth.pca_like)."""
    from synth import pca_like
    return pca_like(n, d, comps, seed)


def case(z, name: str) -> dict:
    n, d, comps, seed, k, cs = (int(v) for v in z[f"{name}_shape"])
    X = knn_pcs(n, d, comps, seed)
    assert hashlib.sha256(X.tobytes()).hexdigest() == str(z[f"{name}_fingerprint"]), \
        "regenerated PCs differ from the ones the reference saw"
    so = z[f"{name}_sorted_order"]
    return dict(X=np.ascontiguousarray(X[so]), sorted_order=so,
                centroids=z[f"{name}_centroids"],
                num_cells_per_cluster=z[f"{name}_num_cells_per_cluster"],
                cell_norms=z[f"{name}_cell_norms"], num_neighbors=k,
                num_clusters_searched=cs,
                ref_neighbors=z[f"{name}_neighbors"],
                ref_distances=z[f"{name}_distances"],
                ref_nearest=z[f"{name}_nearest_clusters"],
                ref_cdist=z[f"{name}_centroid_distances"])


def check_against(c: dict, nbr, dist, near, cdist, *, min_same: float = 0.99) -> None:
    """A knn_self result agrees with the reference's: nearest-cluster lists
    identical except at near-ties of the partial distance; on rows with the
    same clusters, neighbour sets identical except at near-ties (oracle.knn
    .compare); distances within FP32 rounding of the squared norms."""
    from oracle import knn as oknn
    norms = c["cell_norms"].astype(np.float64)
    C = c["centroids"].astype(np.float64)
    cn = np.einsum("ij,ij->i", C, C)
    band_c = 2e-6 * (norms + cn.max())
    rows_same_c = np.all(np.sort(near, 1) == np.sort(c["ref_nearest"], 1), axis=1)
    assert rows_same_c.mean() >= min_same, rows_same_c.mean()
    for i in np.flatnonzero(~rows_same_c):  # boundary swaps are near-ties
        a = set(near[i].tolist()) ^ set(c["ref_nearest"][i].tolist())
        pd = cn[list(a)] - 2.0 * (C[list(a)] @ c["X"][i].astype(np.float64))
        kth = max(cdist[i].max(), c["ref_cdist"][i].max())
        assert np.all(pd >= kth - 2 * band_c[i]), (i, pd, kth)
    np.testing.assert_allclose(cdist, c["ref_cdist"], rtol=0,
                               atol=float(2 * band_c.max()))
    sel = np.flatnonzero(rows_same_c)
    same, worst = oknn.compare(c["X"], c["sorted_order"], c["cell_norms"], nbr,
                               c["ref_neighbors"], rows=sel)
    assert same >= min_same and worst <= 1.0, (same, worst)
    band = 2e-6 * (norms + norms.max())
    assert np.all(np.abs(dist[sel] - c["ref_distances"][sel]) <= 2 * band[sel, None] + 1e-30)
