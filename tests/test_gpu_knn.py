"""knn_self on the GPU (brisc_gb300/knn.py over csrc/knn.cu) against the
reference's own outputs (tests/golden/knn.npz, from brisc/knn.pyx:13 after
brisc/kmeans.pyx:889) and the NumPy oracle (oracle/knn.py).

Tolerance: the same nearest clusters and neighbour sets except at near-ties
within FP32 rounding of the squared norms (2e-6 relative, doubled), distances
within that rounding, run-to-run bit identity."""
import numpy as np
import pytest

from knn_cases import case, check_against

pytestmark = pytest.mark.gpu


def _run(c, **kw):
    from brisc_gb300 import knn
    n, k, cs = c["X"].shape[0], c["num_neighbors"], c["num_clusters_searched"]
    out = dict(neighbors=np.zeros((n, k), np.uint32), distances=np.zeros((n, k), np.float32),
               centroid_distances=np.zeros((n, cs), np.float32),
               nearest_clusters=np.zeros((n, cs), np.uint32))
    knn.knn_self(X=c["X"], sorted_order=c["sorted_order"], centroids=c["centroids"],
                 num_cells_per_cluster=c["num_cells_per_cluster"],
                 cell_norms=c["cell_norms"], num_neighbors=k,
                 num_clusters_searched=cs, chunk_size_kmeans=min(4096, n),
                 chunk_size_search=min(256, n), is_mac=False, num_threads=1, **out, **kw)
    return out


@pytest.mark.parametrize("name", ["knn_a", "knn_b"])
def test_knn_self_matches_reference(cuda, golden, name):
    c = case(golden("knn"), name)
    o = _run(c)
    check_against(c, o["neighbors"], o["distances"], o["nearest_clusters"],
                  o["centroid_distances"])


def test_knn_self_bit_identical_and_device_tensors(cuda, golden):
    """Two runs from host arrays and one on CUDA tensors (int32 holding the
    uint32 arrays) give the same bits."""
    import torch
    from brisc_gb300 import knn
    c = case(golden("knn"), "knn_a")
    a, b = _run(c), _run(c)
    for key in a:
        np.testing.assert_array_equal(a[key], b[key])
    T = lambda x: torch.from_numpy(np.ascontiguousarray(  # noqa: E731
        x.view(np.int32) if x.dtype == np.uint32 else x)).to(cuda)
    n, k, cs = c["X"].shape[0], c["num_neighbors"], c["num_clusters_searched"]
    dev = dict(neighbors=torch.zeros((n, k), dtype=torch.int32, device=cuda),
               distances=torch.zeros((n, k), dtype=torch.float32, device=cuda),
               centroid_distances=torch.zeros((n, cs), dtype=torch.float32, device=cuda),
               nearest_clusters=torch.zeros((n, cs), dtype=torch.int32, device=cuda))
    knn.knn_self(X=T(c["X"]), sorted_order=T(c["sorted_order"]),
                 centroids=T(c["centroids"]),
                 num_cells_per_cluster=T(c["num_cells_per_cluster"]),
                 cell_norms=T(c["cell_norms"]), num_neighbors=k,
                 num_clusters_searched=cs, **dev)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(dev["neighbors"].cpu().numpy().view(np.uint32),
                                  a["neighbors"])
    np.testing.assert_array_equal(dev["distances"].cpu().numpy(), a["distances"])


def _lloyd(X, nc, iters=3, seed=0):
    """A small deterministic k-means (random init + Lloyd steps) standing in
    for the reference's, to make knn_self inputs at sizes with no fixture."""
    rng = np.random.default_rng(seed)
    C = X[rng.choice(len(X), nc, replace=False)].astype(np.float64)
    X64 = X.astype(np.float64)
    for _ in range(iters):
        lab = np.argmin(-2 * X64 @ C.T + (C * C).sum(1), 1)
        for j in range(nc):
            if np.any(lab == j):
                C[j] = X64[lab == j].mean(0)
    lab = np.argmin(-2 * X64 @ C.T + (C * C).sum(1), 1)
    keep = np.unique(lab)
    remap = np.zeros(nc, np.int64)
    remap[keep] = np.arange(len(keep))
    lab, C = remap[lab], C[keep]
    order = np.argsort(C[:, 0])
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    lab, C = inv[lab], C[order]
    so = np.argsort(lab, kind="stable").astype(np.uint32)
    Xs = np.ascontiguousarray(X[so])
    norms = np.einsum("ij,ij->i", Xs, Xs).astype(np.float32)
    counts = np.bincount(lab, minlength=len(C)).astype(np.uint32)
    return Xs, so, np.ascontiguousarray(C.astype(np.float32)), counts, norms


@pytest.mark.parametrize("n,d,nc,k,cs", [(15000, 50, 120, 20, 24), (4000, 100, 40, 64, 40),
                                         (3000, 13, 30, 33, 30), (2500, 7, 250, 128, 200)])
def test_knn_self_matches_oracle(cuda, n, d, nc, k, cs):
    """Shapes beyond the fixtures: 50 and 100 dimensions, 33/64/128
    neighbours, up to 200 clusters searched, empty-ish clusters."""
    from knn_cases import knn_pcs
    from oracle import knn as oknn
    X = knn_pcs(n, d, 30, seed=n + d)
    Xs, so, C, counts, norms = _lloyd(X, nc)
    cs = min(cs, len(C))
    c = dict(X=Xs, sorted_order=so, centroids=C, num_cells_per_cluster=counts,
             cell_norms=norms, num_neighbors=k, num_clusters_searched=cs)
    nbr, dist, near, cdist = oknn.knn_self(Xs, so, C, counts, norms, k, cs)
    c.update(ref_neighbors=nbr, ref_distances=dist, ref_nearest=near, ref_cdist=cdist)
    o = _run(c)
    check_against(c, o["neighbors"], o["distances"], o["nearest_clusters"],
                  o["centroid_distances"])


@pytest.mark.parametrize("name", ["knn_a", "knn_b"])
def test_kmeans_matches_reference(cuda, golden, name):
    """GPU k-means (random initialisation, the reference's M-step order)
    against the reference's kmeans on the same PCs: the same iteration count,
    labels identical except at FP32 near-ties of the E step, centroids and
    cluster sizes accordingly."""
    from brisc_gb300 import knn
    from knn_cases import knn_pcs
    z = golden("knn")
    n, d, comps, seed, k, cs = (int(v) for v in z[f"{name}_shape"])
    X = knn_pcs(n, d, comps, seed)
    ref_c = z[f"{name}_km_final_centroids"]
    nc = ref_c.shape[0]
    out = dict(cluster_labels=np.zeros(n, np.uint32), min_distances=np.zeros(n, np.float32),
               cell_norms=np.zeros(n, np.float32),
               centroids=np.zeros((nc, d), np.float32),
               centroids_new=np.zeros((nc, d), np.float32),
               num_cells_per_cluster=np.zeros(nc, np.uint32))
    it = knn.kmeans(X=X, seed=0, chunk_size=min(4096, n), **out)
    assert it == int(z[f"{name}_km_iterations"])
    C = out["centroids_new"] if it & 1 else out["centroids"]
    same = (out["cluster_labels"] == z[f"{name}_km_cluster_labels"]).mean()
    assert same >= 0.999, same
    scale = np.abs(ref_c).max()
    if same == 1.0:  # same assignments: the reference's summation order
        np.testing.assert_allclose(C, ref_c, rtol=0, atol=2e-6 * scale)
        np.testing.assert_array_equal(out["num_cells_per_cluster"],
                                      z[f"{name}_km_num_cells_per_cluster"])
    else:
        np.testing.assert_allclose(C, ref_c, rtol=0, atol=1e-2 * scale)
    np.testing.assert_allclose(out["cell_norms"], z[f"{name}_cell_norms"][
        np.argsort(z[f"{name}_sorted_order"])], rtol=2e-6)


@pytest.mark.parametrize("name", ["knn_a", "knn_b"])
def test_neighbors_pipeline_matches_reference(cuda, golden, name):
    """brisc_gb300.knn.neighbors (GPU k-means, neighbors()'s preparation, GPU
    knn_self) against the reference's neighbours, both in the original cell
    order: the same sets except at near-ties."""
    from brisc_gb300 import knn
    from knn_cases import knn_pcs
    from oracle import knn as oknn
    z = golden("knn")
    n, d, comps, seed, k, cs = (int(v) for v in z[f"{name}_shape"])
    X = knn_pcs(n, d, comps, seed)
    so = z[f"{name}_sorted_order"]
    ref = np.empty_like(z[f"{name}_neighbors"])
    ref[so] = z[f"{name}_neighbors"]
    nbr, dist = knn.neighbors(X, num_neighbors=k,
                              num_clusters_searched=None if name == "knn_b" else cs)
    ident = np.arange(n, dtype=np.uint32)
    norms = np.einsum("ij,ij->i", X, X).astype(np.float32)
    same, worst = oknn.compare(X, ident, norms, nbr, ref)
    assert same >= 0.99 and worst <= 1.0, (same, worst)
