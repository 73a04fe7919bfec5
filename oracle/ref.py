"""ORACLE (test/baseline infrastructure): the reference's own compiled modules.

``load()`` imports brisc's ``pca``, ``normalize``, ``cysparse``, ``hvg`` and the
``ref_probe`` harness from ``oracle/_ref/<machine>/`` (built by
oracle/build_ref.py from the reference checkout, or from the generated C++
that travels with the repository when no checkout is present). Returns None
when neither is available.

``run_irlba`` calls the reference's ``irlba`` exactly as ``SingleCell.pca()``
does (brisc/single_cell.py:12037-12091): CSR for the matvec, the reference's
own ``csr_tocsc`` for the rmatvec copy, ``match_parallel=False``, inside
``threadpool_limits(1, 'blas')`` when threadpoolctl is available.
"""
from __future__ import annotations

import contextlib
import importlib
import os
import platform
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_mods = None


def _machine_dir() -> Path:
    return HERE / "_ref" / platform.machine().lower()


def available() -> bool:
    return (_machine_dir() / "brisc").exists() or (HERE / "_ref" / "gen").exists()


def load(build: bool = True):
    global _mods
    if _mods is not None:
        return _mods
    d = _machine_dir()
    pkg = d / "brisc"
    have = pkg.exists() and any(pkg.glob("pca*.so"))
    if not have and build:
        from . import build_ref
        try:
            if build_ref.have_reference():
                build_ref.cythonize(build_ref.reference_dir())
            build_ref.compile_all(os.cpu_count() or 4,
                                  modules=build_ref.BASELINE_MODULES)
        except Exception as e:  # noqa: BLE001 - reported to the caller
            print(f"[oracle.ref] reference build unavailable: {e}", file=sys.stderr)
            return None
        have = any(pkg.glob("pca*.so"))
    if not have:
        return None
    if str(d) not in sys.path:
        sys.path.insert(0, str(d))
    _mods = {}
    for name in ("cyutils", "pca", "normalize", "cysparse", "hvg", "kmeans", "knn",
                 "harmonize", "hdf5", "ref_probe"):
        try:
            _mods[name] = importlib.import_module(f"brisc.{name}")
        except ImportError:
            if name not in ("cysparse", "hvg", "kmeans", "knn", "harmonize", "hdf5"):
                raise
    return _mods


@contextlib.contextmanager
def _blas1():
    try:
        from threadpoolctl import threadpool_limits
    except ImportError:
        yield
        return
    with threadpool_limits(1, user_api="blas"):
        yield


def tocsc(indptr, indices, data, n_row: int, n_col: int, num_threads: int):
    """The reference's csr_tocsc (brisc/cysparse.pyx:1179) on int32/int64 arrays."""
    M = load()
    Bp = np.empty(n_col + 1, dtype=indptr.dtype)
    Bi = np.empty(indices.shape[0], dtype=indices.dtype)
    Bx = np.empty(data.shape[0], dtype=data.dtype)
    # bit views, as brisc/sparse.py:933-934 passes them (fused type bit_width)
    bits = np.uint32 if data.dtype.itemsize == 4 else np.uint64
    M["cysparse"].csr_tocsc(n_row, n_col, indptr, indices, data.view(bits), Bp,
                            Bi, Bx.view(bits), num_threads)
    return Bp, Bi, Bx


def normalize(indptr, indices, data, method: int, num_threads: int, qc=None):
    """The reference's normalize_csr (brisc/normalize.pyx:9)."""
    M = load()
    n = indptr.shape[0] - 1
    out = np.empty(data.shape[0], dtype=np.float32)
    rs = np.empty(n, dtype=np.uint64)
    q = np.array([], dtype=bool) if qc is None else np.ascontiguousarray(qc, dtype=bool)
    M["normalize"].normalize_csr(data, indices, indptr, q.view(np.int8), out, rs,
                                 n, method, num_threads)
    return out, rs


def run_irlba(indptr, indices, data_f32, n: int, g: int, k: int = 50,
              m: int = 100, tol: float = 1e-6, max_iterations: int = 100,
              seed: int = 0, num_threads: int | None = None,
              chunk_size: int = 1024, csc=None, match_parallel=None):
    """Returns (PCs, converged). `csc` = (indptr, indices, data) to reuse.

    Array selection follows brisc/single_cell.py:12037-12055 for CSR input:
    the rmatvec gets the CSC copy unless num_threads == 1 and not
    match_parallel, where it gets the CSR arrays again. match_parallel
    defaults to True for one thread (the reference tests' golden setting,
    tests/test_pca.py:9-10), so every thread count runs the same arithmetic.
    """
    M = load()
    num_threads = num_threads or os.cpu_count() or 1
    if match_parallel is None:
        match_parallel = num_threads == 1
    m = min(m, n, g)
    serial = num_threads == 1 and not match_parallel
    if serial:
        csc = (indptr, indices, data_f32)
    elif csc is None and "cysparse" in M:
        csc = tocsc(indptr, indices, data_f32, n, g, num_threads)
    elif csc is None:
        # cysparse is left out of the baseline build (24 MB of C++): scipy's
        # transpose keeps rows ascending inside each column, as csr_tocsc
        # does (brisc/cysparse.pyx:1179-1295), so the arrays are the same
        import scipy.sparse as sp
        t = sp.csr_matrix((data_f32, indices, indptr), shape=(n, g)).tocsc()
        t.sort_indices()
        csc = (t.indptr.astype(indptr.dtype), t.indices.astype(indices.dtype), t.data)
    PCs = np.zeros((n, k), dtype=np.float32)
    with _blas1():
        conv = M["pca"].irlba(
            data_matvec=data_f32, indices_matvec=indices, indptr_matvec=indptr,
            data_rmatvec=csc[2], indices_rmatvec=csc[1], indptr_rmatvec=csc[0],
            num_cells=n, num_genes=g, k=k, subspace_size=m, tolerance=tol,
            max_iterations=max_iterations, seed=seed,
            match_parallel=bool(match_parallel), is_csr=True,
            num_threads=num_threads, chunk_size=chunk_size, PCs=PCs)
    return PCs, bool(conv)


def run_kmeans_for_knn(PCs, num_neighbors: int = 20, num_clusters=None,
                       num_clusters_searched=None, num_kmeans_iterations: int = 2,
                       kmeans_tolerance: float = 1e-2, kmeans_barbar: bool = False,
                       num_init_iterations: int = 5, oversampling_factor: float = 1,
                       chunk_size_kmeans=None, chunk_size_search=None, seed: int = 0,
                       num_threads: int | None = None) -> dict:
    """The k-means half of the reference's neighbors() on a float32 PCs array
    (every cell passing QC): its compiled kmeans (brisc/kmeans.pyx:889), then
    the argument preparation of brisc/single_cell.py:12451-12611 -- default
    cluster counts and chunk sizes, empty-cluster removal, the minimum number
    of clusters searched, centroids ordered by PC 1, cells sorted by cluster.
    Returns every input knn_self (brisc/knn.pyx:13) takes, as a dict, plus
    the raw kmeans outputs under "kmeans"."""
    X = np.ascontiguousarray(PCs, dtype=np.float32)
    num_threads = num_threads or os.cpu_count() or 1
    n, d = X.shape
    if num_clusters is None:
        num_clusters = max(1, int(np.ceil(min(4 * np.sqrt(n), n / 100))))
    if num_clusters_searched is None:
        num_clusters_searched = min(64, num_clusters)
    if chunk_size_kmeans is None:
        chunk_size_kmeans = min(4096, n)
    if chunk_size_search is None:
        chunk_size_search = min(256, n)
    raw = run_kmeans(X, num_clusters, num_kmeans_iterations=num_kmeans_iterations,
                     kmeans_tolerance=kmeans_tolerance, kmeans_barbar=kmeans_barbar,
                     num_init_iterations=num_init_iterations,
                     oversampling_factor=oversampling_factor,
                     chunk_size=chunk_size_kmeans, seed=seed, num_threads=num_threads)
    it, labels, centroids, centroids_new, counts, cell_norms = (
        raw["iterations"], raw["cluster_labels"].copy(), raw["centroids"],
        raw["centroids_new"], raw["num_cells_per_cluster"].copy(), raw["cell_norms"])
    if it & 1:
        centroids = centroids_new
    non_empty = counts > 0
    if not non_empty.all():
        centroids = centroids[non_empty]
        counts = counts[non_empty]
        num_clusters = len(centroids)
        remap = np.zeros(len(non_empty), dtype=np.uint32)
        remap[non_empty] = np.arange(num_clusters, dtype=np.uint32)
        labels = remap[labels]
    cumsum = np.sort(counts).cumsum(dtype=np.uint64)
    min_searched = int(np.searchsorted(cumsum, num_neighbors + 1)) + 1
    num_clusters_searched = min(max(num_clusters_searched, min_searched), num_clusters)
    order = np.argsort(centroids[:, 0]).astype(np.uint32)
    centroids = np.ascontiguousarray(centroids[order])
    counts = np.ascontiguousarray(counts[order])
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order), dtype=np.uint32)
    labels = inv[labels]
    sorted_order = np.argsort(labels).astype(np.uint32)
    return dict(X=np.ascontiguousarray(X[sorted_order]), sorted_order=sorted_order,
                centroids=centroids, num_cells_per_cluster=counts,
                cell_norms=np.ascontiguousarray(cell_norms[sorted_order]),
                num_neighbors=int(num_neighbors),
                num_clusters_searched=int(num_clusters_searched),
                chunk_size_kmeans=int(chunk_size_kmeans),
                chunk_size_search=int(chunk_size_search), kmeans=raw)


def run_kmeans(X, num_clusters: int, num_kmeans_iterations: int = 2,
               kmeans_tolerance: float = 1e-2, kmeans_barbar: bool = False,
               num_init_iterations: int = 5, oversampling_factor: float = 1,
               chunk_size: int | None = None, seed: int = 0,
               num_threads: int | None = None) -> dict:
    """The reference's compiled kmeans (brisc/kmeans.pyx:889) called as
    neighbors() calls it (brisc/single_cell.py:12515-12545). Returns its raw
    outputs: iterations, cluster_labels, centroids, centroids_new (the final
    centroids are in centroids_new when iterations is odd), the cluster
    sizes, min_distances and cell_norms."""
    M = load()
    X = np.ascontiguousarray(X, dtype=np.float32)
    n, d = X.shape
    num_threads = num_threads or os.cpu_count() or 1
    chunk_size = chunk_size or min(4096, n)
    out = dict(cluster_labels=np.zeros(n, dtype=np.uint32),
               min_distances=np.zeros(n, dtype=np.float32),
               cell_norms=np.zeros(n, dtype=np.float32),
               centroids=np.empty((num_clusters, d), dtype=np.float32),
               centroids_new=np.empty((num_clusters, d), dtype=np.float32),
               num_cells_per_cluster=np.empty(num_clusters, dtype=np.uint32))
    with _blas1():
        out["iterations"] = int(M["kmeans"].kmeans(
            X=X, kmeans_barbar=kmeans_barbar, num_init_iterations=num_init_iterations,
            num_kmeans_iterations=num_kmeans_iterations, tolerance=kmeans_tolerance,
            oversampling_factor=oversampling_factor, seed=seed, chunk_size=chunk_size,
            is_mac=False, num_threads=num_threads, **out))
    return out


def run_knn_self(prep: dict, num_threads: int | None = None):
    """The reference's knn_self (brisc/knn.pyx:13) on run_kmeans_for_knn's
    outputs. Returns (neighbors, distances) in cluster-sorted row order, as
    knn_self leaves them (squared Euclidean distances, self excluded,
    neighbour indices already mapped to the original cell order)."""
    M = load()
    n = prep["X"].shape[0]
    k, cs = prep["num_neighbors"], prep["num_clusters_searched"]
    neighbors = np.zeros((n, k), dtype=np.uint32)
    distances = np.zeros((n, k), dtype=np.float32)
    cdist = np.zeros((n, cs), dtype=np.float32)
    near = np.zeros((n, cs), dtype=np.uint32)
    with _blas1():
        M["knn"].knn_self(
            X=prep["X"], sorted_order=prep["sorted_order"],
            centroids=prep["centroids"],
            num_cells_per_cluster=prep["num_cells_per_cluster"],
            neighbors=neighbors, distances=distances, cell_norms=prep["cell_norms"],
            centroid_distances=cdist, nearest_clusters=near, num_neighbors=k,
            num_clusters_searched=cs, chunk_size_kmeans=prep["chunk_size_kmeans"],
            chunk_size_search=prep["chunk_size_search"], is_mac=False,
            num_threads=num_threads or os.cpu_count() or 1)
    return neighbors, distances, near, cdist


def run_harmonize(PCs, batch_labels, num_batches: int, num_clusters=None,
                  max_iterations: int = 10, num_kmeans_iterations: int = 25,
                  kmeans_tolerance: float = 1e-2, max_clustering_iterations: int = 5,
                  block_proportion: float = 0.05, tolerance: float = 0.01,
                  early_stopping: bool = False, clustering_tolerance: float = 1e-3,
                  theta: float = 2, tau: float = 0, alpha: float = 0.2,
                  sigma: float = 0.1, chunk_size_kmeans=None, chunk_size_Harmony=None,
                  seed: int = 0, num_threads: int | None = None) -> dict:
    """The reference's harmonize() core for one dataset (every cell passing
    QC): row-normalised PCs (brisc/harmonize.pyx:244 normalize_rows), its
    kmeans on them for the initial centroids, and harmony
    (brisc/harmonize.pyx:269), with the argument preparation of
    brisc/single_cell.py:13777-13876. Returns Z (the Harmony embedding), R,
    the initial Y and the k-means iteration count."""
    M = load()
    H = M["harmonize"]
    PCs = np.ascontiguousarray(PCs, dtype=np.float32)
    n, d = PCs.shape
    num_threads = num_threads or os.cpu_count() or 1
    if num_clusters is None:
        num_clusters = max(min(100, int(round(n / 30))), 1)
    chunk_size_kmeans = chunk_size_kmeans or min(4096, n)
    chunk_size_Harmony = chunk_size_Harmony or min(256, n)
    Z = np.empty((n, d), dtype=np.float32)
    H.normalize_rows(arr=PCs, out=Z, num_threads=num_threads)
    km = run_kmeans(Z, num_clusters, num_kmeans_iterations=num_kmeans_iterations,
                    kmeans_tolerance=kmeans_tolerance, chunk_size=chunk_size_kmeans,
                    seed=seed, num_threads=num_threads)
    Y0 = km["centroids_new"] if km["iterations"] & 1 else km["centroids"]
    Y = np.ascontiguousarray(Y0[:num_clusters]).copy()
    Y_init = Y.copy()
    R = np.empty((n, num_clusters), dtype=np.float32)
    with _blas1():
        H.harmony(PCs=PCs, Z=Z, Y=Y, R=R,
                  batch_labels=np.ascontiguousarray(batch_labels, dtype=np.uint32),
                  num_batches=num_batches, max_iterations=max_iterations,
                  max_clustering_iterations=max_clustering_iterations,
                  block_proportion=block_proportion, tolerance=tolerance,
                  early_stopping=early_stopping, clustering_tolerance=clustering_tolerance,
                  theta=theta, tau=tau, alpha=alpha, sigma=sigma,
                  chunk_size=chunk_size_Harmony, seed=seed, verbose=False,
                  num_threads=num_threads)
    return dict(Z=Z, R=R, Y_init=Y_init, Y=Y, kmeans_iterations=km["iterations"],
                num_clusters=num_clusters)


def run_read_all_datasets(path, datasets, num_threads: int | None = None):
    """The reference's contiguous-dataset reader (brisc/hdf5.pyx:163
    read_all_datasets) as SingleCell._read_parallel calls it for large
    fixed-width datasets (brisc/single_cell.py:1964-2200): one pread slice per
    thread of every dataset, into NumPy arrays. ``datasets`` is a list of
    (file_offset, dtype, num_elements); the offsets come from the caller (the
    reference gets them from h5py, absent here). Returns the arrays."""
    M = load()
    H = M["hdf5"]
    num_threads = num_threads or os.cpu_count() or 1
    arrays = [np.empty(int(n), dtype=dt) for _, dt, n in datasets]
    u64 = lambda v: np.asarray(v, dtype=np.uint64)  # noqa: E731
    fd = os.open(path, os.O_RDONLY)
    try:
        H.read_all_datasets(
            fd, arrays, u64([off for off, _, _ in datasets]), u64([]), u64([]), u64([]),
            u64([0] * (num_threads + 1)), u64([]), u64([]), 8, 8, num_threads)
    finally:
        os.close(fd)
    return arrays
