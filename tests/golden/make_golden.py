"""Generate tests/golden/*.npz from the reference's own compiled modules.

Run in a checkout that has the reference (built into oracle/_ref by
oracle/build_ref.py). Every fixture stores its inputs as well as the
reference's outputs, so the tests never regenerate data:

* rng.npz        PCG32 outputs, Box-Muller normals and pca.pyx's normalised
                 start vector (brisc/cyutils.pyx:1153-1232, pca.pyx:801-806)
                 for several seeds.
* normalize.npz  normalize_csr outputs (brisc/normalize.pyx:9) for methods
                 0/1/2, with and without a QC mask, on a small NB count matrix.
* tocsc.npz      csr_tocsc (brisc/cysparse.pyx:1179) of the same matrix.
* irlba.npz      irlba PCs (brisc/pca.pyx:661) on clustered NB matrices whose
                 top singular values are separated, plus one flat-spectrum case.
* parity50k.npz  irlba at the 50,000 x 2,000 configuration (50 PCs, subspace
                 100, seed 0) on the flat and the 13-cluster NB matrix: the
                 singular values, the right vectors A^T PCs / s^2 (genes x 50,
                 FP64 from the reference's PCs), the convergence flag, the
                 reference's own accuracy against the FP64 oracle, and a
                 fingerprint of the seeded input.
* knn.npz        the reference's kmeans (brisc/kmeans.pyx:889; labels, final
                 centroids, sizes, min distances, iterations) and knn_self
                 (brisc/knn.pyx:13) after neighbors()'s argument
                 preparation (brisc/single_cell.py:12451-12611), on seeded
                 Gaussian-mixture "PCs" (regenerated from the seed, with a
                 fingerprint): the k-means outputs knn_self takes and its
                 neighbours, distances and nearest clusters.
* harmony.npz    the reference's harmonize() core (brisc/single_cell.py:
                 13776-13875: normalize_rows, kmeans, harmony at
                 brisc/harmonize.pyx:269) on seeded batch-shifted "PCs"
                 (synth.batched_pcs, regenerated from the seed, with a
                 fingerprint): the k-means centroids harmony starts from, the
                 embedding Z, the first rows of R and the k-means iteration
                 count, for the default settings, for one case with early
                 stopping, a larger block and a smaller chunk, and for
                 tau > 0 (where the reference's output is NaN).
* hvg.npz        gene_mean_and_variance_csr/_csc and clipped_sum_csr/_csc
                 (brisc/hvg.pyx) on an NB count matrix with a few large
                 counts, over all cells and over a cell subset, uint32 and
                 float32 counts, int32 and int64 indices.

    python tests/golden/make_golden.py          # every fixture
    python tests/golden/make_golden.py hvg      # hvg.npz only
    python tests/golden/make_golden.py parity   # parity50k.npz only
    python tests/golden/make_golden.py knn      # knn.npz only
    python tests/golden/make_golden.py harmony  # harmony.npz only
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from synth import nb_counts  # noqa: E402
from oracle import ref  # noqa: E402

OUT = Path(__file__).resolve().parent
SEEDS = [0, 1, 7, 42, 12345, 2**63 + 5]


def make_hvg(M) -> None:
    import scipy.sparse as sp
    H = M["hvg"]
    C = nb_counts(900, 160, seed=23, density=0.1, workers=1)
    A = sp.csr_matrix((C.data.astype(np.uint32), C.indices, C.indptr),
                      shape=(C.num_cells, C.num_genes))
    big = np.random.default_rng(5).random(A.nnz) < 0.003  # counts above 2^16
    A.data[big] = A.data[big] * 4099 + 70000
    B = A.tocsc()
    B.sort_indices()
    n, g = A.shape
    cells = np.arange(0, n, 3, dtype=np.int64)
    mask = np.zeros(n, np.int8)
    mask[cells] = 1
    clip = (np.random.default_rng(6).random(g) * 12 + 0.5).astype(np.float32)
    out = {"n": np.int64(n), "g": np.int64(g), "csr_data": A.data, "csr_indices": A.indices,
           "csr_indptr": A.indptr, "csc_data": B.data, "csc_indices": B.indices,
           "csc_indptr": B.indptr, "cells": cells, "mask": mask, "clip": clip}
    for dt in (np.uint32, np.float32):
        for it in (np.int32, np.int64):
            tag = f"{np.dtype(dt).name}_{np.dtype(it).name}"
            ad, ai, ap = A.data.astype(dt), A.indices.astype(it), A.indptr.astype(it)
            bd, bi, bp = B.data.astype(dt), B.indices.astype(it), B.indptr.astype(it)
            for sub in ("all", "sub"):
                c = cells if sub == "sub" else np.zeros(0, np.int64)
                mk = mask if sub == "sub" else np.zeros(0, np.int8)
                nc = len(cells) if sub == "sub" else n
                for form in ("csr", "csc"):
                    m_, v_, z_ = (np.zeros(g, np.float32), np.zeros(g, np.float32),
                                  np.zeros(g, np.uint32))
                    if form == "csr":
                        H.gene_mean_and_variance_csr(ad, ai, ap, c, nc, g, m_, v_, z_, 4)
                    else:
                        H.gene_mean_and_variance_csc(bd, bi, bp, mk, nc, g, m_, v_, z_, 4)
                    b_, q_ = np.zeros(g, np.float32), np.zeros(g, np.float32)
                    if form == "csr":
                        H.clipped_sum_csr(ad, ai, ap, nc, g, c, clip, b_, q_, 4)
                    else:
                        H.clipped_sum_csc(bd, bi, bp, mk, clip, b_, q_, 4)
                    key = f"{form}_{tag}_{sub}"
                    out.update({f"{key}_mean": m_, f"{key}_var": v_, f"{key}_nnz": z_,
                                f"{key}_bsum": b_, f"{key}_bsq": q_})
    np.savez_compressed(OUT / "hvg.npz", **out)


def make_parity() -> None:
    import json
    from oracle import accuracy as A
    out = {}
    for name in A.PARITY_CASES:
        c, xn = A.parity_input(name)
        n, g, k, m = c.num_cells, c.num_genes, 50, 100
        ip32, ix32 = c.indptr.astype(np.int32), c.indices.astype(np.int32)
        pcs, conv = ref.run_irlba(ip32, ix32, xn, n, g, k, m, 1e-6, 100, seed=0,
                                  num_threads=8, match_parallel=False)
        ip, ix = c.indptr.astype(np.int64), c.indices.astype(np.int64)
        mean, sd = A.gene_moments64(ip, ix, xn, n, g)
        G = A.gram64(ip, ix, xn, n, g, mean, sd)
        S, V = A.truth(G, k + 1)
        Vr = A.right_vectors(ip, ix, xn, n, g, mean, sd, pcs)
        rep = A.solution_report(pcs, Vr, S, V, G, k)
        out[f"{name}_fingerprint"] = A.fingerprint(c.indptr, c.indices, c.data)
        out[f"{name}_S"] = np.linalg.norm(pcs.astype(np.float64), axis=0)
        out[f"{name}_V"] = Vr.astype(np.float32)
        out[f"{name}_converged"] = np.array(conv)
        out[f"{name}_report"] = np.array(json.dumps(rep))
        print(name, "converged", conv, "max rel sv", rep["max_rel_sv_error"],
              "gapped", rep["gapped_j"], "max top-j angle", rep["max_top_j_angle"])
    np.savez_compressed(OUT / "parity50k.npz", **out)


KNN_CASES = {  # name: (cells, dims, components, seed, num_neighbors, clusters searched)
    "knn_a": (8000, 20, 24, 3, 12, 12),
    "knn_b": (3000, 8, 10, 4, 5, None),
}


def knn_pcs(n: int, d: int, comps: int, seed: int) -> np.ndarray:
    """Seeded stand-in for principal components (synth.pca_like), regenerated
    by the tests from the seed (numpy's Generator streams are stable)."""
    from synth import pca_like
    return pca_like(n, d, comps, seed)


def make_knn() -> None:
    import hashlib
    out = {}
    for name, (n, d, comps, seed, k, cs) in KNN_CASES.items():
        X = knn_pcs(n, d, comps, seed)
        prep = ref.run_kmeans_for_knn(X, num_neighbors=k, num_clusters_searched=cs,
                                      seed=0, num_threads=1)
        nbr, dist, near, cdist = ref.run_knn_self(prep, num_threads=1)
        out[f"{name}_shape"] = np.array([n, d, comps, seed, k, prep["num_clusters_searched"]])
        out[f"{name}_fingerprint"] = np.array(hashlib.sha256(X.tobytes()).hexdigest())
        for key in ("sorted_order", "centroids", "num_cells_per_cluster", "cell_norms"):
            out[f"{name}_{key}"] = prep[key]
        km = prep["kmeans"]
        out[f"{name}_km_iterations"] = np.array(km["iterations"])
        for key in ("cluster_labels", "num_cells_per_cluster", "min_distances"):
            out[f"{name}_km_{key}"] = km[key]
        out[f"{name}_km_final_centroids"] = (km["centroids_new"] if km["iterations"] & 1
                                             else km["centroids"])
        out[f"{name}_neighbors"] = nbr
        out[f"{name}_distances"] = dist
        out[f"{name}_nearest_clusters"] = near
        out[f"{name}_centroid_distances"] = cdist
        print(name, "clusters", len(prep["centroids"]), "searched",
              prep["num_clusters_searched"])
    np.savez_compressed(OUT / "knn.npz", **out)


HARMONY_CASES = {  # name: (cells, dims, components, batches, seed, harmony keywords)
    "harm_a": (3000, 20, 12, 3, 9, {}),
    "harm_b": (2500, 30, 8, 4, 11, dict(num_clusters=40, early_stopping=True,
                                         block_proportion=0.1, chunk_size_Harmony=100,
                                         max_clustering_iterations=6, seed=3)),
    # tau > 0: the reference's discount negates an unsigned count, so its
    # theta is -inf and its output NaN (harmonize.pyx:416)
    "harm_tau": (800, 10, 5, 2, 13, dict(tau=5.0, max_iterations=2)),
}
HARMONY_R_ROWS = 400  # rows of R stored


def make_harmony() -> None:
    import hashlib
    import json
    from synth import batched_pcs
    out = {}
    for name, (n, d, comps, B, seed, kw) in HARMONY_CASES.items():
        X, labels = batched_pcs(n, d, comps, B, seed)
        r = ref.run_harmonize(X, labels, B, num_threads=1, **kw)
        out[f"{name}_shape"] = np.array([n, d, comps, B, seed])
        out[f"{name}_kwargs"] = np.array(json.dumps(kw))
        out[f"{name}_fingerprint"] = np.array(
            hashlib.sha256(X.tobytes() + labels.tobytes()).hexdigest())
        out[f"{name}_Y_init"] = r["Y_init"]
        out[f"{name}_Z"] = r["Z"]
        out[f"{name}_R_head"] = r["R"][:HARMONY_R_ROWS]
        out[f"{name}_kmeans_iterations"] = np.array(r["kmeans_iterations"])
        print(name, "clusters", r["num_clusters"], "k-means iterations",
              r["kmeans_iterations"])
    np.savez_compressed(OUT / "harmony.npz", **out)


def main() -> int:
    M = ref.load()
    if M is None:
        print("reference modules unavailable", file=sys.stderr)
        return 1
    if sys.argv[1:] == ["parity"]:
        make_parity()
        return 0
    if sys.argv[1:] == ["knn"]:
        make_knn()
        return 0
    if sys.argv[1:] == ["harmony"]:
        make_harmony()
        return 0
    if "hvg" in M:
        make_hvg(M)
    if "knn" in M and not sys.argv[1:]:
        make_knn()
    if "harmonize" in M and not sys.argv[1:]:
        make_harmony()
    if sys.argv[1:] == ["hvg"]:
        return 0
    probe = M["ref_probe"]

    rng = {}
    for i, s in enumerate(SEEDS):
        rng[f"seed_{i}"] = np.uint64(s)
        rng[f"rand_{i}"] = probe.raw_rand(s, 64)
        rng[f"normals_{i}"] = probe.raw_normals(s, 4096)
        rng[f"start_{i}"] = probe.start_vector(s, 2000)
    rng["start_small"] = probe.start_vector(0, 37)
    np.savez_compressed(OUT / "rng.npz", **rng)

    C = nb_counts(800, 150, seed=11, density=0.08, workers=1)
    ip32 = C.indptr.astype(np.int32)
    ix32 = C.indices.astype(np.int32)
    data_f = C.data.astype(np.float32)
    qc = (np.arange(C.num_cells) % 5) != 2
    norm = {"indptr": ip32, "indices": ix32, "counts": C.data, "qc": qc}
    for method in (0, 1, 2):
        for tag, q in (("all", None), ("qc", qc)):
            out, rs = ref.normalize(ip32, ix32, data_f, method, 1, q)
            out4, rs4 = ref.normalize(ip32, ix32, data_f, method, 4, q)
            assert np.array_equal(out, out4) and np.array_equal(rs, rs4)
            norm[f"m{method}_{tag}"] = out
            norm[f"rowsums_{tag}"] = rs
    np.savez_compressed(OUT / "normalize.npz", **norm)

    bp, bi, bx = ref.tocsc(ip32, ix32, data_f, C.num_cells, C.num_genes, 4)
    ip64, ix64 = C.indptr.astype(np.int64), C.indices.astype(np.int64)
    bp64, bi64, bx64 = ref.tocsc(ip64, ix64, data_f, C.num_cells, C.num_genes, 3)
    np.savez_compressed(OUT / "tocsc.npz", indptr=ip32, indices=ix32, data=data_f,
                        n_col=C.num_genes, Bp=bp, Bi=bi, Bx=bx, Bp64=bp64,
                        Bi64=bi64, Bx64=bx64)

    cases = [  # (name, cells, genes, clusters, density, k, m, seed)
        ("clustered_a", 5000, 500, 12, 0.08, 10, 20, 3),
        ("clustered_b", 4000, 400, 13, 0.05, 8, 24, 5),
        ("flat", 3000, 300, 0, 0.08, 10, 40, 3),
    ]
    ir = {}
    for name, n, g, cl, dens, k, m, seed in cases:
        Cm = nb_counts(n, g, seed=seed, density=dens, clusters=cl, workers=1)
        ip = Cm.indptr.astype(np.int32)
        ix = Cm.indices.astype(np.int32)
        x, _ = ref.normalize(ip, ix, Cm.data.astype(np.float32), 0, 4)
        pcs, conv = ref.run_irlba(ip, ix, x, Cm.num_cells, g, k, m, 1e-6, 100,
                                  seed=0, num_threads=4)
        pcs1, conv1 = ref.run_irlba(ip, ix, x, Cm.num_cells, g, k, m, 1e-6, 100,
                                    seed=0, num_threads=1)
        assert np.array_equal(pcs, pcs1), "reference not thread-count invariant"
        ir[f"{name}_indptr"] = ip
        ir[f"{name}_indices"] = ix
        ir[f"{name}_counts"] = Cm.data
        ir[f"{name}_data"] = x
        ir[f"{name}_shape"] = np.array([Cm.num_cells, g, k, m])
        ir[f"{name}_pcs"] = pcs
        ir[f"{name}_converged"] = np.array(conv)
    np.savez_compressed(OUT / "irlba.npz", **ir)
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)
    return 0


if __name__ == "__main__":
    sys.exit(main())
