"""The oracle pinned against the reference's own outputs (tests/golden/).

CPU only. Integer and byte work must match bit for bit; float work within the
stated tolerance.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import clib, dense
from oracle import irlba as oirlba


def _ulp(a, b):
    return int(np.max(np.abs(a.view(np.int32).astype(np.int64) -
                             b.view(np.int32).astype(np.int64))))


def test_pcg32_and_box_muller_bit_exact(golden):
    z = golden("rng")
    i = 0
    while f"seed_{i}" in z.files:
        seed = int(z[f"seed_{i}"])
        assert np.array_equal(clib.raw_rand(seed, 64), z[f"rand_{i}"])
        assert np.array_equal(clib.raw_normals(seed, 4096), z[f"normals_{i}"])
        i += 1
    assert i >= 5


def test_start_vector_within_ulps(golden):
    # The normals are bit-exact; the reference binary sums the squares for the
    # norm in vectorised order (-Ofast), so the normalised vector may differ
    # by a few ulp from the sequential sum written in pca.pyx:804.
    z = golden("rng")
    i = 0
    while f"seed_{i}" in z.files:
        seed = int(z[f"seed_{i}"])
        sv = clib.start_vector(seed, 2000)
        assert _ulp(sv, z[f"start_{i}"]) <= 8
        i += 1
    assert _ulp(clib.start_vector(0, 37), z["start_small"]) <= 8


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("tag", ["all", "qc"])
def test_normalize_bit_exact(golden, method, tag):
    z = golden("normalize")
    qc = z["qc"] if tag == "qc" else None
    out, rs, isf, post = clib.normalize_csr(z["indptr"], z["counts"], method, qc)
    assert np.array_equal(rs, z[f"rowsums_{tag}"])
    assert np.array_equal(out, z[f"m{method}_{tag}"])


def test_csr_tocsc_bit_exact(golden):
    z = golden("tocsc")
    bp, bi, bx = clib.csr_tocsc(z["indptr"], z["indices"], z["data"], int(z["n_col"]))
    assert np.array_equal(bp, z["Bp"]) and np.array_equal(bi, z["Bi"])
    assert np.array_equal(bx.view(np.uint32), z["Bx"].view(np.uint32))
    assert np.array_equal(z["Bp"], z["Bp64"]) and np.array_equal(z["Bi"], z["Bi64"])


def test_thread_offsets_balance():
    ip = np.array([0, 5, 5, 9, 30, 31, 40, 41, 60], dtype=np.int64)
    off = clib.thread_offsets(ip, 3)
    assert off[0] == 0 and off[-1] == 8 and np.all(np.diff(off.astype(int)) >= 0)


def _case(z, name):
    n, g, k, m = (int(v) for v in z[f"{name}_shape"])
    X = sp.csr_matrix((z[f"{name}_data"], z[f"{name}_indices"], z[f"{name}_indptr"]),
                      shape=(n, g))
    return X, k, m


@pytest.mark.parametrize("passes", [1, 0])
@pytest.mark.parametrize("name", ["clustered_a", "clustered_b"])
def test_oracle_irlba_matches_reference(golden, name, passes):
    """The reference's single pass, and the adaptive mode (a second U-side
    pass only where the first cancels, two V-side passes), both agree with
    the reference's own PCs."""
    z = golden("irlba")
    X, k, m = _case(z, name)
    ref_pcs = z[f"{name}_pcs"]
    o = oirlba.irlba(X, k, m, reorth_passes=passes)
    assert o["converged"] == bool(z[f"{name}_converged"])
    s_ref = dense.sv_from_pcs(ref_pcs)
    s_or = dense.sv_from_pcs(o["PCs"])
    assert np.max(np.abs(s_or - s_ref) / s_ref) < 1e-5
    assert dense.max_angle(o["PCs"], ref_pcs) < 1e-3
    # sign-aligned per-PC agreement
    a = dense.align_signs(o["PCs"], ref_pcs)
    cos = np.sum(a * ref_pcs, 0) / np.linalg.norm(a, axis=0) / np.linalg.norm(ref_pcs, axis=0)
    assert np.min(cos) > 1 - 1e-5


def test_reference_vs_fp64(golden):
    """Pins the FP64 oracle: the reference's PCs meet the accuracy gates on
    the gapped fixtures (rel SV <= 1e-4; principal angle <= 1e-3 rad)."""
    z = golden("irlba")
    for name in ["clustered_a", "clustered_b"]:
        X, k, m = _case(z, name)
        S, U, Vt = dense.top_svd(X, k + 2)
        pcs = z[f"{name}_pcs"]
        assert dense.rel_sv_error(pcs, S).max() < 1e-4
        gaps = dense.gap_mask(S, k, 0.01)
        assert gaps, "fixture should have separated singular values"
        j = max(gaps)
        assert dense.max_angle(pcs[:, :j], U[:, :j]) < 1e-3


def test_flat_spectrum_singular_values(golden):
    z = golden("irlba")
    X, k, m = _case(z, "flat")
    S, U, Vt = dense.top_svd(X, k + 2)
    o = oirlba.irlba(X, k, m, reorth_passes=2)
    assert dense.rel_sv_error(z["flat_pcs"], S).max() < 1e-4
    assert dense.rel_sv_error(o["PCs"], S).max() < 1e-4


HVG_TAGS = ["uint32_int32", "uint32_int64", "float32_int32", "float32_int64"]


def hvg_case(z, form, tag):
    """(data, indices, indptr) of the hvg fixture in one dtype combination."""
    dt, it = (np.dtype(t) for t in tag.split("_"))
    return (z[f"{form}_data"].astype(dt), z[f"{form}_indices"].astype(it),
            z[f"{form}_indptr"].astype(it))


@pytest.mark.parametrize("sub", ["all", "sub"])
@pytest.mark.parametrize("form", ["csr", "csc"])
@pytest.mark.parametrize("tag", HVG_TAGS)
def test_hvg_oracle_bit_exact(golden, tag, form, sub):
    """The HVG restatement against the reference's own outputs
    (brisc/hvg.pyx), integer and float results alike, bit for bit."""
    from oracle import hvg as oh
    z = golden("hvg")
    n, g = int(z["n"]), int(z["g"])
    d, ix, ip = hvg_case(z, form, tag)
    cells = z["cells"] if sub == "sub" else np.zeros(0, np.int64)
    mask = z["mask"] if sub == "sub" else np.zeros(0, np.int8)
    nc = len(cells) if sub == "sub" else n
    key = f"{form}_{tag}_{sub}"
    if form == "csr":
        m, v, c = oh.gene_mean_and_variance_csr(d, ix, ip, cells, nc, g)
        b, q = oh.clipped_sum_csr(d, ix, ip, nc, g, cells, z["clip"])
    else:
        m, v, c = oh.gene_mean_and_variance_csc(d, ix, ip, mask, nc, g)
        b, q = oh.clipped_sum_csc(d, ix, ip, mask, z["clip"])
    for got, name in ((m, "mean"), (v, "var"), (c, "nnz"), (b, "bsum"), (q, "bsq")):
        assert np.array_equal(got, z[f"{key}_{name}"]), name


def test_hvg_oracle_fma_forms():
    """The clipped sums are fused multiply-adds in the reference's build (the
    fixture above pins that); the restatement's fma rounds once: for
    a = b = 1 + 2^-12, c = -1 it keeps the 2^-24 term that two roundings
    lose."""
    from oracle import hvg as oh
    a = np.float32(1 + 2.0 ** -12)
    one = np.float32(-1)
    assert oh.fma_f32(a, a, one) == np.float32(2.0 ** -11 + 2.0 ** -24)
    assert np.float32(np.float32(a * a) + one) == np.float32(2.0 ** -11)
    assert oh.fma_f32(np.float32(0), np.float32(5), np.float32(-2.5)) == np.float32(-2.5)
    assert oh.fma_f32(np.float32(3e38), np.float32(10), np.float32(0)) == np.float32(np.inf)


def test_oracle_adaptive_mode_second_passes_where_needed(golden):
    """The adaptive restatement (reorth_passes=0) takes a second pass only
    where the first cancels: none on an NB fixture, some on a near-low-rank
    matrix, and both meet the FP64 singular-value gate."""
    z = golden("irlba")
    Xb, kb, mb = _case(z, "clustered_b")
    ob = oirlba.irlba(Xb, kb, mb, reorth_passes=0)
    assert ob["second_passes"] == 0 and ob["second_passes_v"] == 0
    Sb, _, _ = dense.top_svd(Xb, kb + 2)
    assert dense.rel_sv_error(ob["PCs"], Sb).max() < 1e-4
    rng = np.random.default_rng(0)
    n, g, r = 4000, 400, 8
    W = rng.random((n, r)) * (rng.random((n, r)) < 0.3)
    H = rng.random((r, g)) * (rng.random((r, g)) < 0.5)
    A = W @ H
    A = A + 1e-3 * rng.random((n, g)) * (A > 0)
    X = sp.csr_matrix(A.astype(np.float32))
    o = oirlba.irlba(X, 6, 16, reorth_passes=0)
    assert 0 < o["second_passes"] < o["steps"] - 1
    S, U, Vt = dense.top_svd(X.astype(np.float64), 8)
    assert dense.rel_sv_error(o["PCs"], S).max() < 1e-4


@pytest.mark.parametrize("name", ["knn_a", "knn_b"])
def test_knn_oracle_matches_reference(golden, name):
    """oracle/knn.py (the NumPy restatement of brisc/knn.pyx:13) against the
    compiled reference's knn_self on the fixture's k-means outputs: the same
    nearest clusters and neighbour sets up to FP32 near-ties, distances
    within FP32 rounding of the squared norms."""
    from knn_cases import case, check_against
    from oracle import knn as oknn
    c = case(golden("knn"), name)
    nbr, dist, near, cdist = oknn.knn_self(
        c["X"], c["sorted_order"], c["centroids"], c["num_cells_per_cluster"],
        c["cell_norms"], c["num_neighbors"], c["num_clusters_searched"])
    check_against(c, nbr, dist, near, cdist)


@pytest.mark.parametrize("name", ["harm_a", "harm_b"])
def test_harmony_oracle_matches_reference(golden, name):
    """oracle/harmony.py (the NumPy restatement of brisc/harmonize.pyx:269)
    against the compiled reference's harmony from the same k-means centroids:
    the embedding within 3e-6 of max |Z| (float rounding amplified by the
    iterations; 6e-7 measured), every row's direction within 1e-9 of cosine
    1, the first 400 rows of R within 2e-5. Agreement at this level also
    pins the PCG32 Fisher-Yates cell order the restatement draws."""
    from harmony_cases import case, check_against
    from oracle import harmony as oh
    c = case(golden("harmony"), name)
    Z, R = oh.harmony(c["PCs"], oh.normalize_rows(c["PCs"]), c["Y_init"],
                      c["batch_labels"], c["num_batches"], **c["harmony_kwargs"])
    check_against(c, Z, R[:len(c["ref_R_head"])], z_rel=3e-6, r_abs=2e-5,
                  min_cos=1 - 1e-9)


def test_harmony_oracle_tau_matches_reference_nan(golden):
    """With tau > 0 the reference's theta discount negates an unsigned count
    (brisc/harmonize.pyx:416) and its output is NaN throughout; the
    restatement does the same arithmetic."""
    from harmony_cases import case
    from oracle import harmony as oh
    c = case(golden("harmony"), "harm_tau")
    assert np.isnan(c["ref_Z"]).all() and np.isnan(c["ref_R_head"]).all()
    with np.errstate(all="ignore"):
        Z, R = oh.harmony(c["PCs"], oh.normalize_rows(c["PCs"]), c["Y_init"],
                          c["batch_labels"], c["num_batches"], **c["harmony_kwargs"])
    assert np.isnan(Z).all() and np.isnan(R).all()


def test_fisher_yates_is_a_permutation():
    """The inside-out Fisher-Yates draw behind Harmony's cell order is a
    permutation, and a different seed gives a different one."""
    from oracle import clib
    a, b = clib.fisher_yates(1000, 0), clib.fisher_yates(1000, 1)
    assert np.array_equal(np.sort(a), np.arange(1000))
    assert not np.array_equal(a, b)
