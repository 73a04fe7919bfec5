"""End-to-end IRLBA on the GPU vs the reference's own outputs and FP64.

Tolerances (the accuracy gates of this path): relative singular-value error
<= 1e-4, max principal angle <= 1e-3 rad on subspaces with a spectral gap,
sign-aligned per-PC cosine >= 1 - 1e-4 against the reference's PCs on the
gapped fixtures, and run-to-run bit identity.
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

import brisc_gb300 as bg
from brisc_gb300 import DeviceMatrix, _lib
from synth import nb_counts
from oracle import dense
from oracle import irlba as oirlba

pytestmark = pytest.mark.gpu


def _case(z, name):
    n, g, k, m = (int(v) for v in z[f"{name}_shape"])
    X = sp.csr_matrix((z[f"{name}_data"], z[f"{name}_indices"],
                       z[f"{name}_indptr"]), shape=(n, g))
    return X, n, g, k, m


def _cos(a, b):
    a = dense.align_signs(a, b)
    return np.sum(a * b, 0) / np.linalg.norm(a, axis=0) / np.linalg.norm(b, axis=0)


@pytest.mark.parametrize("name", ["clustered_a", "clustered_b"])
def test_dropin_irlba_matches_reference(cuda, golden, name):
    z = golden("irlba")
    X, n, g, k, m = _case(z, name)
    ref = z[f"{name}_pcs"]
    PCs = np.empty((n, k), dtype=np.float32)
    csc = X.tocsc()
    conv = bg.irlba(data_matvec=X.data, indices_matvec=X.indices,
                    indptr_matvec=X.indptr, data_rmatvec=csc.data,
                    indices_rmatvec=csc.indices, indptr_rmatvec=csc.indptr,
                    num_cells=n, num_genes=g, k=k, subspace_size=m,
                    tolerance=1e-6, max_iterations=100, seed=0,
                    match_parallel=False, is_csr=True, num_threads=8,
                    chunk_size=1024, PCs=PCs)
    assert conv == bool(z[f"{name}_converged"])
    s_ref, s = dense.sv_from_pcs(ref), dense.sv_from_pcs(PCs)
    assert np.max(np.abs(s - s_ref) / s_ref) < 1e-4
    assert dense.max_angle(PCs, ref) < 1e-3
    assert _cos(PCs, ref).min() > 1 - 1e-4
    S, U, Vt = dense.top_svd(X, k + 2)
    assert dense.rel_sv_error(PCs, S).max() < 1e-4
    j = max(dense.gap_mask(S, k, 0.01))
    assert dense.max_angle(PCs[:, :j], U[:, :j]) < 1e-3


def test_dropin_csc_input_matches_csr_input(cuda, golden):
    """is_csr=False (the matvec arrays hold a CSC copy, as the reference's
    single-thread CSC path passes them) gives the CSR call's PCs bit for bit:
    the GPU transpose restores the same sorted CSR layout."""
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_b")
    X.sort_indices()
    csc = X.tocsc()
    csc.sort_indices()
    out = []
    for is_csr in (True, False):
        PCs = np.empty((n, k), dtype=np.float32)
        mv, rmv = (X, csc) if is_csr else (csc, X)
        bg.irlba(data_matvec=mv.data, indices_matvec=mv.indices, indptr_matvec=mv.indptr,
                 data_rmatvec=rmv.data, indices_rmatvec=rmv.indices,
                 indptr_rmatvec=rmv.indptr, num_cells=n, num_genes=g, k=k,
                 subspace_size=m, tolerance=1e-6, max_iterations=100, seed=0,
                 match_parallel=False, is_csr=is_csr, num_threads=1,
                 chunk_size=1024, PCs=PCs)
        out.append(PCs)
    assert np.array_equal(out[0], out[1])


def test_bit_identical_runs(cuda, golden):
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_a")
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    a = M.solve(k, m)
    b = M.solve(k, m)
    M.close()
    M2 = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    c = M2.solve(k, m)
    M2.close()
    assert np.array_equal(a.PCs, b.PCs) and np.array_equal(a.PCs, c.PCs)
    assert np.array_equal(a.singular_values, c.singular_values)


@pytest.mark.parametrize("passes,rotation",
                         [("auto", 0), (1, 0), (2, 0), (2, 1), (2, 2)])
def test_reorth_passes_both_meet_gates(cuda, golden, passes, rotation):
    """Every Gram-Schmidt mode (adaptive, one pass, CGS2) and both restart
    rotations (SIMT FP32 and the tensor-core 3 x BF16 split) meet the FP64
    gates."""
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_b")
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    r = M.solve(k, m, reorth_passes=passes, rotation_mode=rotation, loadings=True)
    M.close()
    S, U, Vt = dense.top_svd(X, k + 2)
    assert r.converged
    assert dense.rel_sv_error(r.PCs, S).max() < 1e-4
    np.testing.assert_allclose(r.singular_values, dense.sv_from_pcs(r.PCs), rtol=1e-4)
    # loadings are the right singular vectors: A^T u = s v
    assert dense.max_angle(r.loadings, Vt.T[:, :k]) < 1e-3
    assert dense.residuals(X, r.PCs).max() < 1e-3


@pytest.mark.parametrize("name", ["clustered_a", "clustered_b", "flat"])
def test_restart_svd_modes_agree(cuda, golden, name):
    """The restart SVD by secular-equation merge (default), the FP64 Jacobi of
    the whole B and the FP32 Jacobi + FP64 Newton of the whole B all give
    the FP64 singular values within 1e-4, PCs within the angle gate of each
    other on the gapped fixtures, and restart counts within one of each
    other (all three are FP64-accurate, so they converge alike)."""
    z = golden("irlba")
    X, n, g, k, m = _case(z, name)
    S, U, Vt = dense.top_svd(X, k + 2)
    out = {}
    for mode in (0, 1, 2):
        M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
        r = M.solve(k, m, svd_mode=mode)
        M.close()
        assert r.converged, mode
        assert dense.rel_sv_error(r.PCs, S).max() < 1e-4, mode
        out[mode] = r
    for mode in (1, 2):
        assert abs(out[mode].info["restarts"] - out[0].info["restarts"]) <= 1
        np.testing.assert_allclose(out[mode].singular_values, out[0].singular_values,
                                   rtol=1e-5)
        if name != "flat":
            assert dense.max_angle(out[mode].PCs, out[0].PCs) < 1e-3


def test_flat_spectrum_singular_values(cuda, golden):
    z = golden("irlba")
    X, n, g, k, m = _case(z, "flat")
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    r = M.solve(k, m)
    M.close()
    S, U, Vt = dense.top_svd(X, k + 2)
    assert dense.rel_sv_error(r.PCs, S).max() < 1e-4
    assert dense.rel_sv_error(z["flat_pcs"], S).max() < 1e-4


@pytest.mark.parametrize("method", ["logCP10k", "log1pPF", "PFlog1pPF"])
def test_fused_counts_path_matches_materialised(cuda, golden, method):
    """PCA on raw counts with the normalisation fused into every product
    equals PCA on the normalised float32 matrix (the reference's route).

    Both solves are FP32 and stop at the same residual tolerance; their sums
    round differently, so interior singular values may differ at the level of
    that tolerance (observed up to ~1.1e-5 relative). Each is held to the FP64
    bar (1e-4), and the two to 5e-5 of each other."""
    from oracle import clib
    z = golden("irlba")
    ip, ix, cnt = z["clustered_a_indptr"], z["clustered_a_indices"], z["clustered_a_counts"]
    n, g, k, m = (int(v) for v in z["clustered_a_shape"])
    counts = sp.csr_matrix((cnt, ix, ip), shape=(n, g))
    mnum = {"logCP10k": 0, "log1pPF": 1, "PFlog1pPF": 2}[method]
    xn, rs, isf, post = clib.normalize_csr(ip, cnt, mnum)
    Xn = sp.csr_matrix((xn, ix, ip), shape=(n, g))
    pcs_f, rf = bg.pca(Xn, num_PCs=k, subspace_size=m, return_result=True)
    pcs_c, rc = bg.pca_counts(counts, method=method, num_PCs=k, subspace_size=m,
                              return_result=True)
    s_f, s_c = dense.sv_from_pcs(pcs_f), dense.sv_from_pcs(pcs_c)
    S = dense.top_svd(Xn, k + 2)[0]
    assert dense.rel_sv_error(pcs_f, S).max() < 1e-4
    assert dense.rel_sv_error(pcs_c, S).max() < 1e-4
    assert np.max(np.abs(s_c - s_f) / s_f) < 5e-5
    assert dense.max_angle(pcs_c, pcs_f) < 1e-3


def test_pca_qc_backfill_and_joint(cuda, golden):
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_a")
    qc = (np.arange(n) % 9) != 4
    pcs = bg.pca(X, QC_column=qc, num_PCs=k, subspace_size=m)
    assert pcs.shape == (n, k) and np.isnan(pcs[~qc]).all()
    sub = bg.pca(X[np.flatnonzero(qc)], num_PCs=k, subspace_size=m)
    assert np.array_equal(pcs[qc], sub)
    a, b = bg.pca(X[: n // 2], X[n // 2:], num_PCs=k, subspace_size=m)
    joint = bg.pca(X, num_PCs=k, subspace_size=m)
    assert np.array_equal(np.vstack([a, b]), joint)


def test_pca_loadings_in_varm_layout(cuda, golden):
    """pca(..., loadings=True): loadings over every gene (NaN outside the HVG
    mask); on the HVGs they are the right singular vectors (A^T u = s v)."""
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_a")
    hvg = (np.arange(g) % 7) != 3
    (pcs, ld), res = bg.pca(X, hvg_column=hvg, num_PCs=k, subspace_size=m,
                            loadings=True, return_result=True)
    assert ld.shape == (g, k) and ld.dtype == np.float32
    assert np.isnan(ld[~hvg]).all() and np.isfinite(ld[hvg]).all()
    Xh = sp.csr_matrix(X[:, np.flatnonzero(hvg)])
    S, U, Vt = dense.top_svd(Xh, k + 2)
    j = max(dense.gap_mask(S, k, 0.01))
    assert dense.max_angle(ld[hvg][:, :j], Vt.T[:, :j]) < 1e-3
    np.testing.assert_allclose(np.linalg.norm(ld[hvg], axis=0), 1.0, rtol=1e-4)


def test_nonconverged_returns_ritz_vectors(cuda, golden):
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_a")
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    r = M.solve(k, m, max_iterations=1)
    M.close()
    o = oirlba.irlba(X, k, m, max_iterations=1, reorth_passes=2)
    assert not r.converged and not o["converged"]
    s, so = dense.sv_from_pcs(r.PCs), dense.sv_from_pcs(o["PCs"])
    assert np.max(np.abs(s - so) / so) < 1e-4
    np.testing.assert_allclose(s, r.singular_values, rtol=1e-5)


def test_small_problem_full_subspace(cuda):
    c = nb_counts(60, 12, seed=8, density=0.3, workers=1)
    X = sp.csr_matrix((c.normalized_f32(), c.indices, c.indptr), shape=(c.num_cells, 12))
    pcs = bg.pca(X, num_PCs=5, subspace_size=100)  # clipped to min(n, g) = 12
    S, U, Vt = dense.top_svd(X, 5)
    assert dense.rel_sv_error(pcs, S).max() < 1e-4


def test_cancel_flag(cuda, golden):
    z = golden("irlba")
    X, n, g, k, m = _case(z, "clustered_a")
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    flag = C.c_int32(1)
    o = _lib.SolveOpts()
    _lib.lib().bgpu_solve_opts_default(C.byref(o))
    o.k, o.subspace_size = k, m
    o.cancel = C.cast(C.pointer(flag), C.c_void_p)
    pcs = np.empty((n, k), dtype=np.float32)
    rc = _lib.lib().bgpu_irlba(M.handle, C.byref(o), pcs.ctypes.data, 0, None,
                               None, None, None)
    assert rc == _lib.ERR_CANCELLED
    r = M.solve(k, m)  # the context stays usable
    assert r.converged
    M.close()


def test_large_solve_meets_fp64_gate(cuda):
    """200k cells x 2000 genes at 5% density (the 1M workload's generator),
    default settings (secular-merge restart SVD, adaptive Gram-Schmidt,
    tensor-core rotation): relative singular-value error <= 1e-4 against the
    FP64 Gram-matrix oracle, and the solve converges."""
    from synth import nb_counts
    c = nb_counts(200_000, 2000, seed=0, density=0.05)
    M = DeviceMatrix(c.indptr.astype(np.int32), c.indices, c.data, c.num_cells, 2000,
                     norm="logCP10k", inv_size_factors=c.isf)
    r = M.solve(50, 100)
    M.close()
    X = c.to_scipy(np.float64)
    rows = np.repeat(np.arange(X.shape[0]), np.diff(X.indptr))
    X.data = np.log1p(X.data * c.isf[rows].astype(np.float64))
    S64 = dense.top_svd(X, 52)[0]
    assert r.converged
    assert dense.rel_sv_error(r.PCs, S64).max() < 1e-4


def _near_low_rank(seed=0, n=4000, g=400, rank=8):
    rng = np.random.default_rng(seed)
    W = rng.random((n, rank)) * (rng.random((n, rank)) < 0.3)
    H = rng.random((rank, g)) * (rng.random((rank, g)) < 0.5)
    A = W @ H
    A = A + 1e-3 * rng.random((n, g)) * (A > 0)
    return sp.csr_matrix(A.astype(np.float32))


def test_adaptive_second_pass_where_first_cancels(cuda):
    """On a near-low-rank matrix the first Gram-Schmidt pass cancels most of
    X.v at some steps; the adaptive mode runs the second pass at exactly the
    steps where the oracle's FP32 norms say so and meets the FP64 gates.
    A fixed-CGS2 solve reports a second pass at every step past the first."""
    X = _near_low_rank()
    n, g = X.shape
    k, m = 6, 16
    o = oirlba.irlba(X, k, m, reorth_passes=0)
    assert 0 < o["second_passes"] < o["steps"] - 1
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    r = M.solve(k, m)
    r2 = M.solve(k, m, reorth_passes=2)
    M.close()
    assert r.info["lanczos_steps"] == o["steps"]
    assert r.info["second_passes"] == o["second_passes"]
    assert r2.info["second_passes"] == r2.info["lanczos_steps"] - 1
    S, U, Vt = dense.top_svd(X, k + 2)
    assert r.converged
    assert dense.rel_sv_error(r.PCs, S).max() < 1e-4
    # the adaptive solve reads U fewer times than CGS2
    assert r.info["reorth_bytes"] < r2.info["reorth_bytes"]


@pytest.mark.parametrize("name", ["clustered_a", "clustered_b", "flat"])
def test_adaptive_equals_single_pass_when_no_cancellation(cuda, golden, name):
    """Where no step cancels (the oracle takes no second pass on either
    side), the adaptive mode is the reference's single pass bit for bit: the
    first pass is the same kernel sequence and the gated kernels write
    nothing."""
    z = golden("irlba")
    X, n, g, k, m = _case(z, name)
    o = oirlba.irlba(X, k, m, reorth_passes=0)
    assert o["second_passes"] == 0 and o["second_passes_v"] == 0
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    a = M.solve(k, m)
    b = M.solve(k, m, reorth_passes=1)
    M.close()
    assert a.info["second_passes"] == 0
    assert np.array_equal(a.PCs, b.PCs)
    assert np.array_equal(a.singular_values, b.singular_values)
