"""GPU building blocks vs the oracle, through the C ABI.

Integer work (transpose, row sums) bit-exact; float work within the stated
tolerances: log1pf on the device vs glibc <= 2 ulp; sparse products vs an
FP64 product <= 2e-5 relative (float32 accumulation of ~100-term rows).
"""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from brisc_gb300 import DeviceMatrix, _lib
from synth import nb_counts
from oracle import clib, dense

pytestmark = pytest.mark.gpu


def T(a, dev):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _u16(a):
    return a.view(np.int16)  # torch has no general uint16; the bits are what matter


@pytest.mark.parametrize("itype", [np.int32, np.int64])
def test_csr_tocsc_bit_exact(cuda, golden, itype):
    import torch
    z = golden("tocsc")
    ip, ix = z["indptr"].astype(itype), z["indices"].astype(itype)
    x = z["data"]
    n, g = ip.shape[0] - 1, int(z["n_col"])
    Bp = torch.empty(g + 1, dtype=getattr(torch, np.dtype(itype).name), device=cuda)
    Bi = torch.empty(x.shape[0], dtype=Bp.dtype, device=cuda)
    Bx = torch.empty(x.shape[0], dtype=torch.float32, device=cuda)
    dip, dix, dx = T(ip, cuda), T(ix, cuda), T(x, cuda)
    _lib.call("bgpu_csr_tocsc", n, g, dip.data_ptr(), dix.data_ptr(), dx.data_ptr(),
              _lib.INDEX_I64 if itype == np.int64 else _lib.INDEX_I32,
              Bp.data_ptr(), Bi.data_ptr(), Bx.data_ptr(), None)
    torch.cuda.synchronize()
    assert np.array_equal(Bp.cpu().numpy(), z["Bp"])
    assert np.array_equal(Bi.cpu().numpy(), z["Bi"])
    assert np.array_equal(Bx.cpu().numpy().view(np.uint32), z["Bx"].view(np.uint32))


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("tag", ["all", "qc"])
def test_size_factors_and_normalize(cuda, golden, method, tag):
    import torch
    z = golden("normalize")
    ip, counts = z["indptr"], z["counts"]
    n = ip.shape[0] - 1
    qc = z["qc"] if tag == "qc" else None
    ref_norm = z[f"m{method}_{tag}"]
    _, ors, oisf, opost = clib.normalize_csr(ip, counts, method, qc)
    dip, dv = T(ip, cuda), T(_u16(counts), cuda)
    isf = torch.empty(n, dtype=torch.float32, device=cuda)
    post = torch.empty(n, dtype=torch.float32, device=cuda)
    rs = torch.empty(n, dtype=torch.int64, device=cuda)
    dq = T(qc.astype(np.uint8), cuda) if qc is not None else None
    _lib.call("bgpu_size_factors", dip.data_ptr(), _lib.INDEX_I32, dv.data_ptr(),
              _lib.VALUE_U16, n, method, dq.data_ptr() if dq is not None else None,
              isf.data_ptr(), post.data_ptr() if method == 2 else None,
              rs.data_ptr(), None)
    out = torch.empty(counts.shape[0], dtype=torch.float32, device=cuda)
    _lib.call("bgpu_normalize_csr", dip.data_ptr(), _lib.INDEX_I32, dv.data_ptr(),
              _lib.VALUE_U16, n, isf.data_ptr(),
              post.data_ptr() if method == 2 else None, out.data_ptr(), None)
    torch.cuda.synchronize()
    assert np.array_equal(rs.cpu().numpy().view(np.uint64), z[f"rowsums_{tag}"])
    assert np.array_equal(isf.cpu().numpy(), oisf)  # float division, exact
    if method == 2:
        np.testing.assert_allclose(post.cpu().numpy(), opost, rtol=2e-6)
        np.testing.assert_allclose(out.cpu().numpy(), ref_norm, rtol=4e-6, atol=1e-7)
    else:
        d = np.abs(out.cpu().numpy().view(np.int32).astype(np.int64) -
                   ref_norm.view(np.int32).astype(np.int64))
        assert d.max() <= 2  # device log1pf vs glibc log1pf


def _mat(n=6000, g=700, density=0.05, seed=4, empty_rows=True):
    c = nb_counts(n, g, seed=seed, density=density, workers=1)
    X = c.to_scipy()
    X.data[::331] = np.minimum(X.data[::331].astype(np.int64) * 97 + 16,
                               65535).astype(X.data.dtype)  # counts beyond the tables
    if empty_rows:  # a few cells with no counts, and the last cell empty
        X = X.tolil()
        for r in (3, 17, X.shape[0] - 1):
            X[r, :] = 0
        X = sp.csr_matrix(X)
        X.eliminate_zeros()
    X.sort_indices()
    rs = np.asarray(X.sum(axis=1)).ravel()
    isf = np.where(rs > 0, np.float32(1e4) / np.maximum(rs, 1).astype(np.float32),
                   np.float32(1)).astype(np.float32)
    return X, isf


def _normalized(X, isf, post=None):
    rows = np.repeat(np.arange(X.shape[0]), np.diff(X.indptr))
    v = np.log1p(X.data.astype(np.float64) * isf[rows].astype(np.float64))
    if post is not None:
        v *= post[rows].astype(np.float64)
    return sp.csr_matrix((v, X.indices, X.indptr), shape=X.shape)


@pytest.mark.parametrize("mode", ["counts", "counts_post", "float"])
@pytest.mark.parametrize("itype", [np.int32, np.int64])
@pytest.mark.parametrize("panel_rows", [0, 2048])
@pytest.mark.parametrize("impl", ["auto", "rows", "seg", "vector", "words32"])
def test_matvec_rmatvec_stddev(cuda, mode, itype, panel_rows, impl):
    """Both sparse products and the gene std on every layout: automatic
    (sliced-ELL for counts), and the panel layout with each X.v kernel and
    with X^T.u over the 32-bit words."""
    import torch
    kernels = {"auto": (), "rows": ("panels", "xv_rows"), "seg": ("panels", "xv_seg"),
               "vector": ("panels", "vector"), "words32": ("panels", "words32")}[impl]
    X, isf = _mat()
    n, g = X.shape
    post = None
    if mode == "counts_post":  # per-cell post-log factors (PFlog1pPF layout)
        post = np.random.default_rng(1).uniform(0.5, 2.0, n).astype(np.float32)
    Xn = _normalized(X, isf, post)
    ip, ix = X.indptr.astype(itype), X.indices.astype(itype)
    if mode == "counts":
        M = DeviceMatrix(ip, ix, X.data.astype(np.uint16), n, g, norm="logCP10k",
                         inv_size_factors=isf, panel_rows=panel_rows, kernels=kernels)
    elif mode == "counts_post":
        M = DeviceMatrix(ip, ix, X.data.astype(np.uint16), n, g, norm="PFlog1pPF",
                         inv_size_factors=isf, post_factors=post,
                         panel_rows=panel_rows, kernels=kernels)
    else:
        M = DeviceMatrix(ip, ix, Xn.data.astype(np.float32), n, g,
                         panel_rows=panel_rows, kernels=kernels)
    rng = np.random.default_rng(0)
    v = rng.standard_normal(g).astype(np.float32)
    u = rng.standard_normal(n).astype(np.float32)
    u -= u.mean()
    sd = torch.empty(g, dtype=torch.float32, device=cuda)
    M.gene_stddev(sd)
    torch.cuda.synchronize()
    sd_h = sd.cpu().numpy()
    _, sd64 = dense.gene_std64(Xn)
    np.testing.assert_allclose(sd_h, sd64, rtol=2e-6)
    y = torch.empty(n, dtype=torch.float32, device=cuda)
    z = torch.empty(g, dtype=torch.float32, device=cuda)
    dv, du = T(v, cuda), T(u, cuda)
    M.matvec(dv, sd, y)
    M.rmatvec(du, sd, z)
    torch.cuda.synchronize()
    y_ref = Xn @ (v.astype(np.float64) / sd_h)
    z_ref = (Xn.T @ u.astype(np.float64)) / sd_h
    scale_y = np.abs(Xn) @ np.abs(v.astype(np.float64) / sd_h)
    scale_z = (np.abs(Xn).T @ np.abs(u.astype(np.float64))) / sd_h
    assert np.max(np.abs(y.cpu().numpy() - y_ref) / (scale_y + 1e-30)) < 2e-5
    assert np.max(np.abs(z.cpu().numpy() - z_ref) / (scale_z + 1e-30)) < 2e-5
    assert y.cpu().numpy()[-1] == 0.0  # empty last cell
    # run-to-run bit identity
    y2 = torch.empty_like(y)
    z2 = torch.empty_like(z)
    M.matvec(dv, sd, y2)
    M.rmatvec(du, sd, z2)
    torch.cuda.synchronize()
    assert torch.equal(y, y2) and torch.equal(z, z2)
    M.close()


def test_stddev_matches_reference_formula(cuda, golden):
    """FP64 accumulation vs the reference's float32 single-pass formula."""
    import torch
    z = golden("irlba")
    n, g, k, m = (int(x) for x in z["clustered_a_shape"])
    X = sp.csr_matrix((z["clustered_a_data"], z["clustered_a_indices"],
                       z["clustered_a_indptr"]), shape=(n, g))
    M = DeviceMatrix(X.indptr, X.indices, X.data, n, g)
    sd = torch.empty(g, dtype=torch.float32, device=cuda)
    M.gene_stddev(sd)
    torch.cuda.synchronize()
    csc = X.tocsc()
    csc.sort_indices()
    ref32 = clib.clipped_stddev_csc(csc.data, csc.indptr, n)
    np.testing.assert_allclose(sd.cpu().numpy(), ref32, rtol=1e-4)


@pytest.mark.parametrize("m", [2, 7, 20, 100, 130, 200])
def test_small_svd(cuda, m):
    import torch
    rng = np.random.default_rng(m)
    # an IRLBA-like B: diagonal + residual column block, then bidiagonal
    B = np.zeros((m, m + 1), dtype=np.float64)
    kc = m // 2
    B[np.arange(kc), np.arange(kc)] = np.sort(rng.uniform(1, 100, kc))[::-1]
    B[:kc, kc] = rng.normal(0, 1, kc)
    for i in range(kc, m):
        B[i, i] = rng.uniform(1, 50)
        B[i, i + 1] = rng.uniform(0.1, 20)
    Bf = np.asfortranarray(B.astype(np.float32))
    dB = torch.from_numpy(Bf.ravel(order="F").copy()).to(cuda)
    Ub = torch.empty(m * m, dtype=torch.float32, device=cuda)
    Sb = torch.empty(m, dtype=torch.float32, device=cuda)
    Vbt = torch.empty(m * (m + 1), dtype=torch.float32, device=cuda)
    _lib.call("bgpu_small_svd", dB.data_ptr(), m, Ub.data_ptr(), Sb.data_ptr(),
              Vbt.data_ptr(), None)
    torch.cuda.synchronize()
    U = Ub.cpu().numpy().reshape(m, m, order="F").astype(np.float64)
    S = Sb.cpu().numpy().astype(np.float64)
    Vt = Vbt.cpu().numpy().reshape(m, m + 1, order="F").astype(np.float64)
    S64 = np.linalg.svd(Bf.astype(np.float64), compute_uv=False)
    assert np.all(np.diff(S) <= 0)
    np.testing.assert_allclose(S, S64, rtol=1e-5, atol=1e-5 * S64[0])
    assert np.abs(U.T @ U - np.eye(m)).max() < 1e-5
    assert np.abs(U @ np.diag(S) @ Vt - Bf).max() < 1e-5 * S64[0]


@pytest.mark.parametrize("rows,K,ncols", [(5000, 100, 99), (5000, 100, 100),
                                          (1000, 100, 37), (300, 7, 3), (128, 64, 1),
                                          # K / column chunks (the m = 200 solve)
                                          (5000, 200, 199), (3000, 150, 129),
                                          (777, 256, 256), (1000, 113, 5)])
def test_rotate_basis_tensor_cores(cuda, rows, K, ncols):
    """U . Ub[:, :kc] on the tensor cores (3 x BF16 split, six cross products,
    FP32 accumulation) against the SIMT FP32 GEMM and an FP64 product, for a
    general orthogonal Ub (no dominated columns): both within 2e-6 of the
    FP64 scale (the chunked shapes add their K parts in FP32, in chunk
    order)."""
    rng = np.random.default_rng(rows + K + ncols)
    lda = rows + 64 - rows % 64
    A = np.zeros((K, lda), dtype=np.float32)  # column-major rows x K, ld = lda
    A[:, :rows] = rng.standard_normal((K, rows)).astype(np.float32) / np.sqrt(rows)
    Q, _ = np.linalg.qr(rng.standard_normal((K, K)))
    out, ref, scale = _rotate_both(cuda, A, Q, rows, K, ncols)
    for mode in (1, 2):
        err = np.abs(out[mode] - ref) / scale
        assert np.isfinite(out[mode]).all()
        assert err.max() < 2e-6, (mode, err.max())


def _rotate_both(cuda, A, Q, rows, K, ncols):
    import torch
    lda = A.shape[1]
    Bm = np.asfortranarray(Q.astype(np.float32))
    dA, dB = T(A.ravel(), cuda), T(Bm.ravel(order="F"), cuda)
    out = {}
    for mode in (1, 2):
        dC = torch.full((ncols * lda,), np.nan, dtype=torch.float32, device=cuda)
        _lib.call("bgpu_rotate_basis", dA.data_ptr(), lda, rows, K, dB.data_ptr(), K,
                  ncols, dC.data_ptr(), lda, mode, None)
        out[mode] = dC.cpu().numpy().reshape(ncols, lda)[:, :rows].astype(np.float64)
    ref = (A[:, :rows].T.astype(np.float64) @ Bm[:, :ncols].astype(np.float64)).T
    scale = (np.abs(A[:, :rows]).T.astype(np.float64) @ np.abs(Bm[:, :ncols])).T
    return out, ref, scale


@pytest.mark.parametrize("rows,K,ncols", [(20000, 100, 99), (20000, 100, 60),
                                          (8000, 200, 150), (5000, 64, 64)])
def test_rotate_basis_ritz_rotation_unbiased(cuda, rows, K, ncols):
    """The restart's rotation of converged Ritz vectors: Ub is a signed,
    partly permuted near-identity (each column dominated by one entry), and
    one column is exactly a unit vector. The tensor core's FP32 accumulation
    truncates toward zero; the pivoted delta form adds the dominant column in
    FP32, so the rotated columns keep their norms: the signed relative error
    stays at the FP32 GEMM's level (|bias| < 3e-8, where a plain tensor-core
    product of these shapes measured 5e-7), the RMS error within 1.5x the FP32
    GEMM's, and the unit-vector column is copied exactly."""
    rng = np.random.default_rng(rows + K)
    lda = rows + 64 - rows % 64
    Q0, _ = np.linalg.qr(rng.standard_normal((rows, K)))
    A = np.zeros((K, lda), dtype=np.float32)
    A[:, :rows] = Q0.T.astype(np.float32)
    Q, _ = np.linalg.qr(np.eye(K) + 1e-3 * rng.standard_normal((K, K)))
    Q = Q * np.sign(np.diag(Q))[None, :]
    Q[:, 1::3] *= -1.0                    # sign flips
    perm = np.arange(K)
    perm[[2, 5]] = perm[[5, 2]]           # two Ritz values swapped places
    Q = Q[:, perm]
    Q[:, 0] = 0.0
    Q[3, 0] = -1.0                        # a deflated (exactly converged) vector
    Q[:, K - 1] = np.linalg.qr(rng.standard_normal((K, 1)))[0][:, 0]  # a mixed column
    out, ref, _ = _rotate_both(cuda, A, Q, rows, K, ncols)
    stats = {}
    for mode in (1, 2):
        err = out[mode] - ref
        bias = float(np.sum(err * np.sign(ref)) / np.sum(np.abs(ref)))
        rms = float(np.sqrt(np.mean(err ** 2) / np.mean(ref ** 2)))
        stats[mode] = (bias, rms)
    assert abs(stats[2][0]) < 3e-8, stats
    assert stats[2][1] <= 1.5 * stats[1][1] + 1e-8, stats
    np.testing.assert_array_equal(out[2][0], -A[3, :rows].astype(np.float64))


def test_row_order_does_not_change_products(cuda):
    """X.v with the length-ordered row schedule is bit-identical to the natural
    order: the schedule only changes which 8-lane group sums a row."""
    import torch
    X, isf = _mat(n=9000, g=600, density=0.08)
    n, g = X.shape
    out = []
    for kernels in (("panels", "xv_rows"), ("panels", "xv_rows", "natural")):
        M = DeviceMatrix(X.indptr.astype(np.int32), X.indices.astype(np.int32),
                         X.data.astype(np.uint16), n, g, norm="logCP10k",
                         inv_size_factors=isf, kernels=kernels)
        v = T(np.random.default_rng(3).standard_normal(g).astype(np.float32), cuda)
        sd = torch.ones(g, dtype=torch.float32, device=cuda)
        y = torch.empty(n, dtype=torch.float32, device=cuda)
        M.matvec(v, sd, y)
        torch.cuda.synchronize()
        out.append(y.cpu().numpy())
        M.close()
    assert np.array_equal(out[0], out[1])
