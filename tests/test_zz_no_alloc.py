"""bgpu_small_svd_noalloc against bgpu_small_svd, through the C ABI.

The no-alloc entry point serves callers that cannot let a library allocate
device memory (their pool allocator owns the GPU's memory, or cudaMalloc would
stall a latency-critical loop). It must give the same SVD as the allocating
entry point, call after call, although every call reuses one fixed scratch
array. This file is collected last, so a run that stops at the first failure
has run every other test before it.
"""
import numpy as np
import pytest

from brisc_gb300 import _lib

pytestmark = pytest.mark.gpu


def _irlba_like_b(m, seed):
    """m x (m+1) column-major float32: diagonal + residual column, then bidiagonal."""
    rng = np.random.default_rng(seed)
    B = np.zeros((m, m + 1), dtype=np.float64)
    kc = m // 2
    B[np.arange(kc), np.arange(kc)] = np.sort(rng.uniform(1, 100, kc))[::-1]
    B[:kc, kc] = rng.normal(0, 1, kc)
    for i in range(kc, m):
        B[i, i] = rng.uniform(1, 50)
        B[i, i + 1] = rng.uniform(0.1, 20)
    return B.astype(np.float32)


def _svd(fn, Bf, m, dev):
    import torch
    dB = torch.from_numpy(Bf.ravel(order="F").copy()).to(dev)
    Ub = torch.empty(m * m, dtype=torch.float32, device=dev)
    Sb = torch.empty(m, dtype=torch.float32, device=dev)
    Vbt = torch.empty(m * (m + 1), dtype=torch.float32, device=dev)
    _lib.call(fn, dB.data_ptr(), m, Ub.data_ptr(), Sb.data_ptr(), Vbt.data_ptr(),
              None)
    torch.cuda.synchronize()
    return (Ub.cpu().numpy().reshape(m, m, order="F"), Sb.cpu().numpy(),
            Vbt.cpu().numpy().reshape(m, m + 1, order="F"))


# 100: matrices in shared memory; 200: Jacobi workspace in the scratch array;
# 256: the largest m, whose workspace fills the fixed scratch array exactly
@pytest.mark.parametrize("m", [100, 200, 256])
def test_noalloc_small_svd_matches_allocating_entry(cuda, m):
    for call, seed in enumerate((11, 12)):  # two calls in a row, new input each
        Bf = _irlba_like_b(m, seed + m)
        U0, S0, V0 = _svd("bgpu_small_svd", Bf, m, cuda)
        U1, S1, V1 = _svd("bgpu_small_svd_noalloc", Bf, m, cuda)
        S64 = np.linalg.svd(Bf.astype(np.float64), compute_uv=False)
        # the small-SVD tolerance of the other tests: 1e-5 of sigma_max
        tol = 1e-5 * S64[0]
        np.testing.assert_allclose(S1, S0, rtol=1e-5, atol=tol)
        np.testing.assert_allclose(np.abs(U1), np.abs(U0), atol=1e-5)
        np.testing.assert_allclose(np.abs(V1), np.abs(V0), atol=1e-5)
        rec = U1.astype(np.float64) @ np.diag(S1) @ V1.astype(np.float64)
        assert np.abs(rec - Bf).max() < tol, f"call {call}"


def test_noalloc_small_svd_rejects_oversize(cuda):
    m = 257
    with pytest.raises(ValueError, match="scratch limit"):
        _lib.call("bgpu_small_svd_noalloc", 1, m, 1, 1, 1, None)
