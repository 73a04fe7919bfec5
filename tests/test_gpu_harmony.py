"""Harmony on the GPU (brisc_gb300/harmony.py over csrc/harmony.cu) against
the reference's own outputs (tests/golden/harmony.npz, from
brisc/harmonize.pyx:269 after brisc/kmeans.pyx:889) and the NumPy oracle
(oracle/harmony.py).

Tolerance: FP32 sums in another order than the reference's sgemm and
per-thread loops, amplified by Harmony's iterations: every entry of Z within
1e-5 of max |Z|, every row's cosine with the reference's >= 1 - 1e-8, R
within 1e-4; run-to-run bit identity."""
import numpy as np
import pytest

from harmony_cases import case, check_against

pytestmark = pytest.mark.gpu

TOL = dict(z_rel=1e-5, r_abs=1e-4, min_cos=1 - 1e-8)


def _harmony(c, Y=None, Z=None, **over):
    from brisc_gb300 import harmony as H
    from oracle import harmony as oh
    n, d = c["PCs"].shape
    Y = np.array(c["Y_init"] if Y is None else Y, dtype=np.float32)
    Z = oh.normalize_rows(c["PCs"]) if Z is None else Z
    R = np.zeros((n, Y.shape[0]), np.float32)
    kw = dict(c["harmony_kwargs"], **over)
    it = H.harmony(PCs=c["PCs"], Z=Z, Y=Y, R=R, batch_labels=c["batch_labels"],
                   num_batches=c["num_batches"], **kw)
    return Z, Y, R, it


@pytest.mark.parametrize("name", ["harm_a", "harm_b"])
def test_harmony_matches_reference(cuda, golden, name):
    c = case(golden("harmony"), name)
    Z, Y, R, it = _harmony(c)
    assert 1 <= it <= c["harmony_kwargs"].get("max_iterations", 10)
    check_against(c, Z, R[:len(c["ref_R_head"])], **TOL)
    np.testing.assert_allclose(R.sum(1), 1.0, atol=1e-5)
    np.testing.assert_allclose(np.linalg.norm(Y, axis=1), 1.0, atol=1e-5)


def test_harmony_tau_gives_the_references_nan(cuda, golden):
    """tau > 0: the reference's theta is -inf (an unsigned count negated,
    brisc/harmonize.pyx:416) and its output NaN; the GPU path's too."""
    c = case(golden("harmony"), "harm_tau")
    Z, Y, R, it = _harmony(c)
    assert np.isnan(c["ref_Z"]).all()
    assert np.isnan(Z).all() and np.isnan(R).all()


def test_harmony_matches_oracle_at_20k(cuda):
    """A larger case the fixture does not hold: 20,000 cells, 30 PCs, 5
    batches, 100 clusters from the oracle's own starting centroids."""
    from synth import batched_pcs
    from oracle import harmony as oh
    X, b = batched_pcs(20000, 30, 16, 5, seed=21)
    rng = np.random.default_rng(0)
    Z0 = oh.normalize_rows(X)
    Y0 = np.ascontiguousarray(Z0[rng.choice(len(X), 100, replace=False)])
    Zo, Ro = oh.harmony(X, Z0.copy(), Y0, b, 5, seed=4)
    c = dict(PCs=X, batch_labels=b, num_batches=5, harmony_kwargs=dict(seed=4),
             Y_init=Y0, ref_Z=Zo, ref_R_head=Ro[:2000])
    Z, Y, R, it = _harmony(c)
    check_against(c, Z, R[:2000], **TOL)


def test_harmony_bit_identical_and_device_tensors(cuda, golden):
    """Two runs from host arrays and one on CUDA tensors (int32 holding the
    uint32 labels) give the same bits."""
    import torch
    from brisc_gb300 import harmony as H
    from oracle import harmony as oh
    c = case(golden("harmony"), "harm_b")
    a, b = _harmony(c), _harmony(c)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    T = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(cuda)  # noqa: E731
    n = len(c["PCs"])
    Z, Y = T(oh.normalize_rows(c["PCs"])), T(c["Y_init"])
    R = torch.zeros((n, Y.shape[0]), dtype=torch.float32, device=cuda)
    it = H.harmony(PCs=T(c["PCs"]), Z=Z, Y=Y, R=R,
                   batch_labels=T(c["batch_labels"].view(np.int32)),
                   num_batches=c["num_batches"], **c["harmony_kwargs"])
    torch.cuda.synchronize()
    assert it == a[3]
    np.testing.assert_array_equal(Z.cpu().numpy(), a[0])
    np.testing.assert_array_equal(Y.cpu().numpy(), a[1])
    np.testing.assert_array_equal(R.cpu().numpy(), a[2])


def test_normalize_rows_matches_oracle(cuda):
    from brisc_gb300 import harmony as H
    from oracle import harmony as oh
    X = np.random.default_rng(3).standard_normal((5001, 37)).astype(np.float32) * 7
    out = np.empty_like(X)
    H.normalize_rows(X, out)
    np.testing.assert_allclose(out, oh.normalize_rows(X), rtol=0, atol=4e-7)


@pytest.mark.parametrize("name", ["harm_a", "harm_b"])
def test_harmonize_pipeline_matches_reference(cuda, golden, name):
    """normalize_rows, k-means and harmony, all on the GPU, against the
    reference's harmonize() core: the same k-means iteration count and
    centroids to FP32 rounding, then the embedding as above."""
    from brisc_gb300 import harmony as H
    c = case(golden("harmony"), name)
    kw = c["kwargs"]
    Z = H.harmonize(c["PCs"], c["batch_labels"], c["num_batches"], **kw)
    check_against(c, Z, c["ref_R_head"], z_rel=1e-4, r_abs=np.inf, min_cos=1 - 1e-6)


def test_harmony_rejects_a_label_out_of_range(cuda, golden):
    """A batch label >= num_batches is an error, not an out-of-bounds write."""
    from brisc_gb300 import harmony as H
    c = case(golden("harmony"), "harm_b")
    n = len(c["PCs"])
    with pytest.raises(ValueError, match="batch label"):
        H.harmony(PCs=c["PCs"], Z=c["PCs"].copy(), Y=c["Y_init"].copy(),
                  R=np.zeros((n, len(c["Y_init"])), np.float32),
                  batch_labels=c["batch_labels"], num_batches=2)


@pytest.mark.parametrize("n,d,C,B,chunk", [(6000, 100, 200, 10, 256),  # 8 clusters a lane,
                                           #  128-dim correction tiles, large tiles
                                           (3000, 12, 20, 2, 64),      # one cluster a lane
                                           (4000, 64, 64, 33, 300)])   # many batches
def test_harmony_shapes_match_oracle(cuda, n, d, C, B, chunk):
    """The kernel shapes the fixtures do not reach, against the oracle from
    the same starting centroids: cluster counts above 128 and below 32, PCs
    above 64, 33 batches (the block kernel's larger shared-memory tiles), a
    chunk size that is not a power of two."""
    from synth import batched_pcs
    from oracle import harmony as oh
    X, b = batched_pcs(n, d, 12, B, seed=n + C)
    rng = np.random.default_rng(1)
    Z0 = oh.normalize_rows(X)
    Y0 = np.ascontiguousarray(Z0[rng.choice(n, C, replace=False)])
    kw = dict(seed=2, chunk_size=chunk, max_iterations=4)
    Zo, Ro = oh.harmony(X, Z0.copy(), Y0, b, B, **kw)
    c = dict(PCs=X, batch_labels=b, num_batches=B, harmony_kwargs=kw, Y_init=Y0,
             ref_Z=Zo, ref_R_head=Ro[:500])
    Z, Y, R, it = _harmony(c)
    check_against(c, Z, R[:500], **TOL)
