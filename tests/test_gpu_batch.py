"""Batched per-subset PCAs (row subsets of one resident count matrix).

Each subset's PCs must be bit-identical whether solved alone from host arrays,
sequentially from the shared device matrix, concurrently on streams, or in
the lock-step batch (one launch per step kernel over all subsets); and meet
the FP64 gate (relative singular-value error <= 1e-4).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from brisc_gb300 import DeviceMatrix
from brisc_gb300.batch import (SUBSET_PANEL_ROWS, SharedMatrix, pca_subsets,
                               subset_solve_params)
from synth import nb_counts
from oracle import dense

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def counts():
    c = nb_counts(12000, 400, seed=7, density=0.08, workers=1, clusters=5)
    return c


def _partition(n, sizes, seed=3):
    perm = np.random.default_rng(seed).permutation(n)
    out, at = [], 0
    for s in sizes:
        out.append(np.sort(perm[at:at + s]).astype(np.int64))
        at += s
    return out


def test_subsets_bit_identical_alone_sequential_batched(cuda, counts):
    c = counts
    n, g = c.num_cells, c.num_genes
    subsets = _partition(n, [5000, 3000, 1500, 900, 400, 150])
    S = SharedMatrix(c.indptr, c.indices, c.data, n, g, inv_size_factors=c.isf)
    seq = pca_subsets(S, subsets, num_PCs=12, concurrency=1, mode="streams")
    bat = pca_subsets(S, subsets, num_PCs=12, concurrency=4, mode="streams")
    info = {}
    fus = pca_subsets(S, subsets, num_PCs=12, concurrency=4, mode="fused", info=info)
    assert info["mode"] == "fused" and info["kernel_launches"] > 0
    X = c.to_scipy()
    for rows, a, b, f in zip(subsets, seq, bat, fus):
        assert a.rows == rows.shape[0]
        assert np.array_equal(a.result.PCs, b.result.PCs)
        assert np.array_equal(a.result.PCs, f.result.PCs)
        assert np.array_equal(a.result.singular_values, f.result.singular_values)
        for key in ("restarts", "lanczos_steps", "converged", "second_passes"):
            assert a.result.info[key] == f.result.info[key], key
        # alone, from host arrays sliced on the host
        sub = sp.csr_matrix(X[rows])
        sub.sort_indices()
        k, m = subset_solve_params(rows.shape[0], g, 12, None)
        M = DeviceMatrix(sub.indptr.astype(np.int32), sub.indices.astype(np.int32),
                         sub.data.astype(np.uint16), rows.shape[0], g,
                         norm="logCP10k", inv_size_factors=c.isf[rows],
                         sell_panel_rows=SUBSET_PANEL_ROWS)
        alone = M.solve(k, m)
        M.close()
        assert np.array_equal(alone.PCs, a.result.PCs)


def test_subset_meets_fp64_gate(cuda, counts):
    c = counts
    n, g = c.num_cells, c.num_genes
    rows = _partition(n, [4000])[0]
    S = SharedMatrix(c.indptr, c.indices, c.data, n, g, inv_size_factors=c.isf)
    r = pca_subsets(S, [rows], num_PCs=10)[0].result
    X = sp.csr_matrix(c.to_scipy()[rows])
    rr = np.repeat(np.arange(X.shape[0]), np.diff(X.indptr))
    Xn = sp.csr_matrix((np.log1p(X.data.astype(np.float64) * c.isf[rows][rr]),
                        X.indices, X.indptr), shape=X.shape)
    S64 = dense.top_svd(Xn, 12)[0]
    assert r.converged
    assert dense.rel_sv_error(r.PCs, S64).max() < 1e-4


def test_host_row_subset_matches_host_slice(cuda, counts):
    c = counts
    n, g = c.num_cells, c.num_genes
    rows = np.random.default_rng(5).permutation(n)[:600].astype(np.int64)  # any order
    X = c.to_scipy()
    sub = sp.csr_matrix(X[rows])
    M1 = DeviceMatrix(c.indptr.astype(np.int32), c.indices, c.data, n, g,
                      norm="logCP10k", inv_size_factors=c.isf, rows=rows)
    M2 = DeviceMatrix(sub.indptr.astype(np.int32), sub.indices.astype(np.int32),
                      sub.data.astype(np.uint16), rows.shape[0], g,
                      norm="logCP10k", inv_size_factors=c.isf[rows])
    a, b = M1.solve(8, 16), M2.solve(8, 16)
    M1.close()
    M2.close()
    assert np.array_equal(a.PCs, b.PCs)


def test_row_subset_rejects_bad_rows(cuda, counts):
    c = counts
    with pytest.raises(ValueError, match="outside"):
        DeviceMatrix(c.indptr.astype(np.int32), c.indices, c.data, c.num_cells,
                     c.num_genes, norm="logCP10k", inv_size_factors=c.isf,
                     rows=np.array([0, c.num_cells], dtype=np.int64))


def test_fused_batch_over_many_subsets_and_an_iteration_cap(cuda, counts):
    """70 subsets (two launches of at most 64 tasks per step kernel) of very
    different sizes, with a restart cap that stops some unconverged: every
    subset bit-identical to its sequential solve, restart counts included."""
    c = counts
    n, g = c.num_cells, c.num_genes
    sizes = [3000, 1200] + [40 + 2 * i for i in range(68)]  # 11,476 of 12,000 cells
    subsets = _partition(n, sizes, seed=11)
    S = SharedMatrix(c.indptr, c.indices, c.data, n, g, inv_size_factors=c.isf)
    kw = dict(num_PCs=6, max_iterations=4)
    seq = pca_subsets(S, subsets, concurrency=1, mode="streams", **kw)
    info = {}
    fus = pca_subsets(S, subsets, concurrency=8, mode="fused", info=info, **kw)
    assert info["mode"] == "fused"
    assert any(not a.result.converged for a in seq)
    for a, f in zip(seq, fus):
        assert np.array_equal(a.result.PCs, f.result.PCs)
        assert a.result.info["restarts"] == f.result.info["restarts"]
        assert a.result.converged == f.result.converged


def test_fused_batch_needs_adaptive_passes(cuda, counts):
    """The lock-step batch runs the adaptive U pass only: mode="fused" with
    two fixed passes is refused before anything runs; mode="auto" runs the
    independent solves instead, with the same PCs as sequential ones."""
    from brisc_gb300._lib import BriscGPUError
    c = counts
    n, g = c.num_cells, c.num_genes
    subsets = _partition(n, [2000, 800])
    S = SharedMatrix(c.indptr, c.indices, c.data, n, g, inv_size_factors=c.isf)
    with pytest.raises(BriscGPUError, match="reorth_passes"):
        pca_subsets(S, subsets, num_PCs=5, mode="fused", reorth_passes=2)
    info = {}
    auto = pca_subsets(S, subsets, num_PCs=5, mode="auto", reorth_passes=2, info=info)
    assert info["mode"] == "streams"
    seq = pca_subsets(S, subsets, num_PCs=5, concurrency=1, mode="streams", reorth_passes=2)
    for a, b in zip(auto, seq):
        assert np.array_equal(a.result.PCs, b.result.PCs)
