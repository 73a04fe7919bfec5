"""Host-side logic of the pca() mirror and the workload generator (CPU only).

Argument errors are raised before anything touches the GPU, with the
reference's messages (brisc/single_cell.py:11750-11958).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from brisc_gb300 import pca
from synth import nb_counts


def _X(n=50, g=20, dtype=np.float32):
    rng = np.random.default_rng(0)
    d = (rng.random((n, g)) < 0.3) * rng.random((n, g))
    return sp.csr_matrix(d.astype(dtype))


@pytest.mark.parametrize("kw, err, msg", [
    (dict(num_PCs=0), ValueError, "num_PCs"),
    (dict(num_PCs=2.5), TypeError, "num_PCs"),
    (dict(num_PCs=10, subspace_size=5), ValueError, "subspace_size"),
    (dict(tolerance=0), ValueError, "tolerance"),
    (dict(max_iterations=0), ValueError, "max_iterations"),
    (dict(chunk_size=0), ValueError, "chunk_size"),
    (dict(seed=1.5), TypeError, "seed"),
    (dict(match_parallel=True, num_threads=4), ValueError, "match_parallel"),
    (dict(num_PCs=30, subspace_size=40), ValueError, "number of genes"),
])
def test_pca_argument_errors(kw, err, msg):
    base = dict(num_PCs=5, subspace_size=10)
    base.update(kw)
    with pytest.raises(err, match=msg):
        pca(_X(), **base)


def test_pca_requires_float32():
    with pytest.raises(TypeError, match="float32"):
        pca(_X(dtype=np.float64), num_PCs=5, subspace_size=10)


def test_pca_all_false_qc():
    with pytest.raises(ValueError, match="no cells pass QC"):
        pca(_X(), QC_column=np.zeros(50, dtype=bool), num_PCs=5, subspace_size=10)


def test_pca_one_cell():
    with pytest.raises(ValueError, match="num_PCs"):
        pca(_X(n=1), num_PCs=5, subspace_size=10)


def test_generator_deterministic_across_workers():
    a = nb_counts(40000, 64, seed=9, density=0.08, workers=1)
    b = nb_counts(40000, 64, seed=9, density=0.08, workers=3)
    assert np.array_equal(a.indptr, b.indptr)
    assert np.array_equal(a.indices, b.indices)
    assert np.array_equal(a.data, b.data)
    assert np.array_equal(a.isf, b.isf)


def test_generator_density_and_layout():
    c = nb_counts(20000, 2000, seed=1, density=0.05, workers=2)
    assert 0.035 < c.density < 0.065
    assert c.indptr.dtype == np.int64 and c.indices.dtype == np.int32
    assert c.data.dtype == np.uint16 and c.isf.dtype == np.float32
    assert np.all(np.diff(c.indptr) > 0)  # empty cells dropped
    rows = np.repeat(np.arange(c.num_cells), np.diff(c.indptr))
    rs = np.bincount(rows, weights=c.data.astype(np.float64))
    assert np.array_equal(c.isf, (np.float32(1e4) / rs.astype(np.float32)))


def test_generator_clusters():
    c = nb_counts(5000, 100, seed=2, density=0.08, clusters=13, workers=1)
    assert c.clusters is not None and c.clusters.shape[0] == c.num_cells
    assert set(np.unique(c.clusters)) <= set(range(13))


def test_reorth_modes():
    from brisc_gb300.pca import reorth_code
    assert (reorth_code("auto"), reorth_code(1), reorth_code(2)) == (0, 1, 2)
    for bad in (0, 3, "two", None, 1.5):
        with pytest.raises(ValueError, match="reorth_passes"):
            reorth_code(bad)


def test_hvg_argument_checks():
    """Type and shape checks of the HVG entry points run before any GPU call."""
    from brisc_gb300 import hvg
    ip = np.array([0, 1, 2], np.int32)
    ix = np.array([0, 1], np.int32)
    d = np.array([1, 2], np.uint32)
    m, v, c = np.zeros(2, np.float32), np.zeros(2, np.float32), np.zeros(2, np.uint32)
    with pytest.raises(TypeError, match="same dtype"):
        hvg.gene_mean_and_variance_csr(d, ix.astype(np.int64), ip, np.zeros(0, np.int64),
                                       2, 2, m, v, c, 1)
    with pytest.raises(TypeError, match="data has dtype int8"):
        hvg.gene_mean_and_variance_csr(d.astype(np.int8), ix, ip, np.zeros(0, np.int64),
                                       2, 2, m, v, c, 1)
    with pytest.raises(ValueError, match="entries"):
        hvg.gene_mean_and_variance_csr(d, ix, ip, np.zeros(0, np.int64), 2, 3, m, v, c, 1)
    with pytest.raises(TypeError, match="cell_indices"):
        hvg.clipped_sum_csr(d, ix, ip, 2, 2, np.array([0], np.int32),
                            np.ones(2, np.float32), m, v, 1)
    with pytest.raises(ValueError, match="C-contiguous"):
        hvg.clipped_sum_csc(d, ix, ip, np.zeros(0, np.int8),
                            np.ones(4, np.float32)[::2], m, v, 1)


def test_install_hvg_binds_and_returns_previous():
    import types
    from brisc_gb300 import hvg
    fake = types.SimpleNamespace(gene_mean_and_variance_csr="old")
    prev = hvg.install_hvg(fake)
    assert prev["gene_mean_and_variance_csr"] == "old"
    assert prev["clipped_sum_csc"] is None
    for name in hvg.NAMES:
        assert getattr(fake, name) is getattr(hvg, name)


def test_batch_modes_and_subset_params():
    """pca_subsets checks its mode before any device work, and each subset's
    (k, m) is clipped to its shape as pca() clips it."""
    from brisc_gb300.batch import SUBSET_PANEL_ROWS, pca_subsets, subset_solve_params
    with pytest.raises(ValueError, match="mode"):
        pca_subsets(None, [np.arange(10)], mode="persistent")
    assert subset_solve_params(5000, 2000, 30, None) == (30, 60)
    assert subset_solve_params(40, 2000, 30, None) == (30, 40)
    assert subset_solve_params(20, 2000, 30, None) == (20, 20)
    assert subset_solve_params(5000, 50, 30, 100) == (30, 50)
    # the subsets' X^T.u panels: what the sliced-ELL layout accepts
    assert SUBSET_PANEL_ROWS % 32 == 0 and 128 <= SUBSET_PANEL_ROWS <= 512
