"""Seeded synthetic negative-binomial count matrices (the benchmark workloads).

Per gene a mean ``mu_g ~ lognormal(mu, sigma)``; per cell a library factor
``l_c ~ lognormal(0, lib_sigma)``; count ``~ NB(mean l_c * mu_g, dispersion)``
drawn as Poisson(Gamma(1/disp, mean * disp)). ``mu`` is the one parameter
moved away from the literal -1 to reach a target density: -3.381 gives ~8 %,
-3.954 gives ~5 % (the literal value gives ~37 %). Optional cell clusters get
per-gene lognormal mean offsets.

Rows are generated in fixed 16,384-row chunks, each from its own
``numpy.random.default_rng((seed, chunk))`` stream, so the matrix is identical
whatever the number of worker processes. Counts are stored as uint16
(saturating; the maximum is reported), gene indices as int32, indptr as int64,
and the per-cell inverse size factors of logCP10k (1e4 / row sum) as float32.
Cells with no counts are dropped, as QC would.
"""
from __future__ import annotations

import hashlib
import os
import tempfile
from concurrent.futures import ProcessPoolExecutor
from dataclasses import dataclass
from multiprocessing import get_context
from pathlib import Path

import numpy as np

CHUNK = 16384
MU_FOR_DENSITY = {0.08: -3.381, 0.05: -3.954}


def mu_for_density(density: float) -> float:
    """Log-mean of the per-gene means giving about `density` stored entries:
    the two calibrated points, interpolated (and extended) linearly in
    log(density)."""
    if density in MU_FOR_DENSITY:
        return MU_FOR_DENSITY[density]
    (d0, m0), (d1, m1) = sorted(MU_FOR_DENSITY.items())
    t = (np.log(density) - np.log(d0)) / (np.log(d1) - np.log(d0))
    return float(m0 + t * (m1 - m0))


@dataclass
class CountMatrix:
    indptr: np.ndarray      # int64, n + 1
    indices: np.ndarray     # int32, nnz
    data: np.ndarray        # uint16, nnz
    num_genes: int
    isf: np.ndarray         # float32, n: 1e4 / row sum (logCP10k)
    max_count: int
    clusters: np.ndarray | None = None

    @property
    def num_cells(self) -> int:
        return self.indptr.shape[0] - 1

    @property
    def nnz(self) -> int:
        return int(self.indptr[-1])

    @property
    def density(self) -> float:
        return self.nnz / (self.num_cells * self.num_genes)

    def to_scipy(self, dtype=None):
        import scipy.sparse as sp
        d = self.data if dtype is None else self.data.astype(dtype)
        return sp.csr_matrix((d, self.indices, self.indptr),
                             shape=(self.num_cells, self.num_genes))

    def normalized_f32(self) -> np.ndarray:
        """log1p(count * isf) as float32 per stored entry (logCP10k values)."""
        rows = np.repeat(np.arange(self.num_cells), np.diff(self.indptr))
        return np.log1p(self.data.astype(np.float32) * self.isf[rows]).astype(np.float32)


def _gene_params(seed, g, mu, sigma, clusters, cluster_sigma):
    rng = np.random.default_rng((seed, 0x6E6E))
    gm = rng.lognormal(mu, sigma, g)
    offs = None
    if clusters:
        offs = rng.lognormal(0.0, cluster_sigma, (clusters, g))
    return gm, offs


def _chunk(args):
    (seed, ci, rows, g, mu, sigma, disp, lib_sigma, clusters, cluster_sigma) = args
    gm, offs = _gene_params(seed, g, mu, sigma, clusters, cluster_sigma)
    rng = np.random.default_rng((seed, ci))
    lib = rng.lognormal(0.0, lib_sigma, rows)
    cl = None
    if clusters:
        cl = rng.integers(0, clusters, rows)
        mean = lib[:, None] * gm[None, :] * offs[cl]
    else:
        mean = lib[:, None] * gm[None, :]
    r = 1.0 / disp
    lam = rng.gamma(r, mean / r)
    counts = rng.poisson(lam)
    counts = np.minimum(counts, 65535)
    nzr, nzc = np.nonzero(counts)
    vals = counts[nzr, nzc].astype(np.uint16)
    rowcnt = np.bincount(nzr, minlength=rows)
    return rowcnt, nzc.astype(np.int32), vals, cl


def nb_counts(num_cells: int, num_genes: int = 2000, seed: int = 0, *,
              density: float | None = 0.05, mu: float | None = None,
              sigma: float = 1.5, disp: float = 0.3, lib_sigma: float = 0.4,
              clusters: int = 0, cluster_sigma: float = 0.8,
              workers: int | None = None) -> CountMatrix:
    if mu is None:
        mu = mu_for_density(density)
    nchunks = (num_cells + CHUNK - 1) // CHUNK
    jobs = [(seed, ci, min(CHUNK, num_cells - ci * CHUNK), num_genes, mu,
             sigma, disp, lib_sigma, clusters, cluster_sigma)
            for ci in range(nchunks)]
    workers = workers if workers is not None else min(nchunks, os.cpu_count() or 1)
    if workers > 1 and nchunks > 1:
        with ProcessPoolExecutor(workers, mp_context=get_context("spawn")) as ex:
            parts = list(ex.map(_chunk, jobs))
    else:
        parts = [_chunk(j) for j in jobs]
    rowcnt = np.concatenate([p[0] for p in parts])
    indices = np.concatenate([p[1] for p in parts])
    data = np.concatenate([p[2] for p in parts])
    cl = np.concatenate([p[3] for p in parts]) if clusters else None
    keep = rowcnt > 0
    indptr_all = np.zeros(num_cells + 1, dtype=np.int64)
    np.cumsum(rowcnt, out=indptr_all[1:])
    if not keep.all():  # drop empty cells
        rowcnt = rowcnt[keep]
        if cl is not None:
            cl = cl[keep]
    indptr = np.zeros(rowcnt.shape[0] + 1, dtype=np.int64)
    np.cumsum(rowcnt, out=indptr[1:])
    rows = np.repeat(np.arange(indptr.shape[0] - 1), np.diff(indptr))
    rs = np.bincount(rows, weights=data.astype(np.float64),
                     minlength=indptr.shape[0] - 1).astype(np.uint64)
    isf = (np.float32(10000.0) / rs.astype(np.float32)).astype(np.float32)
    return CountMatrix(indptr, indices, data, num_genes, isf,
                       int(data.max()) if data.size else 0, cl)


def cached_nb_counts(num_cells: int, num_genes: int = 2000, seed: int = 0,
                     cache_dir: str | os.PathLike | None = None,
                     **kw) -> CountMatrix:
    """nb_counts() with an on-disk cache (keyed by every argument), so two
    processes benchmarking the same workload generate it once."""
    key = repr((num_cells, num_genes, seed, sorted(kw.items())))
    h = hashlib.sha1(key.encode()).hexdigest()[:16]
    d = Path(cache_dir or os.environ.get("BRISC_GB300_CACHE")
             or Path(tempfile.gettempdir()) / "brisc_gb300_cache")
    f = d / f"nb_{num_cells}x{num_genes}_s{seed}_{h}.npz"
    if f.exists():
        z = np.load(f)
        return CountMatrix(z["indptr"], z["indices"], z["data"], int(z["g"]),
                           z["isf"], int(z["max_count"]),
                           z["clusters"] if "clusters" in z.files else None)
    M = nb_counts(num_cells, num_genes, seed, **kw)
    try:
        d.mkdir(parents=True, exist_ok=True)
        tmp = f.with_suffix(f".{os.getpid()}.npz")
        extra = {"clusters": M.clusters} if M.clusters is not None else {}
        np.savez(tmp, indptr=M.indptr, indices=M.indices, data=M.data,
                 g=M.num_genes, isf=M.isf, max_count=M.max_count, **extra)
        os.replace(tmp, f)
    except OSError:
        pass
    return M


def pca_like(num_cells: int, num_dims: int, components: int, seed: int) -> np.ndarray:
    """Seeded stand-in for principal components (float32, C order): a Gaussian
    mixture of ``components`` centres whose per-dimension scale falls like a
    PCA spectrum (10 / sqrt(1 + dim)), each cell its centre plus 0.35-scaled
    noise. Used where a kNN search needs PCs of a given shape."""
    rng = np.random.default_rng(seed)
    scale = 10.0 / np.sqrt(1.0 + np.arange(num_dims))
    centres = rng.standard_normal((components, num_dims)) * scale
    lab = rng.integers(0, components, num_cells)
    X = centres[lab] + 0.35 * rng.standard_normal((num_cells, num_dims)) * scale
    return np.ascontiguousarray(X.astype(np.float32))


def batched_pcs(num_cells: int, num_dims: int, components: int, num_batches: int,
                seed: int, shift: float = 2.0):
    """Seeded stand-in for the PCs of several batches: ``pca_like`` cells,
    each given a uniformly drawn batch label and its batch's offset (a
    ``shift``-scaled Gaussian vector per batch) -- the batch effect Harmony
    removes. Returns (PCs float32, batch labels uint32)."""
    X = pca_like(num_cells, num_dims, components, seed)
    rng = np.random.default_rng((seed, 1))
    labels = rng.integers(0, num_batches, num_cells).astype(np.uint32)
    offsets = (rng.standard_normal((num_batches, num_dims)) * shift).astype(np.float32)
    return np.ascontiguousarray((X + offsets[labels]).astype(np.float32)), labels
