"""ORACLE (test infrastructure): NumPy restatement of brisc/hvg.pyx.

Only tests/ import it, as the checker of the GPU's HVG statistics.

- gene_mean_and_variance_csr / _csc (hvg.pyx:9-139, :142-252): per-gene
  uint64 sums of the counts, of their squares, and the nonzero counts; then
  mean = float(sum) * inv_num_cells and var = float(double(inv_num_pairs) *
  (double(n) * double(sumsq) - double(sum)^2)) (hvg.pyx:66-70).
- clipped_sum_csr / _csc (hvg.pyx:255-403, :406-530): counts above the gene's
  clip value count apart; then float(sum) + float(out) * clip and
  float(sumsq) + float(out) * clip * clip (hvg.pyx:320-325). The
  reference's -Ofast build evaluates these as fma(out, clip, sum) and
  fma(out, clip * clip, sumsq); tests/test_oracle.py pins both forms against
  the compiled reference.

Casts follow C: `<unsigned long long>` of a signed integer wraps modulo 2^64,
of a float truncates toward zero; the clip test converts the integer to
float32.
"""
from __future__ import annotations

from fractions import Fraction

import numpy as np

F32, F64, U64 = np.float32, np.float64, np.uint64


def as_u64(data: np.ndarray) -> np.ndarray:
    if data.dtype.kind == "f":
        return np.trunc(data.astype(F64)).astype(U64)
    return data.astype(np.int64).astype(U64) if data.dtype.kind == "i" \
        else data.astype(U64)


def _round_f32(q: Fraction) -> F32:
    """q rounded once to the nearest float32 (ties to even)."""
    if q == 0:
        return F32(0.0)
    sign = -1 if q < 0 else 1
    n, d = abs(q.numerator), q.denominator

    def scaled(e):
        return (n, d << e) if e >= 0 else (n << -e, d)

    e = n.bit_length() - d.bit_length() - 24
    while True:
        nn, dd = scaled(e)
        m = nn // dd
        if m >= 1 << 24:
            e += 1
        elif m < 1 << 23:
            e -= 1
        else:
            break
    e = max(e, -149)  # subnormals share the smallest exponent
    nn, dd = scaled(e)
    m, r = divmod(nn, dd)
    if 2 * r > dd or (2 * r == dd and m & 1):
        m += 1
    with np.errstate(over="ignore"):
        return F32(sign * float(m) * 2.0 ** e)


def fma_f32(a, b, c) -> F32:
    return _round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def _entries(data, indices, indptr, is_csr, cells=None, mask=None,
             rows=None, flat=False):
    """(gene, uint64 value) of every entry the reference visits."""
    ip = np.asarray(indptr, dtype=np.int64)
    ix = np.asarray(indices, dtype=np.int64)
    v = as_u64(np.asarray(data))
    if is_csr:
        if flat:
            return ix, v
        if cells is not None:
            sel = np.concatenate([np.arange(ip[c], ip[c + 1]) for c in cells]) \
                if len(cells) else np.zeros(0, np.int64)
            return ix[sel], v[sel]
        lo, hi = ip[0], ip[rows]
        return ix[lo:hi], v[lo:hi]
    lo, hi = ip[0], ip[-1]
    genes = np.repeat(np.arange(len(ip) - 1), np.diff(ip))
    ix, v = ix[lo:hi], v[lo:hi]
    if mask is not None:
        keep = np.asarray(mask)[ix].astype(bool)
        return genes[keep], v[keep]
    return genes, v


def _sums(genes, vals, g, count_mask=None):
    s = np.zeros(g, U64)
    s2 = np.zeros(g, U64)
    c = np.zeros(g, U64)
    with np.errstate(over="ignore"):
        sq = vals * vals
    if count_mask is None:
        np.add.at(s, genes, vals)
        np.add.at(s2, genes, sq)
        np.add.at(c, genes, np.ones_like(vals))
    else:  # count_mask: entries above the clip value
        np.add.at(s, genes[~count_mask], vals[~count_mask])
        np.add.at(s2, genes[~count_mask], sq[~count_mask])
        np.add.at(c, genes[count_mask], np.ones(int(count_mask.sum()), U64))
    return s, s2, c


def _mean_var(s, s2, c, num_cells):
    n = int(num_cells)
    inv_n = F32(1.0 / n) if n else F32(np.inf)
    pairs = (n * (n - 1)) % (1 << 64)
    inv_p = F32(1.0 / pairs) if pairs else F32(np.inf)
    mean = (s.astype(F32) * inv_n).astype(F32)
    sd = s.astype(F64)
    with np.errstate(invalid="ignore", over="ignore"):
        var = (F64(inv_p) * (F64(n) * s2.astype(F64) - sd * sd)).astype(F32)
    return mean, var, c.astype(np.uint32)


def gene_mean_and_variance_csr(data, indices, indptr, cell_indices, num_cells,
                               num_dataset_genes):
    cells = None if len(cell_indices) == 0 else np.asarray(cell_indices)[:num_cells]
    genes, vals = _entries(data, indices, indptr, True, cells=cells,
                           flat=cells is None)
    return _mean_var(*_sums(genes, vals, num_dataset_genes), num_cells)


def gene_mean_and_variance_csc(data, indices, indptr, cell_mask, num_cells,
                               num_dataset_genes):
    mask = None if len(cell_mask) == 0 else cell_mask
    genes, vals = _entries(data, indices, indptr[:num_dataset_genes + 1], False,
                           mask=mask)
    return _mean_var(*_sums(genes, vals, num_dataset_genes), num_cells)


def _clipped(genes, vals, clip, g):
    clip = np.asarray(clip, dtype=F32)
    over = vals.astype(F32) > clip[genes]
    s, s2, c = _sums(genes, vals, g, count_mask=over)
    fs, fs2, fc = s.astype(F32), s2.astype(F32), c.astype(F32)
    b = np.array([fma_f32(fc[i], clip[i], fs[i]) for i in range(g)], F32)
    q = np.array([fma_f32(fc[i], F32(clip[i] * clip[i]), fs2[i]) for i in range(g)], F32)
    return b, q


def clipped_sum_csr(data, indices, indptr, num_cells, num_dataset_genes,
                    cell_indices, clip_val):
    cells = None if len(cell_indices) == 0 else np.asarray(cell_indices)
    genes, vals = _entries(data, indices, indptr, True, cells=cells, rows=num_cells)
    return _clipped(genes, vals, clip_val, num_dataset_genes)


def clipped_sum_csc(data, indices, indptr, cell_mask, clip_val):
    mask = None if len(cell_mask) == 0 else cell_mask
    genes, vals = _entries(data, indices, indptr, False, mask=mask)
    return _clipped(genes, vals, clip_val, len(indptr) - 1)
