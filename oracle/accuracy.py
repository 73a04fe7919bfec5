"""ORACLE (test and benchmark infrastructure): FP64 accuracy of PCs at any size.

The operator is the reference's implicitly centred and scaled matrix
A = (X - 1 mean^T) D^-1 (brisc/single_cell.py:11960-12032, key ideas 1-4;
D holds the per-gene sample std clipped at 1e-8, brisc/pca.pyx:51-103, 687).
Its truth is the FP64 eigendecomposition of the Gram matrix A^T A (genes x
genes), accumulated in FP64 from dense row chunks -- on the GPU through torch
when a device is given (checker arithmetic only: nothing here is timed or
shipped), else with scipy on the host.

A solution is judged in the gene space, where every quantity is small:
for PCs P = U S (cells x k) its right vectors are V_hat = A^T P / s^2, so

* relative singular-value error |s_i - sigma_i| / sigma_i, with s_i = ||P_i||;
* principal angles between span(V_hat[:, :j]) and the true top-j right
  singular subspace, for every j whose gap sigma_j / sigma_{j+1} - 1 is at
  least `min_gap` (a subspace with no gap is not determined to any accuracy
  by the tolerance the solver stops at);
* the sign-aligned angle of every PC isolated by such gaps on both sides;
* the full-matrix residual ||A^T A v_i - s_i^2 v_i|| / s_i^2 (G v with the
  Gram matrix, no dense copy of A).

Only tests/ and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import numpy as np


def gene_moments64(indptr, indices, values, n: int, g: int):
    """Per-gene mean and clipped sample std of the stored values, in FP64."""
    v = np.asarray(values, dtype=np.float64)
    ix = np.asarray(indices)
    s1 = np.bincount(ix, weights=v, minlength=g)[:g]
    s2 = np.bincount(ix, weights=v * v, minlength=g)[:g]
    mean = s1 / n
    var = (n * s2 - s1 * s1) / (n * (n - 1.0))
    sd = np.sqrt(np.maximum(var, 0.0))
    sd[sd < 1e-8] = 1e-8
    return mean, sd


def _torch_dev(device):
    if device is None:
        return None
    import torch
    return torch.device(device)


def gram64(indptr, indices, values, n: int, g: int, mean, sd, device=None,
           chunk: int = 65536) -> np.ndarray:
    """A^T A in FP64 (g x g)."""
    indptr = np.asarray(indptr, dtype=np.int64)
    dev = _torch_dev(device)
    if dev is None:
        import scipy.sparse as sp
        X = sp.csr_matrix((np.asarray(values, dtype=np.float64), indices, indptr),
                          shape=(n, g))
        G = (X.T @ X).toarray()
    else:
        import torch
        G_t = torch.zeros((g, g), dtype=torch.float64, device=dev)
        for r0 in range(0, n, chunk):
            r1 = min(n, r0 + chunk)
            a, b = int(indptr[r0]), int(indptr[r1])
            rows = np.repeat(np.arange(r1 - r0, dtype=np.int64),
                             np.diff(indptr[r0:r1 + 1]))
            D = torch.zeros((r1 - r0) * g, dtype=torch.float64, device=dev)
            flat = torch.from_numpy(rows * g + np.asarray(indices[a:b], dtype=np.int64))
            D[flat.to(dev)] = torch.from_numpy(
                np.asarray(values[a:b], dtype=np.float64)).to(dev)
            D = D.view(r1 - r0, g)
            G_t += D.T @ D
            del D
        G = G_t.cpu().numpy()
    G = G - n * np.outer(mean, mean)
    return G / np.outer(sd, sd)


def truth(G: np.ndarray, k: int):
    """Top-k singular values and right vectors (g x k) from the Gram matrix."""
    w, Q = np.linalg.eigh(G)
    order = np.argsort(w)[::-1][:k]
    return np.sqrt(np.maximum(w[order], 0.0)), Q[:, order]


def right_vectors(indptr, indices, values, n: int, g: int, mean, sd, PCs,
                  device=None) -> np.ndarray:
    """V_hat = A^T PCs / s^2 (g x k, FP64), s = column norms of PCs."""
    P = np.asarray(PCs, dtype=np.float64)
    s2 = np.sum(P * P, axis=0)
    import scipy.sparse as sp
    X = sp.csr_matrix((np.asarray(values, dtype=np.float64), indices, indptr),
                      shape=(n, g))
    dev = _torch_dev(device)
    if dev is None:
        XtP = np.asarray(X.T @ P)
    else:
        import torch
        T = X.T.tocsr()  # the CSR of X^T (genes x cells)
        Xt = torch.sparse_csr_tensor(
            torch.from_numpy(T.indptr.astype(np.int64)),
            torch.from_numpy(T.indices.astype(np.int64)),
            torch.from_numpy(T.data), size=(g, n)).to(dev)
        Pt = torch.from_numpy(P).to(dev)
        XtP = (Xt @ Pt).cpu().numpy()
        del Xt, Pt, T
    AtP = (XtP - np.outer(mean, P.sum(axis=0))) / sd[:, None]
    return AtP / s2


def principal_angles(A, B) -> np.ndarray:
    qa, _ = np.linalg.qr(np.asarray(A, dtype=np.float64))
    qb, _ = np.linalg.qr(np.asarray(B, dtype=np.float64))
    c = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return np.sort(np.arccos(np.clip(c, -1.0, 1.0)))


def gapped(S, k: int, min_gap: float = 0.01) -> list[int]:
    """Subspace sizes j <= k with S[j-1] / S[j] - 1 >= min_gap."""
    return [j for j in range(1, k + 1) if j < len(S) and S[j - 1] / S[j] - 1.0 >= min_gap]


def isolated(S, k: int, min_gap: float = 0.01) -> list[int]:
    """PC indices (0-based) separated from both neighbours by min_gap."""
    out = []
    for i in range(k):
        lo = i == 0 or S[i - 1] / S[i] - 1.0 >= min_gap
        hi = i + 1 < len(S) and S[i] / S[i + 1] - 1.0 >= min_gap
        if lo and hi:
            out.append(i)
    return out


def subspace_report(Va, Vb, S_true, k: int, min_gap: float = 0.01) -> dict:
    """Angles between two gene-space bases on the gapped subspaces, and the
    sign-aligned angle of each isolated PC."""
    js = gapped(S_true, k, min_gap)
    top = {int(j): float(principal_angles(Va[:, :j], Vb[:, :j]).max()) for j in js}
    iso = isolated(S_true, k, min_gap)
    per = {}
    for i in iso:
        a, b = Va[:, i], Vb[:, i]
        c = abs(float(a @ b) / (np.linalg.norm(a) * np.linalg.norm(b)))
        per[int(i)] = float(np.arccos(min(1.0, c)))
    return {"gapped_j": [int(j) for j in js], "top_j_angle": top,
            "max_top_j_angle": max(top.values()) if top else None,
            "isolated_pcs": [int(i) for i in iso], "pc_angle": per,
            "max_pc_angle": max(per.values()) if per else None,
            "full_angle": float(principal_angles(Va[:, :k], Vb[:, :k]).max())}


def solution_report(PCs, V_hat, S_true, V_true, G, k: int,
                    min_gap: float = 0.01) -> dict:
    """One solution against the FP64 truth."""
    s = np.linalg.norm(np.asarray(PCs, dtype=np.float64), axis=0)
    rel = np.abs(s - S_true[:k]) / S_true[:k]
    Vn = V_hat / np.linalg.norm(V_hat, axis=0)
    res = np.linalg.norm(G @ Vn - Vn * s ** 2, axis=0) / s ** 2
    out = subspace_report(V_hat, V_true, S_true, k, min_gap)
    out.update({"rel_sv_error": rel.tolist(), "max_rel_sv_error": float(rel.max()),
                "max_residual": float(res.max())})
    return out


# ---------------------------------------------------------------------------
# Parity cases at the 50,000 x 2,000 configuration (50 PCs, subspace 100,
# seed 0): the flat-spectrum NB matrix of the plain configuration, and the
# same generator with 13 cell-type clusters, whose leading subspaces are
# separated by gaps of 0.6-3 % (so their angles are determined).
PARITY_CASES = {
    "flat_50k": dict(num_cells=50_000, num_genes=2000, seed=0, density=0.08, clusters=0),
    "clustered_50k": dict(num_cells=50_000, num_genes=2000, seed=0, density=0.08,
                          clusters=13),
}


def fingerprint(indptr, indices, counts) -> np.ndarray:
    """nnz, total count and CRC32s of the index and count bytes: the same
    seeded input on every machine, or a clear mismatch."""
    import zlib
    return np.array([int(indptr[-1]), int(np.asarray(counts, dtype=np.uint64).sum()),
                     zlib.crc32(np.ascontiguousarray(indices, dtype=np.int32).tobytes()),
                     zlib.crc32(np.ascontiguousarray(counts, dtype=np.uint16).tobytes())],
                    dtype=np.uint64)


def parity_input(name: str):
    """(counts matrix, normalised float32 values) of a parity case; the values
    are normalize_csr method 0 (logCP10k) as the reference computes them."""
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    if str(root) not in sys.path:
        sys.path.insert(0, str(root))
    from synth import nb_counts
    from . import clib
    c = nb_counts(**PARITY_CASES[name])
    xn, _, _, _ = clib.normalize_csr(c.indptr, c.data, 0)
    return c, xn
