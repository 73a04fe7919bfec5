"""ORACLE (test infrastructure): FP64 ground truth for the PCA of a sparse matrix.

The operator is the reference's implicitly centred and scaled matrix
A = C . X . W^-1 (brisc/single_cell.py:11960-12032, key ideas 1-4): C centres
each gene, W holds the per-gene sample std clipped at 1e-8. Its top singular
triplets are computed in float64 from the Gram matrix A^T A (genes x genes),
which is exact enough for the leading values and cheap for <= ~50k cells.

Metrics used by the parity tests: relative singular-value error, principal
angles between PC subspaces, sign-aligned per-PC cosines, and the full-matrix
residual ||A^T u_i - s_i v_i|| / s_i that needs no dense copy.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def gene_std64(X) -> tuple[np.ndarray, np.ndarray]:
    X = sp.csr_matrix(X)
    n = X.shape[0]
    s1 = np.asarray(X.sum(axis=0), dtype=np.float64).ravel()
    s2 = np.asarray(X.multiply(X).sum(axis=0), dtype=np.float64).ravel()
    mean = s1 / n
    var = (n * s2 - s1 * s1) / (n * (n - 1.0))
    sd = np.sqrt(np.maximum(var, 0.0))
    sd[sd < 1e-8] = 1e-8
    return mean, sd


def top_svd(X, k: int, sd: np.ndarray | None = None):
    """(S, U, Vt) of the top-k singular triplets of C X W^-1 in float64.

    U is cells x k (left vectors), Vt is k x genes. The sign of each pair is
    fixed so the largest-magnitude entry of Vt[i] is positive."""
    X = sp.csr_matrix(X, dtype=np.float64)
    mean, sd64 = gene_std64(X)
    if sd is not None:
        sd64 = np.asarray(sd, dtype=np.float64)
    n = X.shape[0]
    G = (X.T @ X).toarray() - n * np.outer(mean, mean)
    G = G / np.outer(sd64, sd64)
    evals, evecs = np.linalg.eigh(G)
    order = np.argsort(evals)[::-1][:k]
    S = np.sqrt(np.maximum(evals[order], 0.0))
    Vt = evecs[:, order].T
    flip = np.sign(Vt[np.arange(k), np.argmax(np.abs(Vt), axis=1)])
    Vt *= flip[:, None]
    U = apply_A(X, Vt.T, mean, sd64) / S
    return S, U, Vt


def apply_A(X, Vm, mean, sd):
    """A . Vm for A = C X W^-1 (dense Vm, genes x r)."""
    W = Vm / sd[:, None]
    Y = X @ W
    return Y - (mean @ W)[None, :]


def apply_At(X, Um, mean, sd):
    """A^T . Um (dense Um, cells x r)."""
    Uc = Um - Um.mean(axis=0, keepdims=True)
    return (X.T @ Uc) / sd[:, None]


def sv_from_pcs(PCs) -> np.ndarray:
    return np.linalg.norm(np.asarray(PCs, dtype=np.float64), axis=0)


def rel_sv_error(PCs, S_true) -> np.ndarray:
    s = sv_from_pcs(PCs)
    return np.abs(s - S_true[: s.shape[0]]) / S_true[: s.shape[0]]


def principal_angles(A, B) -> np.ndarray:
    """Principal angles (radians, ascending) between span(A) and span(B)."""
    qa, _ = np.linalg.qr(np.asarray(A, dtype=np.float64))
    qb, _ = np.linalg.qr(np.asarray(B, dtype=np.float64))
    c = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return np.sort(np.arccos(np.clip(c, -1.0, 1.0)))


def max_angle(A, B) -> float:
    return float(principal_angles(A, B).max())


def pc_cosines(PCs, U_true) -> np.ndarray:
    """|cos| between each PC column and the matching true left vector."""
    P = np.asarray(PCs, dtype=np.float64)
    P = P / np.linalg.norm(P, axis=0)
    k = P.shape[1]
    return np.abs(np.sum(P * U_true[:, :k], axis=0))


def align_signs(PCs, ref) -> np.ndarray:
    """Flip columns of PCs to best match ref (sign-aligned comparison)."""
    P = np.array(PCs, dtype=np.float64, copy=True)
    s = np.sign(np.sum(P * np.asarray(ref, dtype=np.float64), axis=0))
    s[s == 0] = 1
    return P * s


def residuals(X, PCs, sd=None) -> np.ndarray:
    """||A A^T u_i - s_i^2 u_i|| / s_i^2 for u_i = PC_i / s_i (full matrix)."""
    X = sp.csr_matrix(X, dtype=np.float64)
    mean, sd64 = gene_std64(X)
    if sd is not None:
        sd64 = np.asarray(sd, dtype=np.float64)
    P = np.asarray(PCs, dtype=np.float64)
    s = np.linalg.norm(P, axis=0)
    Uu = P / s
    AtU = apply_At(X, Uu, mean, sd64)
    AAtU = apply_A(X, AtU, mean, sd64)
    return np.linalg.norm(AAtU - Uu * s**2, axis=0) / s**2


def gap_mask(S, k: int, min_gap: float = 0.01) -> list[int]:
    """Subspace sizes j <= k whose gap S[j-1]/S[j] - 1 exceeds min_gap."""
    return [j for j in range(1, k + 1)
            if j < len(S) and S[j - 1] / S[j] - 1.0 > min_gap]
