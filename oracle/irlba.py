"""ORACLE (test infrastructure): NumPy restatement of the reference's IRLBA.

Follows the deterministic parallel code path of brisc/pca.pyx:661-1257 step by
step in float32 -- the per-gene clipped std (pca.pyx:51-103), the start vector
(pca.pyx:801-806), the raw matvec (pca.pyx:440-475) with the centring fused
into the U pass (pca.pyx:997-1090), the rmatvec (pca.pyx:478-511), the V-side
Gram-Schmidt (pca.pyx:1103-1171), LAPACK sgesdd of B (pca.pyx:1178), the
convergence test (pca.pyx:1180-1202), the restart rotation (pca.pyx:1210-1231)
and the final PCs (pca.pyx:1239-1255).

Knobs that the GPU implementation exposes are mirrored so the checker can
model it: ``reorth_passes`` (1 = the reference's single classical
Gram-Schmidt pass, 2 = CGS2, 0 = the GPU's adaptive mode: on either side a
second pass only at steps where the first kept less than half of the squared
norm) and ``sd`` (the per-gene std to use). When
``max_iterations`` runs out without convergence, the reference rotates U once
more and then multiplies by Ub again, reading buffer columns left from an
earlier restart (pca.pyx:1210-1215, 1253); those contents are not defined by
the algorithm, so this restatement (like the GPU product) returns the Ritz
vectors of the final SVD instead.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import it.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg.lapack as lapack
import scipy.sparse as sp

from . import clib

F32 = np.float32


def clipped_stddev(Xcsr) -> np.ndarray:
    csc = Xcsr.tocsc()
    csc.sort_indices()
    return clib.clipped_stddev_csc(csc.data, csc.indptr, Xcsr.shape[0])


def irlba(X, k: int = 50, subspace_size: int = 100, tolerance: float = 1e-6,
          max_iterations: int = 100, seed: int = 0, *,
          reorth_passes: int = 1, sd: np.ndarray | None = None,
          start: np.ndarray | None = None) -> dict:
    """X: scipy CSR, float32 normalised values (cells x genes)."""
    X = sp.csr_matrix(X, dtype=F32)
    n, g = X.shape
    m = int(subspace_size)
    Xt = sp.csr_matrix(X.T)  # the CSC copy, used as a CSR of X^T
    if sd is None:
        sd = clipped_stddev(X)
    sd = np.asarray(sd, dtype=F32)
    tol = F32(tolerance)
    U = np.zeros((n, m), dtype=F32, order="F")
    V = np.zeros((g, m), dtype=F32, order="F")
    B = np.zeros((m, m + 1), dtype=F32, order="F")
    V[:, 0] = clib.start_vector(seed, g) if start is None else start
    rem = np.zeros(g, dtype=F32)
    kc, smax, converged = 0, F32(2.4221817809573368e-05), False
    Ub = Sb = Vbt = None
    restarts = steps = second_passes = second_passes_v = 0
    for it in range(max_iterations):
        j = kc
        while True:
            y = (X @ (V[:, j] / sd)).astype(F32)              # pca.pyx:991-995
            mean = F32(y.sum(dtype=F32) / F32(n))
            if j > 0:                                          # pca.pyx:997-1052
                Uj = U[:, :j]
                w = (Uj.T @ y).astype(F32)
                y0c = (y - mean).astype(F32)
                y = (y - (mean + Uj @ w)).astype(F32)
                second = reorth_passes == 2 or (
                    reorth_passes == 0
                    and F32(np.dot(y, y)) < F32(0.5) * F32(np.dot(y0c, y0c)))
                second_passes += int(second)
                for _ in range(1 if second else 0):
                    w = (Uj.T @ y).astype(F32)
                    y = (y - Uj @ w).astype(F32)
            else:                                              # pca.pyx:1053-1079
                y = (y - mean).astype(F32)
            alpha = F32(np.sqrt(F32(np.dot(y, y))))
            alpha = max(alpha, F32(1e-8))
            U[:, j] = y * (F32(1) / alpha)                     # pca.pyx:1086-1090
            B[j, j] = alpha
            z = ((Xt @ U[:, j]) / sd).astype(F32)              # pca.pyx:1096-1101
            z = (z - alpha * V[:, j]).astype(F32)
            Vj = V[:, :j + 1]
            z0 = z
            for p in range(1 if reorth_passes == 1 else 2):    # pca.pyx:1114-1128
                if p == 1 and reorth_passes == 0:
                    if F32(np.dot(z, z)) >= F32(0.5) * F32(np.dot(z0, z0)):
                        break
                    second_passes_v += 1
                w = (Vj.T @ z).astype(F32)
                z = (z - Vj @ w).astype(F32)
            steps += 1
            if j < m - 1:
                beta = max(F32(np.sqrt(F32(np.dot(z, z)))), F32(1e-8))
                V[:, j + 1] = z * (F32(1) / beta)              # pca.pyx:1164-1170
                B[j, j + 1] = beta
                j += 1
            else:
                rem = z                                         # pca.pyx:1129-1162
                break
        restarts += 1
        Ub, Sb, Vbt, info = lapack.sgesdd(B, compute_uv=1, full_matrices=0)
        if info != 0:
            raise RuntimeError(f"sgesdd failed with info={info}")
        rn = F32(np.sqrt(F32(np.dot(rem, rem))))               # pca.pyx:1181
        rem = (rem / rn).astype(F32)
        smax = max(F32(Sb[0]), smax)                           # pca.pyx:1187
        resid = np.abs(rn * Ub[m - 1, :k].astype(F32))
        nconv = int(np.sum(resid < tol * smax))                # pca.pyx:1190-1193
        if nconv == k:
            converged = True
            break
        kc = min(max(kc, k + nconv), m - 1)                    # pca.pyx:1201-1202
        if it + 1 == max_iterations:
            break
        U[:, :kc] = U @ Ub[:, :kc]                             # pca.pyx:1211
        V[:, :kc] = V @ Vbt.T[:m, :kc]                         # pca.pyx:1218
        V[:, kc] = rem
        B[:] = 0
        for i in range(kc):                                     # pca.pyx:1227-1231
            B[i, i] = Sb[i]
            B[i, kc] = rn * Ub[m - 1, i]
    W = (Ub[:, :k] * Sb[:k]).astype(F32)                       # pca.pyx:1239-1242
    PCs = np.ascontiguousarray(U @ W, dtype=F32)               # pca.pyx:1249-1254
    loadings = np.ascontiguousarray(V @ Vbt[:k, :m].T, dtype=F32)
    return dict(PCs=PCs, S=np.asarray(Sb[:k], dtype=F32), loadings=loadings,
                converged=converged, restarts=restarts, steps=steps, sd=sd,
                second_passes=second_passes, second_passes_v=second_passes_v)
