"""NumPy restatement of the reference's harmony (brisc/harmonize.pyx:269-871).

Test infrastructure: the checker for brisc_gb300's GPU Harmony, pinned
against the compiled reference in tests/test_oracle.py. Never imported by the
product.

Float32 arithmetic throughout, vectorised per chunk; the reference's matrix
products are sgemm calls and its per-cell sums are sequential, so this
restatement and the reference agree to float rounding amplified by the
iteration, not bit for bit (the tests state the tolerance).
"""
from __future__ import annotations

import numpy as np

F = np.float32


def _pcg_order(n: int, seed: int) -> np.ndarray:
    """The "inside-out" Fisher-Yates order of harmonize.pyx:503-509, drawn
    with PCG32 + Lemire's bounded integers from srand(seed)."""
    from oracle import clib
    return clib.fisher_yates(n, seed)


def normalize_rows(a: np.ndarray) -> np.ndarray:
    """harmonize.pyx:216-241: each row times 1 / sqrt(sum of squares)."""
    a = a.astype(F)
    norm = np.sqrt((a * a).sum(1, dtype=F)).astype(F)
    return (a * (F(1) / norm)[:, None]).astype(F)


def _objective(Z, Y, R, O, E, theta_b, sigma):
    dist = (Z @ Y.T).astype(F)
    with np.errstate(divide="ignore", invalid="ignore"):
        RlogR = np.where(R > 0, R * np.log(R), F(0)).astype(F)
    kmeans_error = F(2) * F((R * (F(1) - dist)).sum(dtype=np.float64))
    entropy = F(sigma) * F(RlogR.sum(dtype=np.float64))
    diversity = (O * np.log((O + E + 1) / (E + 1))).astype(F)
    penalty = F(sigma) * F((diversity * theta_b[:, None]).sum(dtype=np.float64))
    return F(kmeans_error + entropy + penalty)


def _batch_sums(R, batch, B):
    out = np.zeros((B, R.shape[1]), dtype=np.float64)
    np.add.at(out, batch, R.astype(np.float64))
    return out.astype(F)


def harmony(PCs, Z, Y, batch, num_batches: int, max_iterations: int = 10,
            max_clustering_iterations: int = 5, block_proportion: float = 0.05,
            tolerance: float = 0.01, early_stopping: bool = False,
            clustering_tolerance: float = 1e-3, theta: float = 2, tau: float = 0,
            alpha: float = 0.2, sigma: float = 0.1, chunk_size: int = 256,
            seed: int = 0):
    """Returns (Z, R): the Harmony embedding and the soft assignments. Z is
    the row-normalised PCs on entry, Y the k-means centroids of Z."""
    PCs = np.asarray(PCs, dtype=F)
    Z = np.array(Z, dtype=F)
    Y = np.array(Y, dtype=F)
    batch = np.asarray(batch, dtype=np.int64)
    n, d = PCs.shape
    C, B = Y.shape[0], int(num_batches)
    N_b = np.bincount(batch, minlength=B).astype(np.int64)
    Pr_b = (N_b.astype(F) / F(n)).astype(F)
    if tau > 0:
        # harmonize.pyx:416 negates an unsigned count: -N_b wraps to
        # 2^32 - N_b, so base is inf (1 for an empty batch) and theta -inf
        neg = (np.uint32(0) - N_b.astype(np.uint32)).astype(F)
        with np.errstate(over="ignore"):
            base = np.exp((neg / (F(C) * F(tau))).astype(np.float64)).astype(F)
            theta_b = (F(theta) * (F(1) - base * base)).astype(F)
    else:
        theta_b = np.full(B, theta, dtype=F)
    tos = F(2) / F(sigma)
    ens = F(np.exp(-tos))
    # initialisation (harmonize.pyx:412-498)
    dist = (Z @ Y.T).astype(F)
    R = np.exp(tos * (dist - F(1))).astype(F)
    R = (R * (F(1) / R.sum(1, dtype=F))[:, None]).astype(F)
    E = (Pr_b[:, None] * R.sum(0, dtype=F)[None, :]).astype(F)
    O = _batch_sums(R, batch, B)
    prev = _objective(Z, Y, R, O, E, theta_b, sigma)
    Y = normalize_rows(Y)
    order = _pcg_order(n, seed)
    # an unsigned long long times a float in the reference: a float product
    block = int(np.ceil(F(n) * F(block_proportion)))
    objective = prev
    for _ in range(max_iterations):
        past = []
        for ci in range(1, max_clustering_iterations + 1):
            Y = normalize_rows((R.T @ Z).astype(F))
            for b0 in range(0, n, block):
                cells_b = order[b0:min(b0 + block, n)]
                dE_tot = np.zeros((B, C), dtype=F)
                dO_tot = np.zeros((B, C), dtype=F)
                for c0 in range(0, len(cells_b), chunk_size):
                    cells = cells_b[c0:c0 + chunk_size]
                    old = R[cells]
                    dO = -_batch_sums(old, batch[cells], B)
                    dE = (-Pr_b[:, None] * old.sum(0, dtype=F)[None, :]).astype(F)
                    Eij = E + dE
                    Oij = O + dO
                    ratio = (ens * ((Eij + 1) / (Oij + Eij + 1)) ** theta_b[:, None]).astype(F)
                    dist = (tos * (Z[cells] @ Y.T)).astype(F)
                    Rn = (np.exp(dist) * ratio[batch[cells]]).astype(F)
                    Rn = (Rn * (F(1) / Rn.sum(1, dtype=F))[:, None]).astype(F)
                    R[cells] = Rn
                    dO_tot += dO + _batch_sums(Rn, batch[cells], B)
                    dE_tot += dE + (Pr_b[:, None] * Rn.sum(0, dtype=F)[None, :]).astype(F)
                E = (E + dE_tot).astype(F)
                O = (O + dO_tot).astype(F)
            if early_stopping or ci == max_clustering_iterations:
                objective = _objective(Z, Y, R, O, E, theta_b, sigma)
                if early_stopping:
                    if ci <= 3:
                        past.append(objective)
                    else:
                        last_two = past[1] + past[2]
                        if (past[0] + last_two) - (last_two + objective) < \
                                clustering_tolerance * abs(past[0] + last_two):
                            break
                        past = [past[1], past[2], objective]
        # correction (harmonize.pyx:758-818)
        W = np.zeros((C, B + 1, d), dtype=F)
        for k in range(C):
            inv1 = np.zeros((B + 1, B + 1), dtype=F)
            inv2 = np.eye(B + 1, dtype=F)
            norm = F(0)
            keep = O[:, k] >= F(1e-5) * N_b.astype(F)
            for i in range(B):
                if keep[i]:
                    factor = F(1) / (O[i, k] + E[i, k] * F(alpha))
                    inv1[i, i] = factor
                    inv2[B, i] = -O[i, k] * factor
                    norm += O[i, k] * (F(1) + inv2[B, i])
            norm = F(1) / norm
            inv1[B, B] = norm
            inv1[B, :B] = inv2[B, :B] * norm
            inv = (inv1.T @ inv2).astype(F)
            rs = np.zeros((d, B + 1), dtype=F)
            rs[:, :B] = (PCs.T.astype(np.float64) @ (
                R[:, k, None].astype(np.float64) * (batch[:, None] == np.arange(B)))).astype(F)
            rs[:, :B] *= keep[None, :]
            rs[:, B] = rs[:, :B].sum(1, dtype=F)
            W[k] = (inv @ rs.T).astype(F)
        Z = (PCs - np.einsum("nk,nkd->nd", R, W[:, batch, :].transpose(1, 0, 2))).astype(F)
        if prev - objective < tolerance * abs(prev):
            return Z, R
        prev = objective
        Z = normalize_rows(Z)
    return Z, R
