"""Shared helpers of the Harmony tests: the fixture cases of
tests/golden/harmony.npz with their regenerated inputs, and the agreement
test against the reference's outputs."""
from __future__ import annotations

import hashlib
import json

import numpy as np

# harmony() keywords of the fixture cases that are harmonize() keywords only
_HARMONIZE_ONLY = ("num_clusters", "chunk_size_Harmony")


def case(z, name: str) -> dict:
    from synth import batched_pcs
    n, d, comps, B, seed = (int(v) for v in z[f"{name}_shape"])
    X, labels = batched_pcs(n, d, comps, B, seed)
    assert hashlib.sha256(X.tobytes() + labels.tobytes()).hexdigest() == \
        str(z[f"{name}_fingerprint"]), "regenerated PCs differ from the ones the reference saw"
    kw = json.loads(str(z[f"{name}_kwargs"]))
    hkw = {k: v for k, v in kw.items() if k not in _HARMONIZE_ONLY}
    hkw["chunk_size"] = kw.get("chunk_size_Harmony", min(256, n))
    return dict(PCs=X, batch_labels=labels, num_batches=B, kwargs=kw, harmony_kwargs=hkw,
                Y_init=z[f"{name}_Y_init"], ref_Z=z[f"{name}_Z"],
                ref_R_head=z[f"{name}_R_head"],
                kmeans_iterations=int(z[f"{name}_kmeans_iterations"]))


def check_against(c: dict, Z, R_head, *, z_rel: float, r_abs: float,
                  min_cos: float) -> None:
    """An embedding agrees with the reference's when every entry is within
    z_rel x max |Z| of it, every row points the same way (cosine >= min_cos)
    and the stored rows of R are within r_abs."""
    ref = c["ref_Z"]
    scale = float(np.abs(ref).max())
    dz = float(np.abs(Z - ref).max())
    assert dz <= z_rel * scale, (dz, scale)
    cos = (Z.astype(np.float64) * ref).sum(1) / (
        np.linalg.norm(Z.astype(np.float64), axis=1) * np.linalg.norm(ref.astype(np.float64), axis=1))
    assert cos.min() >= min_cos, cos.min()
    dr = float(np.abs(R_head - c["ref_R_head"]).max())
    assert dr <= r_abs, dr
