"""GPU IRLBA against the reference's own irlba at the 50,000 x 2,000
configuration: 50 PCs, subspace 100, tol 1e-6, seed 0, logCP10k float32
values with int32 indices (the reference's CPU-runnable case), through the
drop-in ``irlba`` and through the fused-counts path.

Two inputs from the same NB generator: the flat-spectrum matrix the
configuration names, and the same matrix with 13 cell-type clusters, whose
leading subspaces are separated. Gates, with the FP64 oracle the Gram matrix
of the centred and scaled matrix (oracle/accuracy.py):

* both solves converge;
* relative singular-value error <= 1e-4 against FP64 and against the
  reference;
* principal angle <= 1e-3 rad on every top-j subspace whose gap
  sigma_j / sigma_{j+1} - 1 is at least 1 %, and <= 1e-3 rad for every PC
  isolated by such gaps (sign-aligned), against FP64 and against the
  reference;
* full-matrix residual ||A^T A v - s^2 v|| / s^2 <= 1e-4.

The reference's own figures against FP64 are computed beside the GPU's and
printed with them. On the flat spectrum only j = 1 has a 1 % gap: the other
singular values lie within 1.6 % of each other in steps of 0.01-0.2 %, so a
residual tolerance of 1e-6 does not determine their individual vectors (the
reference's own 50-D angle against FP64 there is 3.6e-3 rad).

The reference runs live when its compiled modules are present (built from its
sources by oracle/build_ref.py); otherwise its singular values and right
vectors come from tests/golden/parity50k.npz, which holds a fingerprint of the
seeded input it was computed on.
"""
import json

import numpy as np
import pytest

import brisc_gb300 as bg
from brisc_gb300 import DeviceMatrix
from oracle import accuracy as A

pytestmark = pytest.mark.gpu

K, M = 50, 100


def _reference(name, c, xn, golden):
    from oracle import ref
    n, g = c.num_cells, c.num_genes
    if ref.load() is not None:
        pcs, conv = ref.run_irlba(c.indptr.astype(np.int32), c.indices.astype(np.int32),
                                  xn, n, g, K, M, 1e-6, 100, seed=0,
                                  match_parallel=False)
        return pcs, conv, "live"
    z = golden("parity50k")
    fp = A.fingerprint(c.indptr, c.indices, c.data)
    if not np.array_equal(fp, z[f"{name}_fingerprint"]):
        pytest.fail("reference modules unavailable and the seeded input differs "
                    "from the fixture's")
    return None, bool(z[f"{name}_converged"]), "fixture"


@pytest.mark.parametrize("name", list(A.PARITY_CASES))
def test_configs0_matches_reference(cuda, golden, name):
    c, xn = A.parity_input(name)
    n, g = c.num_cells, c.num_genes
    ip32, ix32 = c.indptr.astype(np.int32), c.indices.astype(np.int32)
    PCs = np.empty((n, K), dtype=np.float32)
    conv = bg.irlba(data_matvec=xn, indices_matvec=ix32, indptr_matvec=ip32,
                    data_rmatvec=None, indices_rmatvec=None, indptr_rmatvec=None,
                    num_cells=n, num_genes=g, k=K, subspace_size=M, tolerance=1e-6,
                    max_iterations=100, seed=0, match_parallel=False, is_csr=True,
                    num_threads=8, chunk_size=1024, PCs=PCs)
    pcs_ref, conv_ref, src = _reference(name, c, xn, golden)

    ip, ix = c.indptr.astype(np.int64), c.indices.astype(np.int64)
    mean, sd = A.gene_moments64(ip, ix, xn, n, g)
    G = A.gram64(ip, ix, xn, n, g, mean, sd, device=cuda)
    S, V = A.truth(G, K + 1)
    Vg = A.right_vectors(ip, ix, xn, n, g, mean, sd, PCs, device=cuda)
    gpu = A.solution_report(PCs, Vg, S, V, G, K)
    if pcs_ref is not None:
        s_ref = np.linalg.norm(pcs_ref.astype(np.float64), axis=0)
        Vr = A.right_vectors(ip, ix, xn, n, g, mean, sd, pcs_ref, device=cuda)
        refrep = A.solution_report(pcs_ref, Vr, S, V, G, K)
    else:
        z = golden("parity50k")
        s_ref, Vr = z[f"{name}_S"], z[f"{name}_V"].astype(np.float64)
        refrep = json.loads(str(z[f"{name}_report"]))
    vs_ref = A.subspace_report(Vg, Vr, S, K)
    s_gpu = np.linalg.norm(PCs.astype(np.float64), axis=0)
    rel_vs_ref = float(np.max(np.abs(s_gpu - s_ref) / s_ref))
    keys = ("max_rel_sv_error", "max_top_j_angle", "max_pc_angle", "full_angle",
            "max_residual")
    print(json.dumps({"case": name, "reference": src,
                      "gpu_vs_fp64": {k: gpu[k] for k in keys},
                      "reference_vs_fp64": {k: refrep[k] for k in keys},
                      "gpu_vs_reference": {"max_rel_sv": rel_vs_ref,
                                           "max_top_j_angle": vs_ref["max_top_j_angle"],
                                           "max_pc_angle": vs_ref["max_pc_angle"]},
                      "gapped_j": gpu["gapped_j"]}))
    assert conv and conv_ref
    assert gpu["max_rel_sv_error"] <= 1e-4
    assert rel_vs_ref <= 1e-4
    assert gpu["gapped_j"], "the gate needs at least one gapped subspace"
    assert gpu["max_top_j_angle"] <= 1e-3
    assert vs_ref["max_top_j_angle"] <= 1e-3
    if gpu["isolated_pcs"]:
        assert gpu["max_pc_angle"] <= 1e-3
        assert vs_ref["max_pc_angle"] <= 1e-3
    assert gpu["max_residual"] <= 1e-4


def test_configs0_fused_counts_path(cuda):
    """The headline path (raw uint16 counts, logCP10k fused into every product)
    on the clustered 50k input meets the same FP64 gates."""
    c, xn = A.parity_input("clustered_50k")
    n, g = c.num_cells, c.num_genes
    Mx = DeviceMatrix(c.indptr.astype(np.int32), c.indices.astype(np.int32), c.data,
                      n, g, norm="logCP10k", inv_size_factors=c.isf)
    r = Mx.solve(K, M)
    Mx.close()
    ip, ix = c.indptr.astype(np.int64), c.indices.astype(np.int64)
    mean, sd = A.gene_moments64(ip, ix, xn, n, g)
    G = A.gram64(ip, ix, xn, n, g, mean, sd, device=cuda)
    S, V = A.truth(G, K + 1)
    Vg = A.right_vectors(ip, ix, xn, n, g, mean, sd, r.PCs, device=cuda)
    rep = A.solution_report(r.PCs, Vg, S, V, G, K)
    assert r.converged
    assert rep["max_rel_sv_error"] <= 1e-4
    assert rep["max_top_j_angle"] <= 1e-3
    assert rep["max_residual"] <= 1e-4
