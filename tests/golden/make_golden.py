"""Generate tests/golden/*.npz from the reference's own compiled modules.

Run in a checkout that has the reference (built into oracle/_ref by
oracle/build_ref.py). Every fixture stores its inputs as well as the
reference's outputs, so the tests never regenerate data:

* rng.npz        PCG32 outputs, Box-Muller normals and pca.pyx's normalised
                 start vector (brisc/cyutils.pyx:1153-1232, pca.pyx:801-806)
                 for several seeds.
* normalize.npz  normalize_csr outputs (brisc/normalize.pyx:9) for methods
                 0/1/2, with and without a QC mask, on a small NB count matrix.
* tocsc.npz      csr_tocsc (brisc/cysparse.pyx:1179) of the same matrix.
* irlba.npz      irlba PCs (brisc/pca.pyx:661) on clustered NB matrices whose
                 top singular values are separated, plus one flat-spectrum case.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from brisc_gb300.synth import nb_counts  # noqa: E402
from oracle import ref  # noqa: E402

OUT = Path(__file__).resolve().parent
SEEDS = [0, 1, 7, 42, 12345, 2**63 + 5]


def main() -> int:
    M = ref.load()
    if M is None:
        print("reference modules unavailable", file=sys.stderr)
        return 1
    probe = M["ref_probe"]

    rng = {}
    for i, s in enumerate(SEEDS):
        rng[f"seed_{i}"] = np.uint64(s)
        rng[f"rand_{i}"] = probe.raw_rand(s, 64)
        rng[f"normals_{i}"] = probe.raw_normals(s, 4096)
        rng[f"start_{i}"] = probe.start_vector(s, 2000)
    rng["start_small"] = probe.start_vector(0, 37)
    np.savez_compressed(OUT / "rng.npz", **rng)

    C = nb_counts(800, 150, seed=11, density=0.08, workers=1)
    ip32 = C.indptr.astype(np.int32)
    ix32 = C.indices.astype(np.int32)
    data_f = C.data.astype(np.float32)
    qc = (np.arange(C.num_cells) % 5) != 2
    norm = {"indptr": ip32, "indices": ix32, "counts": C.data, "qc": qc}
    for method in (0, 1, 2):
        for tag, q in (("all", None), ("qc", qc)):
            out, rs = ref.normalize(ip32, ix32, data_f, method, 1, q)
            out4, rs4 = ref.normalize(ip32, ix32, data_f, method, 4, q)
            assert np.array_equal(out, out4) and np.array_equal(rs, rs4)
            norm[f"m{method}_{tag}"] = out
            norm[f"rowsums_{tag}"] = rs
    np.savez_compressed(OUT / "normalize.npz", **norm)

    bp, bi, bx = ref.tocsc(ip32, ix32, data_f, C.num_cells, C.num_genes, 4)
    ip64, ix64 = C.indptr.astype(np.int64), C.indices.astype(np.int64)
    bp64, bi64, bx64 = ref.tocsc(ip64, ix64, data_f, C.num_cells, C.num_genes, 3)
    np.savez_compressed(OUT / "tocsc.npz", indptr=ip32, indices=ix32, data=data_f,
                        n_col=C.num_genes, Bp=bp, Bi=bi, Bx=bx, Bp64=bp64,
                        Bi64=bi64, Bx64=bx64)

    cases = [  # (name, cells, genes, clusters, density, k, m, seed)
        ("clustered_a", 5000, 500, 12, 0.08, 10, 20, 3),
        ("clustered_b", 4000, 400, 13, 0.05, 8, 24, 5),
        ("flat", 3000, 300, 0, 0.08, 10, 40, 3),
    ]
    ir = {}
    for name, n, g, cl, dens, k, m, seed in cases:
        Cm = nb_counts(n, g, seed=seed, density=dens, clusters=cl, workers=1)
        ip = Cm.indptr.astype(np.int32)
        ix = Cm.indices.astype(np.int32)
        x, _ = ref.normalize(ip, ix, Cm.data.astype(np.float32), 0, 4)
        pcs, conv = ref.run_irlba(ip, ix, x, Cm.num_cells, g, k, m, 1e-6, 100,
                                  seed=0, num_threads=4)
        pcs1, conv1 = ref.run_irlba(ip, ix, x, Cm.num_cells, g, k, m, 1e-6, 100,
                                    seed=0, num_threads=1)
        assert np.array_equal(pcs, pcs1), "reference not thread-count invariant"
        ir[f"{name}_indptr"] = ip
        ir[f"{name}_indices"] = ix
        ir[f"{name}_counts"] = Cm.data
        ir[f"{name}_data"] = x
        ir[f"{name}_shape"] = np.array([Cm.num_cells, g, k, m])
        ir[f"{name}_pcs"] = pcs
        ir[f"{name}_converged"] = np.array(conv)
    np.savez_compressed(OUT / "irlba.npz", **ir)
    for f in sorted(OUT.glob("*.npz")):
        print(f.name, f.stat().st_size)
    return 0


if __name__ == "__main__":
    sys.exit(main())
