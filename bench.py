"""Benchmark: seconds per IRLBA PCA solve on 1,000,000 cells x 2,000 genes.

One step = one full PCA solve (50 PCs, Krylov subspace 100, tol 1e-6, seed 0)
of a synthetic negative-binomial count matrix (~5 % density, ~100M stored
entries, uint16 counts, int32 gene indices, float32 logCP10k size factors)
with the normalisation fused into the sparse products. The matrix is
generated on the host from seeded per-chunk streams (identical on every
machine) and is larger than L2, as are the Lanczos bases.

  value  device-resident solve time (matrix already in HBM) per solve
  e2e    the same solve through the C ABI with host buffers: host->device copy
         of the counts, device layout build, solve, device->host copy of the PCs
  roofline  the sparse product with the most device time: its algorithmic
         bytes per launch (uint16 count + int32 index per stored entry, plus
         offsets, factors and vectors) / its CUDA-event time, against the
         measured HBM copy peak; layout_frac is the same with the bytes the
         sliced-ELL layout actually streams (2 bytes per entry)
  cpu_baseline  the reference's own irlba (compiled from its sources) on this
         machine's host cores, one solve of the whole matrix
  accuracy  the GPU's PCs and the reference's against an FP64 oracle of the
         whole matrix, and against each other

`--impl reference` times the reference's CPU implementation alone (rank 0).
Multi-GPU (`--gpus N` under torchrun): N independent replicas, one per GPU;
the solve itself does not shard ("replicas only").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("s/solve & SpMM HBM GB/s (1M×2000, 50 PCs); batched/served "
          "solves/s, p99 vs plain")
UNIT = "s/solve"
WORKLOADS = {
    # name: (cells, genes, density, k, m)
    "plain_1m": (1_000_000, 2000, 0.05, 50, 100),
    "plain_50k": (50_000, 2000, 0.08, 50, 100),
    # the large solve: ~1B stored entries (int64 offsets), 100 PCs
    "large_10m": (10_000_000, 2000, 0.05, 100, 200),
    # 64 cell-type subsets of one shared matrix, 30 PCs each (m = 60)
    "batched_3m": (3_000_000, 2000, 0.05, 30, 60),
    # Poisson request stream (shapes drawn per request, see run_serve)
    "serve": (0, 0, 0.0, 0, 0),
    # HVG gene statistics (brisc/hvg.pyx) over the same 1M x 2000 counts
    "hvg_1m": (1_000_000, 2000, 0.05, 0, 0),
    # knn_self (brisc/knn.pyx) on 1M cells x 50 PCs, 20 neighbours
    "knn_1m": (1_000_000, 50, 0.0, 20, 0),
    # harmonize() (brisc/harmonize.pyx) on 1M cells x 50 PCs from 4 batches
    "harmony_1m": (1_000_000, 50, 0.0, 4, 0),
    # the 1M x 2000 counts as an .h5ad file, read straight to the device
    "h5ad_1m": (1_000_000, 2000, 0.05, 0, 0),
}
# Generator arguments beyond the density: the large solve has 13 cell-type
# clusters with lognormal(0, 0.8) per-gene mean offsets; their mean factor
# raises the density, so the gene-mean location is recalibrated (-4.24 gives
# ~5 % with the clusters, measured on 50,000 rows).
WORKLOAD_GEN = {"large_10m": {"clusters": 13, "cluster_sigma": 0.8, "mu": -4.24}}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plain_1m", choices=sorted(WORKLOADS))
    ap.add_argument("--cells", type=int, default=0, help="override cell count")
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64 accuracy report of the CPU-baseline leg")
    ap.add_argument("--accuracy", action="store_true",
                    help="FP64 accuracy report even with --no-cpu-baseline")
    ap.add_argument("--svd-mode", type=int, default=0,
                    help="restart SVD: 0 default (merge), 1 FP64 Jacobi, 2 FP32 Jacobi + Newton")
    ap.add_argument("--rotation-mode", type=int, default=0,
                    help="restart rotation of U: 0 default, 1 FP32 SIMT, 2 tensor cores")
    ap.add_argument("--reorth-passes", default="auto",
                    type=lambda x: x if x == "auto" else int(x),
                    help="U-side Gram-Schmidt passes: auto (adaptive), 1 or 2")
    ap.add_argument("--batch-modes", default="sequential,streams,fused",
                    help="batched_3m: which of the sequential, streams and fused runs to "
                         "make (the fused batch is the line's value)")
    ap.add_argument("--concurrency", type=int, default=16,
                    help="concurrent solves (batched_3m, serve)")
    ap.add_argument("--subsets", type=int, default=64)
    ap.add_argument("--serve-rate", type=float, default=20.0, help="requests/s")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-max-cells", type=int, default=2_000_000)
    ap.add_argument("--serve-pool", type=int, default=16)
    ap.add_argument("--serve-seq-requests", type=int, default=200,
                    help="requests the one-at-a-time arm serves (a prefix of the "
                         "stream: at the full stream it would run for minutes)")
    return ap.parse_args()


def reduce_replicas(seconds_or_ms: float, launches: float, device):
    """Across the ranks of a replica run: the largest time (the job ends when
    the slowest replica does) and the summed kernel launches. One rank (or no
    process group): the values themselves."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds_or_ms), float(launches)
    t = torch.tensor([seconds_or_ms], dtype=torch.float64, device=device)
    n = torch.tensor([launches], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n)
    return float(t.item()), float(n.item())


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def workload(args):
    from synth import cached_nb_counts
    n, g, dens, k, m = WORKLOADS[args.workload]
    if args.cells:
        n = args.cells
    gen = dict(WORKLOAD_GEN.get(args.workload, {}))
    if "mu" not in gen:
        gen["density"] = dens
    return cached_nb_counts(n, g, seed=0, **gen), k, m


# ---------------------------------------------------------------------------
class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.idx = gpu_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader",
                 "-i", str(self.idx), "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self) -> dict:
        self.f.flush()
        rows = [r.split(", ") for r in Path(self.f.name).read_text().splitlines()
                if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1].split()[0]))
                smax.append(float(r[2].split()[0]))
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip() == "Active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def reference_solve(C, k: int, m: int, want_pcs: bool = False):
    """One solve of the reference's own irlba (brisc/pca.pyx:661, compiled
    from its sources) on the WHOLE matrix, called as SingleCell.pca() calls it
    (brisc/single_cell.py:12037-12091): logCP10k values from its own
    normalize_csr, CSR for the matvec and a sorted CSC copy for the rmatvec,
    match_parallel=False, every host core, BLAS single-threaded. Only irlba
    itself is timed. Returns (seconds, meta, PCs, normalised values) or None
    when the reference modules are unavailable."""
    from oracle import build_ref, ref
    if ref.load() is None:
        return None
    import scipy.sparse as sp
    n, g = C.num_cells, C.num_genes
    wide = C.nnz >= 2 ** 31
    ip = C.indptr.astype(np.int64 if wide else np.int32)
    ix = C.indices.astype(np.int64 if wide else np.int32)
    threads = os.cpu_count() or 1
    xn, _ = ref.normalize(ip, ix, C.data.astype(np.float32), 0, threads)
    t0 = time.perf_counter()
    csc = sp.csr_matrix((xn, ix, ip), shape=(n, g)).tocsc()
    csc.sort_indices()
    csc_t = (csc.indptr.astype(ip.dtype), csc.indices.astype(ix.dtype), csc.data)
    t_csc = time.perf_counter() - t0
    del csc
    t0 = time.perf_counter()
    pcs, conv = ref.run_irlba(ip, ix, xn, n, g, k, m, 1e-6, 100, 0, threads, 1024,
                              csc=csc_t, match_parallel=False)
    dt = time.perf_counter() - t0
    meta = {"cells": n, "threads": threads, "converged": conv,
            "march": build_ref.built_march(), "csc_copy_s": t_csc}
    return dt, meta, (pcs if want_pcs else None), xn


# Restarts and Lanczos steps of the reference's irlba on the plain_1m matrix
# (same seeded generator, 103,626,493 entries), measured offline: restarts by
# bisecting max_iterations on the compiled reference (x86-64 build, 8 threads;
# the reference is thread-count invariant), steps by its NumPy restatement
# (oracle/irlba.py, pinned to it on the golden fixtures), which converges at
# the same restart.
REFERENCE_COUNTS = {"plain_1m": {"restarts": 69, "lanczos_steps": None,
                                 "how": "bisection of max_iterations on the compiled "
                                        "reference; steps from its NumPy restatement"}}


def run_reference(args):
    ws, rank, _ = dist_init(args)
    if rank != 0:
        return 0
    if args.workload in ("hvg_1m", "knn_1m", "harmony_1m", "h5ad_1m"):
        print(json.dumps({"impl": "reference", "workload": args.workload, "unavailable":
                          "this workload times the reference's own functions inside its "
                          "own line (cpu_baseline)"}))
        return 0
    if args.workload in ("batched_3m", "serve"):
        print(json.dumps({"impl": "reference", "workload": args.workload, "unavailable":
                          "the reference has no batched or served PCA; this workload's line "
                          "compares against the same solves run one at a time"}))
        return 0
    C, k, m = workload(args)
    from oracle import ref
    if ref.load() is None:
        print(json.dumps({"impl": "reference", "unavailable":
                          "reference modules could not be built on this host"}))
        return 0
    times, meta = [], None
    for i in range(args.warmup + args.steps):
        dt, meta, _, _ = reference_solve(C, k, m)
        if i >= args.warmup:
            times.append(dt)
    v = float(np.mean(times))
    sample = (f"the reference's irlba (brisc/pca.pyx, -Ofast -fopenmp {meta['march']}) "
              f"solving the whole {C.num_cells:,} x {C.num_genes:,} matrix, "
              f"{meta['threads']} threads, irlba alone timed (normalisation and the "
              f"CSC copy are one-off host passes outside it)")
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": v * 1e3, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "impl": "reference",
           "config": config_of(args, C, k, m),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": meta["threads"],
                            "kind": "reference", "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0},
           "solve": {"converged": meta["converged"],
                     **REFERENCE_COUNTS.get(args.workload, {})},
           "step_seconds": times}
    print(json.dumps(out))
    return 0


def cpu_baseline_leg(args, C, k: int, m: int, pcs_dev, dev, ws: int):
    """Rank 0 at N = 1: the reference's irlba on the host cores (one solve of
    the whole matrix) and the FP64 accuracy report of the GPU's PCs (and the
    reference's) -- the checker side of the bench, after the timed region."""
    n = C.num_cells
    cpu, accuracy, ref_pcs, xn = None, None, None, None
    if ws != 1:
        return cpu, accuracy
    want_acc = (not args.no_cpu_baseline and not args.no_accuracy) or args.accuracy
    if not args.no_cpu_baseline:
        try:
            res = reference_solve(C, k, m, want_pcs=want_acc)
        except Exception as e:  # noqa: BLE001
            print(f"[bench] cpu baseline failed: {e}", file=sys.stderr)
            res = None
        if res is not None:
            dt, meta, ref_pcs, xn = res
            cpu = {"value": dt, "unit": UNIT, "cores": meta["threads"],
                   "kind": "reference",
                   "sample": f"the reference's irlba ({meta['march']} build) solving "
                             f"the whole {n:,}-cell matrix once, irlba alone timed",
                   "converged": meta["converged"]}
    if want_acc:
        try:
            if xn is None:  # logCP10k values as float32, as normalize_csr writes them
                rows = np.repeat(np.arange(n), np.diff(C.indptr))
                xn = np.log1p(C.data.astype(np.float32) * C.isf[rows]).astype(np.float32)
            accuracy = accuracy_leg(C, xn, pcs_dev.cpu().numpy(), ref_pcs, k, dev)
        except Exception as e:  # noqa: BLE001
            print(f"[bench] accuracy report failed: {e}", file=sys.stderr)
    return cpu, accuracy


def accuracy_leg(C, xn, gpu_pcs, ref_pcs, k: int, device) -> dict:
    """GPU PCs and the reference's PCs against the FP64 oracle (the Gram
    matrix of the whole centred, scaled matrix) and against each other:
    relative singular-value errors, top-j angles on the gapped subspaces,
    isolated-PC angles, full-matrix residuals (oracle/accuracy.py)."""
    from oracle import accuracy as A
    n, g = C.num_cells, C.num_genes
    ip, ix = C.indptr.astype(np.int64), C.indices.astype(np.int64)
    mean, sd = A.gene_moments64(ip, ix, xn, n, g)
    G = A.gram64(ip, ix, xn, n, g, mean, sd, device=device)
    S, V = A.truth(G, k + 1)
    keys = ("max_rel_sv_error", "rel_sv_error", "gapped_j", "max_top_j_angle",
            "top_j_angle", "isolated_pcs", "max_pc_angle", "full_angle",
            "max_residual")
    out = {"oracle": "FP64 eigendecomposition of the Gram matrix of the whole "
                     "centred and scaled matrix",
           "sigma_gap_k": float(S[k - 1] / S[k] - 1.0)}
    Vg = A.right_vectors(ip, ix, xn, n, g, mean, sd, gpu_pcs, device=device)
    rg = A.solution_report(gpu_pcs, Vg, S, V, G, k)
    out["gpu_vs_fp64"] = {key: rg[key] for key in keys}
    if ref_pcs is not None:
        Vr = A.right_vectors(ip, ix, xn, n, g, mean, sd, ref_pcs, device=device)
        rr = A.solution_report(ref_pcs, Vr, S, V, G, k)
        out["reference_vs_fp64"] = {key: rr[key] for key in keys}
        vs = A.subspace_report(Vg, Vr, S, k)
        sg = np.linalg.norm(np.asarray(gpu_pcs, np.float64), axis=0)
        sr = np.linalg.norm(np.asarray(ref_pcs, np.float64), axis=0)
        out["gpu_vs_reference"] = {"max_rel_sv": float(np.max(np.abs(sg - sr) / sr)),
                                   "max_top_j_angle": vs["max_top_j_angle"],
                                   "max_pc_angle": vs["max_pc_angle"],
                                   "full_angle": vs["full_angle"]}
    return out


def config_of(args, C, k, m):
    gen = WORKLOAD_GEN.get(args.workload, {})
    cl = (f", {gen['clusters']} cell-type clusters (lognormal(0, "
          f"{gen['cluster_sigma']}) per-gene mean offsets)") if gen.get("clusters") else ""
    return {"workload": f"{args.workload}: plain IRLBA PCA, {C.num_cells:,} cells x "
                        f"{C.num_genes:,} genes, NB counts at {C.density:.2%} "
                        f"density{cl}, {k} PCs, subspace {m}, tol 1e-6, logCP10k "
                        f"fused",
            "cells": C.num_cells, "genes": C.num_genes, "nnz": C.nnz,
            "num_PCs": k, "subspace_size": m, "value_dtype": "uint16",
            "index_dtype": "int64" if C.nnz >= 2 ** 31 else "int32",
            "l2": "inputs larger than L2 (no flush)",
            "parallelism": f"replicas x{args.gpus}"}


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    ws, rank, local = dist_init(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    torch.cuda.init()
    from brisc_gb300 import DeviceMatrix
    C, k, m = workload(args)
    n, g = C.num_cells, C.num_genes
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # resident matrix (int32 offsets while nnz < 2^31, else int64)
    wide = C.nnz >= 2 ** 31
    ip32 = C.indptr if wide else C.indptr.astype(np.int32)
    idx = C.indices.astype(np.int64) if wide else C.indices
    M = DeviceMatrix(ip32, idx, C.data, n, g, norm="logCP10k",
                     inv_size_factors=C.isf, stream=stream)
    pcs_dev = torch.empty((n, k), dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        r = M.solve(k, m, reorth_passes=args.reorth_passes,
                    rotation_mode=args.rotation_mode, svd_mode=args.svd_mode, PCs=pcs_dev,
                    stream=stream)
    barrier()
    torch.cuda.synchronize()
    infos = []
    with Clocks(local) as clk:
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            r = M.solve(k, m, reorth_passes=args.reorth_passes,
                        rotation_mode=args.rotation_mode, svd_mode=args.svd_mode, PCs=pcs_dev,
                        profile=True, stream=stream)
            infos.append(r.info)
        stop.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = start.elapsed_time(stop)
    clocks = clk.summary()
    ms_max, launch_total = reduce_replicas(
        ms, float(sum(i["kernel_launches"] for i in infos)), dev)
    value = ms_max / 1e3 / (args.steps * ws)
    last = r
    layout = M.layout
    M.close()

    # end-to-end through the C ABI with pinned host buffers
    e2e_steps = args.e2e_steps or min(3, args.steps)
    h_ip = torch.from_numpy(ip32).pin_memory()
    h_ix = torch.from_numpy(idx).pin_memory()
    h_v = torch.from_numpy(C.data.view(np.int16)).pin_memory()
    h_sf = torch.from_numpy(C.isf).pin_memory()
    h_pcs = torch.empty((n, k), dtype=torch.float32).pin_memory()
    np_views = [t.numpy() for t in (h_ip, h_ix, h_v, h_sf, h_pcs)]
    np_views[2] = np_views[2].view(np.uint16)
    h2d = sum(a.nbytes for a in np_views[:4])
    d2h = np_views[4].nbytes
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        Me = DeviceMatrix(np_views[0], np_views[1], np_views[2], n, g,
                          norm="logCP10k", inv_size_factors=np_views[3],
                          stream=stream)
        Me.solve(k, m, reorth_passes=args.reorth_passes,
                 rotation_mode=args.rotation_mode, svd_mode=args.svd_mode, PCs=np_views[4],
                 stream=stream)
        Me.close()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0)
    e2e_max, _ = reduce_replicas(e2e_s, 0.0, dev)
    e2e_value = e2e_max / (e2e_steps * ws)

    if rank != 0:
        return 0
    # roofline: the kernel class with the most device time
    peaks = measured_peaks()
    tot = lambda key: sum(i[key] for i in infos)  # noqa: E731
    # algorithmic bytes per launch of the sparse products: uint16 count +
    # int32 gene index per stored entry, int32 offsets, the per-cell size
    # factor, the dense input and output vectors
    nnz = int(C.nnz)
    mv_alg = nnz * 6 + (n + 1) * 4 + n * 4 + n * 4 + g * 4
    rmv_alg = nnz * 6 + (g + 1) * 4 + n * 4 + n * 4 + g * 4
    classes = {
        "spmv_csr (X.v)": (tot("matvec_seconds"), mv_alg * tot("lanczos_steps")),
        "rmatvec_panels (X^T.u)": (tot("rmatvec_seconds"), rmv_alg * tot("rmatvecs")),
        "u_pass (dots/update)": (tot("reorth_seconds"), tot("reorth_bytes")),
        "restart_rotation": (tot("rotation_seconds"), tot("rotation_bytes")),
        "v_step": (tot("vstep_seconds"), 0.0),
        "small_svd": (tot("svd_seconds"), 0.0),
    }
    # the roofline entry: the sparse product with the most device time (the
    # path's bandwidth-bound kernels); the other classes go into time_share
    avg_row = nnz / max(n, 1)
    if layout == "sell":  # sliced-ELL rows / (panel, gene) segments
        kern = {"spmv_csr (X.v)": "k_xv_sell", "rmatvec_panels (X^T.u)": "k_xt_sell"}
    else:
        kern = {"spmv_csr (X.v)": "k_spmv_rows" if avg_row >= 64 else "k_spmv_seg",
                # the compact 16-bit panel copy serves X^T.u for up to 2048 genes
                "rmatvec_panels (X^T.u)": "k_rmat_seg16" if g <= 2048 else "k_rmat_seg"}
    dominant = max(kern, key=lambda c: classes[c][0])
    secs, byts = classes[dominant]
    launches_dom = tot("lanczos_steps") if dominant.startswith("spmv") else tot("rmatvecs")
    achieved = byts / secs / 1e9 if secs > 0 else None
    traffic = dram_traffic(kern[dominant], nnz)
    sp_secs = tot("matvec_seconds") + tot("rmatvec_seconds")
    sp_bytes = classes["spmv_csr (X.v)"][1] + classes["rmatvec_panels (X^T.u)"][1]
    roof = {"bound": "hbm", "kernel": f"{kern[dominant]} {dominant}",
            "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"] if achieved else None,
            "peak_source": peaks["source"], "traffic": traffic,
            "algorithmic_bytes_per_launch": byts / launches_dom if launches_dom else None,
            "launch_us": secs / launches_dom * 1e6 if launches_dom else None,
            "spmm_achieved_gbs": sp_bytes / sp_secs / 1e9 if sp_secs else None,
            "spmm_frac": (sp_bytes / sp_secs / 1e9 / peaks["hbm_gbs"]) if sp_secs else None,
            # the bytes the layout actually streams per launch (2-byte entries,
            # descriptors, vectors) over the same time: DRAM-side utilisation
            "layout_bytes_per_launch": (last.info["matvec_bytes"]
                                        if dominant.startswith("spmv")
                                        else last.info["rmatvec_bytes"]),
            "layout_frac": ((last.info["matvec_bytes"] if dominant.startswith("spmv")
                             else last.info["rmatvec_bytes"]) * launches_dom / secs
                            / 1e9 / peaks["hbm_gbs"]) if secs > 0 else None,
            "layout": layout,
            "u_pass_achieved_gbs": (classes["u_pass (dots/update)"][1]
                                    / classes["u_pass (dots/update)"][0] / 1e9)
            if classes["u_pass (dots/update)"][0] else None,
            "time_share": {c: classes[c][0] / (ms_max / 1e3) for c in classes}}
    cpu, accuracy = cpu_baseline_leg(args, C, k, m, pcs_dev, dev, ws)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms_max / args.steps, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "config": config_of(args, C, k, m),
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                   "d2h_bytes_per_step": d2h},
           "roofline": roof, "cpu_baseline": cpu, "accuracy": accuracy,
           "clocks": clocks,
           "gpu_launches": int(launch_total),
           "solve": {"restarts": last.info["restarts"],
                     "lanczos_steps": last.info["lanczos_steps"],
                     "second_passes": last.info["second_passes"],
                     "converged": last.converged,
                     "seconds_host": last.info["seconds"],
                     "reference": REFERENCE_COUNTS.get(args.workload)}}
    print(json.dumps(out))
    return 0


def subset_sizes(n: int, count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """`count` subset sizes drawn log-uniform on [lo, hi], scaled to sum to n."""
    rng = np.random.default_rng(seed)
    raw = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    sizes = np.maximum(np.floor(raw * n / raw.sum()), 2).astype(np.int64)
    sizes[np.argmax(sizes)] += n - sizes.sum()
    return sizes


def run_batched(args):
    """Batched subset PCAs: one shared 3M x 2000 matrix partitioned into 64
    cell-type subsets (sizes log-uniform on [2k, 400k]); one 30-PC IRLBA per
    subset, each centred and scaled over its own cells. Sequential solves
    (one at a time) against the lock-step batch (every step kernel one launch
    over all subsets), with independent solves on --concurrency streams
    beside it."""
    import torch
    from brisc_gb300.batch import SharedMatrix, pca_subsets
    torch.cuda.init()
    C, k, m = workload(args)
    n, g = C.num_cells, C.num_genes
    sizes = subset_sizes(n, args.subsets, 2000, 400_000, seed=1)
    perm = np.random.default_rng(2).permutation(n)
    bounds = np.concatenate([[0], np.cumsum(sizes)])
    subsets = [np.sort(perm[bounds[i]:bounds[i + 1]]) for i in range(len(sizes))]
    S = SharedMatrix(C.indptr, C.indices, C.data, n, g, inv_size_factors=C.isf)
    for _ in range(max(args.warmup, 1)):  # warm the kernels on the smallest subsets
        pca_subsets(S, sorted(subsets, key=len)[:4], num_PCs=k, concurrency=4, mode="streams")
        pca_subsets(S, sorted(subsets, key=len)[:4], num_PCs=k, concurrency=4, mode="fused")
    torch.cuda.synchronize()
    modes = set(args.batch_modes.split(","))
    seq = strm = None
    t_seq = t_strm = float("nan")
    if "sequential" in modes:
        t0 = time.perf_counter()
        seq = pca_subsets(S, subsets, num_PCs=k, concurrency=1, mode="streams")
        t_seq = time.perf_counter() - t0
    if "streams" in modes:
        t0 = time.perf_counter()
        strm = pca_subsets(S, subsets, num_PCs=k, concurrency=args.concurrency,
                           mode="streams")
        t_strm = time.perf_counter() - t0
    binfo = {}
    with Clocks(0) as clk:
        torch.cuda.nvtx.range_push("batch")  # selects the batch's kernels for ncu
        t0 = time.perf_counter()
        bat = pca_subsets(S, subsets, num_PCs=k, concurrency=args.concurrency, mode="fused",
                          info=binfo)
        t_bat = time.perf_counter() - t0
        torch.cuda.nvtx.range_pop()
    same = all(np.array_equal(o.result.PCs, b.result.PCs)
               for other in (seq, strm) if other is not None
               for o, b in zip(other, bat))
    from brisc_gb300.serve import percentile
    lat = [r.seconds for r in bat]

    def solve_bytes(info: dict) -> float:
        # algorithmic bytes of one solve: its products, Gram-Schmidt passes
        # and restart rotations
        return (info["lanczos_steps"] * info["matvec_bytes"]
                + info["rmatvecs"] * info["rmatvec_bytes"]
                + info["reorth_bytes"] + info["rotation_bytes"])
    total_bytes = sum(solve_bytes(r.result.info) for r in bat)
    launches = int(binfo["kernel_launches"])  # the fused batch's own launches
    launches_seq = sum(int(r.result.info["kernel_launches"]) for r in seq) if seq else None
    steps = [int(r.result.info["lanczos_steps"]) for r in bat]
    peak = measured_peaks()["hbm_gbs"]

    def ratio(a, b):  # None where a run was not made
        return None if a != a or b != b else a / b
    out = {"metric": "batched subset PCAs: solves/s (64 subsets of 3M x 2000, 30 PCs)",
           "value": len(subsets) / t_bat, "unit": "solves/s", "n_gpus": 1,
           "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"batched_3m: {n:,} cells x {g} genes, "
                                  f"{C.nnz:,} stored entries, {len(subsets)} subsets "
                                  f"of {sizes.min():,}-{sizes.max():,} cells, "
                                  f"{k} PCs, subspace {2 * k}",
                      "mode": "fused lock-step batch (one launch per step kernel "
                              "over all subsets)",
                      "layout_threads": args.concurrency},
           "sequential_solves_per_s": ratio(len(subsets), t_seq),
           "vs_sequential": ratio(t_seq, t_bat),
           "batch_seconds": t_bat, "sequential_seconds": ratio(t_seq, 1.0),
           "layout_build_seconds": binfo.get("build_seconds"),
           "streams": {"concurrency": args.concurrency, "seconds": ratio(t_strm, 1.0),
                       "solves_per_s": ratio(len(subsets), t_strm),
                       "vs_sequential": ratio(t_seq, t_strm)},
           "bit_identical_to_sequential": same if seq is not None else None,
           "subset_seconds_p50": percentile(lat, 50),
           "subset_seconds_p99": percentile(lat, 99),
           "converged": int(sum(r.result.converged for r in bat)),
           # the subsets partition the cells: a step of every subset reads each
           # stored entry once, whether in one pass or in one pass per subset
           "bytes": {"total_algorithmic": total_bytes,
                     "per_solve_mean": total_bytes / len(bat),
                     "batch_gbs": total_bytes / t_bat / 1e9,
                     "batch_frac": total_bytes / t_bat / 1e9 / peak,
                     "sequential_frac": ratio(total_bytes / 1e9 / peak, t_seq)},
           "kernel_launches": launches,
           "kernel_launches_sequential": launches_seq,
           "launches_per_s_batch": launches / t_bat,
           "lanczos_steps": {"min": min(steps), "max": max(steps),
                             "total": int(sum(steps))},
           "clocks": clk.summary()}
    print(json.dumps(out))
    return 0


def serve_requests(args):
    """The request stream: Poisson arrivals at --serve-rate for --serve-seconds.
    Each request draws cells log-uniform on [5k, --serve-max-cells], genes
    uniform on [1k, 4k], density uniform on [3%, 8%] and 20-100 PCs; the count
    matrices come from a pool of --serve-pool seeded matrices (host generation
    of a fresh matrix per request would outrun the solves)."""
    from brisc_gb300.serve import PCARequest
    from synth import cached_nb_counts
    rng = np.random.default_rng(11)
    pool = []
    for i in range(args.serve_pool):
        cells = int(np.exp(rng.uniform(np.log(5000), np.log(args.serve_max_cells))))
        genes = int(rng.integers(1000, 4001))
        dens = float(rng.uniform(0.03, 0.08))
        pool.append(cached_nb_counts(cells, genes, seed=100 + i, density=round(dens, 3)))
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / args.serve_rate)
        if t > args.serve_seconds:
            break
        arrivals.append(t)
    # the pooled matrices live in pinned host memory, as a server's request
    # buffers would: the uploads are then asynchronous DMA
    import torch
    for c in pool:
        for name in ("indices", "data", "isf"):
            a = getattr(c, name)
            t = torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a)
            pinned = t.pin_memory().numpy()
            setattr(c, name, pinned.view(np.uint16) if a.dtype == np.uint16 else pinned)
    reqs = []
    for i, _ in enumerate(arrivals):
        c = pool[i % len(pool)]
        k = int(rng.integers(20, 101))
        reqs.append(PCARequest(c.indptr.astype(np.int32), c.indices, c.data,
                               c.num_genes, c.isf, num_PCs=k, seed=i, tag=i))
    return reqs, arrivals, pool


def run_serve(args):
    """Served PCA requests with continuous batching (--concurrency slots,
    admission by free HBM, aging after 10 s) against plain solves one at a
    time. The stream offers more work than one GPU finishes in its window
    (large requests reach 2M cells), so the served arm's rate is its capacity
    under that mix and its latencies include queueing."""
    import torch
    from brisc_gb300.serve import PCAServer, percentile
    torch.cuda.init()
    reqs, arrivals, pool = serve_requests(args)

    def play(slots, rq, arr, saturate=False):
        # saturate: every request queued at t0, so the run measures capacity
        with PCAServer(slots=slots) as srv:
            t0 = time.perf_counter()
            futs = []
            for r, a in zip(rq, arr):
                if saturate:
                    a = 0.0
                d = t0 + a - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                futs.append(srv.submit(r, arrival=t0 + a))
            res = [f.result() for f in futs]
            span = max(x.finish for x in res) - t0
        errs = [x.error for x in res if x.error is not None]
        if errs:
            raise RuntimeError(f"{len(errs)} requests failed: {errs[0]!r}")
        lat = [x.latency for x in res]
        return {"requests": len(res), "solves_per_s": len(res) / span,
                "p50_s": percentile(lat, 50), "p99_s": percentile(lat, 99),
                "span_s": span, "max_running": srv.max_running,
                "requeued": srv.requeued}, res

    warm = PCAServer(slots=2)
    for f in [warm.submit(r) for r in reqs[:2]]:
        f.result()
    warm.close()
    nseq = min(len(reqs), args.serve_seq_requests)
    seq, _ = play(1, reqs[:nseq], arrivals[:nseq])
    with Clocks(0) as clk:
        cb, res = play(args.concurrency, reqs, arrivals)
    out = {"metric": "served PCA requests: solves/s with p50/p99 latency "
                     "(continuous batching vs one at a time)",
           "value": cb["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
           "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"serve: Poisson {args.serve_rate}/s for "
                                  f"{args.serve_seconds} s ({len(reqs)} requests), "
                                  f"cells log-uniform 5k-{args.serve_max_cells:,}, "
                                  f"genes 1k-4k, density 3-8%, 20-100 PCs, "
                                  f"{len(pool)} pooled matrices",
                      "slots": args.concurrency,
                      "sequential_arm": f"the first {nseq} requests of the same "
                                        "stream, one at a time"},
           "p50_s": cb["p50_s"], "p99_s": cb["p99_s"],
           "max_running": cb["max_running"], "requeued": cb["requeued"],
           "span_s": cb["span_s"],
           "sequential": seq,
           "vs_sequential": cb["solves_per_s"] / seq["solves_per_s"],
           "converged": int(sum(x.result.converged for x in res)),
           "clocks": clk.summary()}
    print(json.dumps(out))
    return 0


def dram_traffic(kernel: str, nnz: int):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/dram_traffic.txt), scaled by stored entries to this workload."""
    p = ROOT / "profiles" / "dram_traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        f = line.split()
        if len(f) == 4 and f[0] == kernel:
            return float(f[3]) * nnz / float(f[2])
    return None


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def run_hvg(args):
    """HVG gene statistics (brisc/hvg.pyx) on the 1M x 2000 NB counts. One step
    is gene_mean_and_variance_csr plus clipped_sum_csr over every cell, on the
    device-resident CSR (uint16 counts, int32 indices); e2e makes the same two
    calls on host arrays (each call copies its inputs to the device). The
    reference's own compiled functions on the host cores are the CPU baseline
    and the full-size parity check."""
    import ctypes as C

    import torch

    from brisc_gb300 import _lib as L
    from brisc_gb300 import hvg
    torch.cuda.init()
    dev = torch.device("cuda", 0)
    Cm, _, _ = workload(args)
    n, g, nnz = Cm.num_cells, Cm.num_genes, int(Cm.data.shape[0])
    ip, ix = Cm.indptr.astype(np.int32), Cm.indices.astype(np.int32)
    data16 = np.ascontiguousarray(Cm.data, dtype=np.uint16)
    # device copies; the uint16 counts travel as int16 words (same bytes)
    d_data = torch.from_numpy(data16.view(np.int16)).to(dev)
    d_ix, d_ip = torch.from_numpy(ix).to(dev), torch.from_numpy(ip).to(dev)
    clip = (np.sqrt(np.float32(n)) * np.linspace(1, 4, g)).astype(np.float32)
    d_clip = torch.from_numpy(clip).to(dev)
    outs = [torch.zeros(g, dtype=torch.float32, device=dev) for _ in range(4)]
    d_nz = torch.zeros(g, dtype=torch.int32, device=dev)
    h = L.HvgInput()
    h.data, h.value_type = d_data.data_ptr(), L.VALUE_U16
    h.indices, h.indptr, h.index_type = d_ix.data_ptr(), d_ip.data_ptr(), L.INDEX_I32
    h.nnz, h.num_major, h.is_csr, h.num_genes, h.on_device = nnz, n, 1, g, 1
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)

    def step():
        L.call("bgpu_gene_mean_var", C.byref(h), n, outs[0].data_ptr(),
               outs[1].data_ptr(), d_nz.data_ptr(), sp)
        L.call("bgpu_clipped_sum", C.byref(h), n, d_clip.data_ptr(),
               outs[2].data_ptr(), outs[3].data_ptr(), sp)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / args.steps
    got = [o.cpu().numpy() for o in outs] + [d_nz.cpu().numpy().view(np.uint32)]

    # e2e: the same two calls on host arrays
    hm, hv, hb, hq = (np.zeros(g, np.float32) for _ in range(4))
    hz = np.zeros(g, np.uint32)
    e2e_steps = args.e2e_steps or min(3, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        hvg.gene_mean_and_variance_csr(data16, ix, ip, np.zeros(0, np.int64), n, g,
                                       hm, hv, hz, 1)
        hvg.clipped_sum_csr(data16, ix, ip, n, g, np.zeros(0, np.int64), clip, hb, hq, 1)
    e2e = (time.perf_counter() - t0) / e2e_steps
    same_paths = all(np.array_equal(a, b) for a, b in
                     zip(got, (hm, hv, hb, hq, hz)))

    alg = 2.0 * (nnz * (2 + 4) + (n + 1) * 4)  # counts + gene indices (+ offsets), twice
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    achieved = alg / sec / 1e9
    cpu, parity = None, None
    if not args.no_cpu_baseline:
        from oracle import ref
        M = ref.load()
        if M is not None and "hvg" in M:
            H = M["hvg"]
            d32 = Cm.data.astype(np.uint32)
            rm, rv, rb, rq = (np.zeros(g, np.float32) for _ in range(4))
            rz = np.zeros(g, np.uint32)
            cores = os.cpu_count() or 1
            t0 = time.perf_counter()
            H.gene_mean_and_variance_csr(d32, ix, ip, np.zeros(0, np.int64), n, g,
                                         rm, rv, rz, cores)
            H.clipped_sum_csr(d32, ix, ip, n, g, np.zeros(0, np.int64), clip, rb, rq, cores)
            t_ref = time.perf_counter() - t0
            cpu = {"value": t_ref, "unit": "s/pass", "cores": cores, "kind": "reference",
                   "sample": "the reference's gene_mean_and_variance_csr and "
                             "clipped_sum_csr on the full matrix (uint32 counts)"}
            parity = all(np.array_equal(a, b) for a, b in
                         zip(got, (rm, rv, rb, rq, rz)))
    out = {"metric": "HVG gene statistics: s per pass (mean/variance + clipped sums, "
                     "1M x 2000)",
           "value": sec, "unit": "s/pass", "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "higher_is_better": False, "dtype": "u64",
           "data": "synthetic",
           "config": {"workload": f"hvg_1m: {n:,} cells x {g:,} genes, {nnz:,} stored "
                                  "uint16 counts, int32 indices, every cell",
                      "l2": "inputs larger than L2 (no flush)"},
           "e2e": {"value": e2e, "unit": "s/pass",
                   "h2d_bytes_per_step": 2 * (nnz * 6 + (n + 1) * 4 + 4 * g),
                   "d2h_bytes_per_step": 5 * 4 * g},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                        "unit": "GB/s", "frac": achieved / peak if peak else None,
                        "traffic": None, "algorithmic_bytes_per_step": alg},
           "cpu_baseline": cpu, "bit_identical_to_reference": parity,
           "host_and_device_paths_identical": same_paths,
           "clocks": clk.summary(), "gpu_launches": 4 * args.steps}
    print(json.dumps(out))
    return 0


def neighbour_agreement(X, so, norms, a, b) -> dict:
    """How two knn_self results compare: rows whose neighbour sets are
    identical, and on the others the worst distance of a differing neighbour
    inside the other list's k-th distance, in units of FP32 rounding of the
    squared norms (<= 1: a near-tie either side may break)."""
    from oracle import knn as oknn
    same = np.all(np.sort(a, 1) == np.sort(b, 1), axis=1)
    rows = np.flatnonzero(~same)
    _, worst = oknn.compare(X, so, norms, a, b, rows=rows[:20000])
    return {"rows_identical": float(same.mean()), "rows_checked": int(min(len(rows), 20000)),
            "worst_tie_excess": float(worst)}


def run_knn(args):
    """knn_self (brisc/knn.pyx:13) over 1M cells x 50 PCs (seeded Gaussian
    mixture with a PCA-like spectrum), 20 neighbours, the reference's default
    cluster counts: its own k-means (brisc/kmeans.pyx:889, compiled from its
    sources, run once on the host, untimed) makes the inputs. A step is one
    knn_self on device-resident inputs; e2e is the same call from host arrays
    through the drop-in (copies included). The reference's knn_self on every
    host core is the CPU baseline and the parity check."""
    import ctypes as C

    import torch

    from brisc_gb300 import _lib as L
    from brisc_gb300 import knn
    from oracle import ref
    from synth import pca_like
    torch.cuda.init()
    dev = torch.device("cuda", 0)
    n, d, _, k, _ = WORKLOADS[args.workload]
    if args.cells:
        n = args.cells
    X = pca_like(n, d, 40, seed=0)
    if ref.load() is None or "kmeans" not in ref.load():
        print(json.dumps({"workload": args.workload, "unavailable":
                          "the reference's kmeans could not be built on this host"}))
        return 0
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    prep = ref.run_kmeans_for_knn(X, num_neighbors=k, seed=0, num_threads=cores)
    t_kmeans = time.perf_counter() - t0
    cs, nc = prep["num_clusters_searched"], len(prep["centroids"])

    def T(a):
        return torch.from_numpy(np.ascontiguousarray(
            a.view(np.int32) if a.dtype == np.uint32 else a)).to(dev)
    dX, dso, dC, dcnt, dnrm = (T(prep[key]) for key in
                               ("X", "sorted_order", "centroids", "num_cells_per_cluster",
                                "cell_norms"))
    dnb = torch.zeros((n, k), dtype=torch.int32, device=dev)
    ddi = torch.zeros((n, k), dtype=torch.float32, device=dev)
    dcd = torch.zeros((n, cs), dtype=torch.float32, device=dev)
    dnc = torch.zeros((n, cs), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp_ = C.c_void_p(stream.cuda_stream)

    def step():
        L.call("bgpu_knn_self", dX.data_ptr(), dso.data_ptr(), dC.data_ptr(),
               dcnt.data_ptr(), dnb.data_ptr(), ddi.data_ptr(), dnrm.data_ptr(),
               dcd.data_ptr(), dnc.data_ptr(), n, d, nc, k, cs, sp_)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / args.steps
    gpu_nbr = dnb.cpu().numpy().view(np.uint32)

    # e2e: host arrays through the drop-in
    hn = np.zeros((n, k), np.uint32)
    hd = np.zeros((n, k), np.float32)
    hcd = np.zeros((n, cs), np.float32)
    hnc = np.zeros((n, cs), np.uint32)
    e2e_steps = args.e2e_steps or min(3, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        knn.knn_self(X=prep["X"], sorted_order=prep["sorted_order"],
                     centroids=prep["centroids"],
                     num_cells_per_cluster=prep["num_cells_per_cluster"],
                     neighbors=hn, distances=hd, cell_norms=prep["cell_norms"],
                     centroid_distances=hcd, nearest_clusters=hnc, num_neighbors=k,
                     num_clusters_searched=cs, num_threads=cores)
    e2e = (time.perf_counter() - t0) / e2e_steps
    same_paths = bool(np.array_equal(hn, gpu_nbr))

    # k-means (the other half of neighbors()): the GPU's on device-resident
    # PCs against the reference's run above, same seed and cluster count
    nck = len(prep["kmeans"]["centroids"])
    kX = torch.from_numpy(X).to(dev)
    kout = dict(cluster_labels=torch.zeros(n, dtype=torch.int32, device=dev),
                min_distances=torch.zeros(n, dtype=torch.float32, device=dev),
                cell_norms=torch.zeros(n, dtype=torch.float32, device=dev),
                centroids=torch.zeros((nck, d), dtype=torch.float32, device=dev),
                centroids_new=torch.zeros((nck, d), dtype=torch.float32, device=dev),
                num_cells_per_cluster=torch.zeros(nck, dtype=torch.int32, device=dev))
    knn.kmeans(X=kX, seed=0, **kout)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    km_it = knn.kmeans(X=kX, seed=0, **kout)
    torch.cuda.synchronize()
    t_km_gpu = time.perf_counter() - t0
    km_same = float((kout["cluster_labels"].cpu().numpy().view(np.uint32) ==
                     prep["kmeans"]["cluster_labels"]).mean())
    kmeans_block = {"gpu_seconds": t_km_gpu, "reference_seconds": t_kmeans,
                    "reference_cores": cores, "iterations": km_it,
                    "reference_iterations": prep["kmeans"]["iterations"],
                    "labels_identical": km_same}
    del kX, kout

    # candidate FLOPs: n C d for the nearest clusters, sum of searched
    # cluster sizes x d for the neighbour search (2 flop per multiply-add)
    near = hnc.astype(np.int64)
    cand = prep["num_cells_per_cluster"].astype(np.int64)[near].sum()
    flops = 2.0 * d * (n * nc + cand)
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12  # TFLOP/s, nominal SIMT FP32
    cpu, parity = None, None
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        rnb, rdi, rnc, _ = ref.run_knn_self(prep, num_threads=cores)
        t_ref = time.perf_counter() - t0
        cpu = {"value": t_ref, "unit": "s/search", "cores": cores, "kind": "reference",
               "sample": "the reference's knn_self on the full 1M-cell input, every "
                         "host core (its k-means outside the timing, as here)"}
        parity = neighbour_agreement(prep["X"], prep["sorted_order"], prep["cell_norms"],
                                     hn, rnb)
        parity["nearest_clusters_rows_identical"] = float(
            np.all(np.sort(hnc, 1) == np.sort(rnc, 1), axis=1).mean())
    out = {"metric": "knn_self: s per search (1M cells x 50 PCs, 20 neighbours)",
           "value": sec, "unit": "s/search", "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "higher_is_better": False, "dtype": "f32",
           "data": "synthetic",
           "config": {"workload": f"knn_1m: {n:,} cells x {d} PCs (Gaussian mixture, "
                                  f"PCA-like spectrum), {k} neighbours, {nc} k-means "
                                  f"clusters, {cs} searched",
                      "l2": "inputs (200 MB PCs) larger than L2 (no flush)",
                      "kmeans_seconds_host": t_kmeans},
           "e2e": {"value": e2e, "unit": "s/search",
                   "h2d_bytes_per_step": int(X.nbytes + n * 8 + nc * (d + 1) * 4),
                   "d2h_bytes_per_step": int(n * (k + cs) * 8)},
           "roofline": {"bound": "fp32-simt", "achieved": flops / sec / 1e12,
                        "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": flops / sec / 1e12 / fp32_peak,
                        "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2.07 GHz)",
                        "traffic": None, "flops_per_step": flops},
           "cpu_baseline": cpu, "agreement_with_reference": parity,
           "host_and_device_paths_identical": same_paths, "kmeans": kmeans_block,
           "clocks": clk.summary(), "gpu_launches": 4 * args.steps}
    print(json.dumps(out))
    return 0


def run_harmony(args):
    """The core of SingleCell.harmonize() (brisc/single_cell.py:13776-13875):
    normalize_rows, k-means on the normalised PCs, harmony
    (brisc/harmonize.pyx:269), with the reference's defaults (100 clusters,
    block_proportion 0.05, chunks of 256, sigma 0.1, theta 2), on 1M cells x
    50 PCs from 4 batches (seeded Gaussian mixture with a PCA-like spectrum
    plus a per-batch offset). A step is one harmonize() on device-resident
    PCs and labels; e2e the same call from host arrays (copies included). The
    reference's own harmonize core on every host core is the CPU baseline and
    the parity check (the embeddings compared row by row)."""
    import torch

    from brisc_gb300 import harmony as H
    from oracle import ref
    from synth import batched_pcs
    torch.cuda.init()
    dev = torch.device("cuda", 0)
    n, d, _, B, _ = WORKLOADS[args.workload]
    if args.cells:
        n = args.cells
    X, lab = batched_pcs(n, d, 30, B, seed=0)
    dX = torch.from_numpy(X).to(dev)
    dlab = torch.from_numpy(lab.view(np.int32)).to(dev)
    stream = torch.cuda.current_stream(dev)
    info = {}

    def step():
        Z, inf = H.harmonize(dX, dlab, B, return_info=True)
        info.update(inf)
        return Z

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            Zd = step()
        e1.record(stream)
        torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / args.steps
    Zg = Zd.cpu().numpy()
    # harmony() alone, from the k-means centroids of the last step's pipeline
    Zn = torch.empty_like(dX)
    H.normalize_rows(dX, Zn)
    nc = info["num_clusters"]
    Y = torch.empty((nc, d), dtype=torch.float32, device=dev)
    Yn = torch.empty_like(Y)
    i32 = dict(dtype=torch.int32, device=dev)
    km_it = H.kmeans(X=Zn, cluster_labels=torch.empty(n, **i32), centroids=Y,
                     centroids_new=Yn, num_cells_per_cluster=torch.empty(nc, **i32),
                     min_distances=torch.empty(n, dtype=torch.float32, device=dev),
                     cell_norms=torch.empty(0, dtype=torch.float32, device=dev),
                     num_kmeans_iterations=25, tolerance=1e-2, chunk_size=min(4096, n),
                     seed=0)
    Y0 = (Yn if km_it & 1 else Y).clone()
    R = torch.empty((n, nc), dtype=torch.float32, device=dev)
    h_times = []
    for _ in range(2):
        Zh, Yh = Zn.clone(), Y0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h_it = H.harmony(PCs=dX, Z=Zh, Y=Yh, R=R, batch_labels=dlab, num_batches=B)
        torch.cuda.synchronize()
        h_times.append(time.perf_counter() - t0)
    del Zh, Yh, R, Zn

    # e2e: host arrays through the drop-in
    e2e_steps = args.e2e_steps or min(3, args.steps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        Zh_host = H.harmonize(X, lab, B)
    e2e = (time.perf_counter() - t0) / e2e_steps
    same_paths = bool(np.array_equal(Zh_host, Zg))

    # FLOPs of the distance-shaped products (2 per multiply-add): per
    # clustering iteration the block passes' Z.Y and R^T Z, per correction
    # round R^T PCs and the Z update; the initial assignments once
    it, ci = info["iterations"], 5
    flops = 2.0 * n * nc * d * (1 + it * (2 * ci + 2))
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    block = int(np.ceil(np.float32(n) * np.float32(0.05)))
    nblocks = -(-n // block)
    launches = 1 + (1 + 6 * info["kmeans_iterations"] + 3) + \
        (2 + it * (ci * (2 + nblocks) + 2))
    cpu, parity = None, None
    if not args.no_cpu_baseline and ref.load() is not None and "harmonize" in ref.load():
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        r = ref.run_harmonize(X, lab, B, num_threads=cores)
        t_ref = time.perf_counter() - t0
        cpu = {"value": t_ref, "unit": "s/harmonize", "cores": cores, "kind": "reference",
               "sample": "the reference's normalize_rows + kmeans + harmony on the full "
                         "1M-cell input, every host core"}
        Zr = r["Z"].astype(np.float64)
        Z64 = Zg.astype(np.float64)
        cos = (Z64 * Zr).sum(1) / (np.linalg.norm(Z64, axis=1) * np.linalg.norm(Zr, axis=1))
        parity = {"max_abs_diff_over_max_abs": float(np.abs(Z64 - Zr).max() / np.abs(Zr).max()),
                  "min_row_cosine": float(cos.min()), "mean_row_cosine": float(cos.mean()),
                  "kmeans_iterations_gpu": info["kmeans_iterations"],
                  "kmeans_iterations_reference": int(r["kmeans_iterations"])}
    out = {"metric": "harmonize: s per run (1M cells x 50 PCs, 4 batches)",
           "value": sec, "unit": "s/harmonize", "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "higher_is_better": False, "dtype": "f32",
           "data": "synthetic",
           "config": {"workload": f"harmony_1m: {n:,} cells x {d} PCs (Gaussian mixture, "
                                  f"PCA-like spectrum, {B} batch offsets), {nc} clusters, "
                                  "the reference's defaults",
                      "l2": "R (400 MB) and the PCs (200 MB) larger than L2 (no flush)"},
           "harmony_only_seconds": min(h_times), "iterations": it,
           "kmeans_iterations": info["kmeans_iterations"],
           "e2e": {"value": e2e, "unit": "s/harmonize",
                   "h2d_bytes_per_step": int(X.nbytes + lab.nbytes),
                   "d2h_bytes_per_step": int(X.nbytes)},
           "roofline": {"bound": "fp32-simt", "achieved": flops / sec / 1e12,
                        "peak": fp32_peak, "unit": "TFLOP/s",
                        "frac": flops / sec / 1e12 / fp32_peak,
                        "peak_source": "nominal (152 SMs x 128 FP32 lanes x 2.07 GHz)",
                        "traffic": None, "flops_per_step": flops,
                        "note": "the block-sequential cluster updates (one launch per "
                                "block, 20 per pass) bound the time, not the FLOPs"},
           "cpu_baseline": cpu, "agreement_with_reference": parity,
           "host_and_device_paths_identical": same_paths,
           "clocks": clk.summary(), "gpu_launches": launches * args.steps}
    print(json.dumps(out))
    return 0


def run_h5ad(args):
    """The 1M x 2000 NB counts written as an .h5ad file (AnnData's CSR group:
    float32 data, int32 indices, int64 indptr, superblock 0 as h5py writes by
    default; h5file.py) and read into device memory. A step is one
    h5ad.read_X: metadata parse, then the copy (the file range registered
    with the driver and copied by the copy engines, or host threads preading
    4 MB pieces into pinned buffers; both are timed apart too). The reference's path to the
    same device arrays is its own reader (brisc/hdf5.pyx:163
    read_all_datasets, every host core, into NumPy arrays) followed by a copy
    of those arrays to the device; its host-only time is reported too. The
    file is in the page cache for both (written, then read once, before
    timing). Also: the time to a solver-ready DeviceMatrix from the file
    (read, size factors, layout)."""
    import tempfile

    import torch

    import h5file
    from brisc_gb300 import h5ad
    from oracle import ref
    from synth import cached_nb_counts
    torch.cuda.init()
    dev = torch.device("cuda", 0)
    n, g, dens, _, _ = WORKLOADS[args.workload]
    if args.cells:
        n = args.cells
    C = cached_nb_counts(n, g, seed=0, density=dens)
    data = C.data.astype(np.float32)
    indices = C.indices.astype(np.int32)
    indptr = C.indptr.astype(np.int64)
    nbytes = data.nbytes + indices.nbytes + indptr.nbytes
    tmpdir = tempfile.mkdtemp(prefix="brisc_h5ad_")
    path = os.path.join(tmpdir, "counts_1m.h5ad")
    h5file.write_h5ad(path, data, indices, indptr, (n, g))
    del data
    cores = os.cpu_count() or 1
    try:
        for _ in range(max(args.warmup, 3)):
            X = h5ad.read_X(path)
        torch.cuda.synchronize()
        times = []
        with Clocks(0) as clk:
            for _ in range(args.steps):
                del X
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                X = h5ad.read_X(path)
                torch.cuda.synchronize()
                times.append(time.perf_counter() - t0)
        sec = float(np.median(times))
        # each method on its own
        per_method = {}
        for meth in ("staged", "mapped"):
            del X
            try:
                X = h5ad.read_X(path, method=meth)
                torch.cuda.synchronize()
                ts = []
                for _ in range(3):
                    del X
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    X = h5ad.read_X(path, method=meth)
                    torch.cuda.synchronize()
                    ts.append(time.perf_counter() - t0)
                per_method[meth] = float(np.median(ts))
            except Exception as e:  # noqa: BLE001 - a refused mapping is reported
                per_method[meth] = f"unavailable: {e}"
                X = h5ad.read_X(path)
        same = bool(np.array_equal(X["indptr"].cpu().numpy(), indptr) and
                    np.array_equal(X["indices"].cpu().numpy(), indices) and
                    np.array_equal(X["data"].cpu().numpy(), C.data.astype(np.float32)))
        del X
        # to a solver-ready matrix
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        M = h5ad.device_matrix(path, method="logCP10k")
        torch.cuda.synchronize()
        t_matrix = time.perf_counter() - t0
        M.close()
        # the host-to-device link: a pinned 1 GB copy, best of 5
        hb = torch.empty(1 << 30, dtype=torch.uint8).pin_memory()
        db = torch.empty(1 << 30, dtype=torch.uint8, device=dev)
        link = []
        for _ in range(5):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            db.copy_(hb, non_blocking=True)
            torch.cuda.synchronize()
            link.append((1 << 30) / (time.perf_counter() - t0) / 1e9)
        link_gbs = max(link)
        del hb, db
        cpu = None
        if not args.no_cpu_baseline and ref.load() is not None and "hdf5" in ref.load():
            info = h5ad.inspect(path)
            dsets = [(info[k]["file_offset"], info[k]["dtype"], info[k]["num_elements"])
                     for k in ("data", "indices", "indptr")]
            ref.run_read_all_datasets(path, dsets, cores)  # warm
            t_host, t_dev = [], []
            for _ in range(3):
                t0 = time.perf_counter()
                arrs = ref.run_read_all_datasets(path, dsets, cores)
                t1 = time.perf_counter()
                on_dev = [torch.from_numpy(a).to(dev) for a in arrs]
                torch.cuda.synchronize()
                t2 = time.perf_counter()
                t_host.append(t1 - t0)
                t_dev.append(t2 - t0)
                del arrs, on_dev
            cpu = {"value": float(np.median(t_dev)), "unit": "s/read", "cores": cores,
                   "kind": "reference",
                   "sample": "the reference's read_all_datasets (brisc/hdf5.pyx, every host "
                             "core) of the whole file's X into NumPy arrays, then a copy of "
                             "them to the device (torch .to(cuda))",
                   "host_only_seconds": float(np.median(t_host))}
    finally:
        try:
            os.remove(path)
            os.rmdir(tmpdir)
        except OSError:
            pass
    out = {"metric": "h5ad X to device: s per read (1M x 2000 counts, 829 MB)",
           "value": sec, "unit": "s/read", "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "higher_is_better": False, "dtype": "bytes",
           "data": "synthetic",
           "config": {"workload": f"h5ad_1m: {n:,} x {g:,} NB counts ({C.nnz:,} entries) as "
                                  "an .h5ad CSR group (float32 data, int32 indices, int64 "
                                  "indptr), superblock 0, contiguous datasets",
                      "page_cache": "warm (the file was written and read before timing)",
                      "threads": cores, "bytes": int(nbytes)},
           "achieved_gbs": nbytes / sec / 1e9, "to_device_matrix_seconds": t_matrix,
           "seconds_by_method": per_method,
           "bit_identical": same,
           "e2e": {"value": sec, "unit": "s/read", "h2d_bytes_per_step": int(nbytes),
                   "d2h_bytes_per_step": 0},
           "roofline": {"bound": "host-to-device link", "achieved": nbytes / sec / 1e9,
                        "peak": link_gbs, "unit": "GB/s", "frac": nbytes / sec / 1e9 / link_gbs,
                        "peak_source": "measured here: a pinned 1 GB torch copy, best of 5",
                        "traffic": None},
           "cpu_baseline": cpu, "clocks": clk.summary(), "gpu_launches": 0,
           "gpu_launches_note": "a read is host threads and cudaMemcpyAsync copies, no "
                                "kernels; device_matrix then runs the size-factor and "
                                "layout kernels"}
    print(json.dumps(out))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "hvg_1m":
        return run_hvg(args)
    if args.workload == "knn_1m":
        return run_knn(args)
    if args.workload == "harmony_1m":
        return run_harmony(args)
    if args.workload == "h5ad_1m":
        return run_h5ad(args)
    if args.workload == "batched_3m":
        return run_batched(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
