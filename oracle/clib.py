"""ORACLE (test infrastructure): builds and loads oracle/oracle.c.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use this,
as the checker. ``build()`` compiles ``oracle/_build/liboracle.so`` with the
host C compiler (no fast-math: the float arithmetic must round as written).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
OUT = HERE / "_build" / "liboracle.so"
_lib = None


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cc = os.environ.get("CC") or shutil.which("cc") or shutil.which("gcc")
    subprocess.run([cc, "-O2", "-fPIC", "-shared", "-fno-fast-math",
                    "-ffp-contract=off", str(SRC), "-o", str(OUT), "-lm"],
                   check=True)
    return OUT


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(OUT))
        vp, u32, u64, i, f = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
        sig = {
            "oracle_raw_rand": (None, [u64, u32, vp]),
            "oracle_raw_normals": (None, [u64, u32, vp]),
            "oracle_start_vector": (None, [u64, u32, vp]),
            "oracle_csr_tocsc": (None, [u64, u32, vp, vp, vp, vp, vp, vp]),
            "oracle_normalize_csr": (None, [vp, vp, u64, vp, i, vp, vp, vp, vp]),
            "oracle_clipped_stddev_csc": (None, [vp, vp, u64, u32, f, vp]),
            "oracle_thread_offsets": (None, [vp, u64, u32, vp]),
            "oracle_fisher_yates": (None, [u64, u32, vp]),
            "oracle_kmeans_init": (None, [u64, u32, u32, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def raw_rand(seed: int, count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.uint32)
    lib().oracle_raw_rand(seed, count, _p(out))
    return out


def raw_normals(seed: int, count: int) -> np.ndarray:
    out = np.empty(count, dtype=np.float32)
    lib().oracle_raw_normals(seed, count, _p(out))
    return out


def start_vector(seed: int, g: int) -> np.ndarray:
    out = np.empty(g, dtype=np.float32)
    lib().oracle_start_vector(seed, g, _p(out))
    return out


def csr_tocsc(indptr, indices, data, n_col: int):
    """Stable transpose; data must be a 4-byte dtype (copied bit for bit)."""
    ap = np.ascontiguousarray(indptr, dtype=np.int64)
    aj = np.ascontiguousarray(indices, dtype=np.int64)
    ax = np.ascontiguousarray(data).view(np.uint32)
    n_row = ap.shape[0] - 1
    bp = np.empty(n_col + 1, dtype=np.int64)
    bi = np.empty(ax.shape[0], dtype=np.int64)
    bx = np.empty(ax.shape[0], dtype=np.uint32)
    lib().oracle_csr_tocsc(n_row, n_col, _p(ap), _p(aj), _p(ax), _p(bp),
                           _p(bi), _p(bx))
    return bp, bi, bx.view(np.asarray(data).dtype)


def normalize_csr(indptr, data, method: int = 0, qc=None):
    """Returns (normalized float32, row_sums uint64, isf float32, post or None)."""
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    d = np.ascontiguousarray(data, dtype=np.float64)
    n = ip.shape[0] - 1
    out = np.empty(d.shape[0], dtype=np.float32)
    rs = np.empty(n, dtype=np.uint64)
    isf = np.empty(n, dtype=np.float32)
    post = np.empty(n, dtype=np.float32) if method == 2 else None
    q = None if qc is None else np.ascontiguousarray(qc, dtype=np.uint8)
    lib().oracle_normalize_csr(_p(d), _p(ip), n, _p(q), method, _p(out),
                               _p(rs), _p(isf), _p(post))
    return out, rs, isf, post


def clipped_stddev_csc(data, indptr, n_cells: int, clip: float = 1e-8):
    d = np.ascontiguousarray(data, dtype=np.float32)
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    g = ip.shape[0] - 1
    out = np.empty(g, dtype=np.float32)
    lib().oracle_clipped_stddev_csc(_p(d), _p(ip), n_cells, g, clip, _p(out))
    return out


def thread_offsets(indptr, num_threads: int) -> np.ndarray:
    ip = np.ascontiguousarray(indptr, dtype=np.int64)
    out = np.empty(num_threads + 1, dtype=np.uint32)
    lib().oracle_thread_offsets(_p(ip), ip.shape[0] - 1, num_threads, _p(out))
    return out


def fisher_yates(n: int, seed: int) -> np.ndarray:
    """brisc/harmonize.pyx:503-509's random cell order."""
    out = np.zeros(n, dtype=np.uint32)
    lib().oracle_fisher_yates(seed & 0xFFFFFFFFFFFFFFFF, n, _p(out))
    return out.astype(np.int64)


def kmeans_init(n: int, num_clusters: int, seed: int) -> np.ndarray:
    """brisc/kmeans.pyx:13-38's random initial cells."""
    out = np.zeros(num_clusters, dtype=np.uint32)
    lib().oracle_kmeans_init(seed & 0xFFFFFFFFFFFFFFFF, n, num_clusters, _p(out))
    return out.astype(np.int64)
