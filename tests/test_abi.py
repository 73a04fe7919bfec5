"""The C-ABI library loads and exports every symbol include/briscgpu.h declares.

CPU only: no call here launches a kernel. Host-only entry points (the start
vector) and argument validation are exercised directly.
"""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "briscgpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_path():
    names = declared_functions()
    for must in ["bgpu_irlba", "bgpu_irlba_f32", "bgpu_matrix_create",
                 "bgpu_matrix_matvec", "bgpu_matrix_rmatvec", "bgpu_small_svd",
                 "bgpu_csr_tocsc", "bgpu_normalize_csr", "bgpu_size_factors",
                 "bgpu_start_vector", "bgpu_matrix_gene_stddev"]:
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header(built_lib):
    from brisc_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_version_and_error_string(built_lib):
    from brisc_gb300 import _lib
    L = _lib.lib()
    assert b"sm_103a" in L.bgpu_version()
    assert isinstance(L.bgpu_last_error(), bytes)


def test_host_start_vector_matches_reference(built_lib, golden):
    """bgpu_start_vector is host code: bit-exact normals, norm within ulps."""
    from brisc_gb300 import _lib
    z = golden("rng")
    out = np.empty(2000, dtype=np.float32)
    i = 0
    while f"seed_{i}" in z.files:
        _lib.call("bgpu_start_vector", int(z[f"seed_{i}"]), 2000, out.ctypes.data)
        d = np.abs(out.view(np.int32).astype(np.int64) -
                   z[f"start_{i}"].view(np.int32).astype(np.int64))
        assert d.max() <= 8
        i += 1


def test_invalid_arguments_rejected_without_gpu(built_lib):
    from brisc_gb300 import _lib
    L = _lib.lib()
    h = C.c_void_p()
    assert L.bgpu_matrix_create(C.byref(h), None, None) == _lib.ERR_INVALID
    assert b"desc" in L.bgpu_last_error()
    o = _lib.SolveOpts()
    L.bgpu_solve_opts_default(C.byref(o))
    assert (o.k, o.subspace_size, o.max_iterations) == (50, 100, 100)
    assert abs(o.tolerance - 1e-6) < 1e-12 and o.reorth_passes == 0
    assert L.bgpu_irlba(None, C.byref(o), None, 0, None, None, None, None) == _lib.ERR_INVALID
    assert L.bgpu_irlba_batch(None, C.byref(o), 1, None, 0, None, None, None,
                              None) == _lib.ERR_INVALID
    d = _lib.MatrixDesc()
    d.num_cells, d.num_genes = 10, 70000
    d.indptr = 1
    assert L.bgpu_matrix_create(C.byref(h), C.byref(d), None) == _lib.ERR_UNSUPPORTED
    d.num_genes = 10
    d.index_type = 7
    assert L.bgpu_matrix_create(C.byref(h), C.byref(d), None) == _lib.ERR_INVALID
    # sliced-ELL panel rows: a multiple of 32 in [128, 512], checked before
    # the arrays are touched
    d.index_type = _lib.INDEX_I32
    d.indices = d.values = 1
    d.norm_method = _lib.NORM_NONE
    d.value_type = _lib.VALUE_F32
    d.nnz = 4
    d.sell_panel_rows = 100
    assert L.bgpu_matrix_create(C.byref(h), C.byref(d), None) == _lib.ERR_INVALID
    assert b"sell_panel_rows" in L.bgpu_last_error()
    with pytest.raises(ValueError):
        _lib.call("bgpu_start_vector", 0, 0, None)


def test_hvg_arguments_rejected_without_gpu(built_lib):
    """bgpu_gene_mean_var validates its input description before any CUDA
    call: unknown element types and a subset of the wrong kind."""
    import numpy as np
    from brisc_gb300 import _lib
    L = _lib.lib()
    ip = np.array([0, 1], np.int32)
    ix = np.array([0], np.int32)
    d = np.array([1], np.uint32)
    out = np.zeros(1, np.float32)
    nz = np.zeros(1, np.uint32)

    def run(**kw):
        h = _lib.HvgInput()
        h.data, h.value_type = d.ctypes.data, _lib.VALUE_U32
        h.indices, h.indptr, h.index_type = ix.ctypes.data, ip.ctypes.data, _lib.INDEX_I32
        h.nnz, h.num_major, h.is_csr, h.num_genes = 1, 1, 1, 1
        for k, v in kw.items():
            setattr(h, k, v)
        return L.bgpu_gene_mean_var(C.byref(h), 1, out.ctypes.data, out.ctypes.data,
                                    nz.ctypes.data, None)

    assert run(value_type=99) == _lib.ERR_INVALID
    assert b"value_type" in L.bgpu_last_error()
    assert run(index_type=7) == _lib.ERR_INVALID
    assert b"index_type" in L.bgpu_last_error()
    mask = np.ones(1, np.int8)
    assert run(cell_mask=mask.ctypes.data, cell_mask_len=1) == _lib.ERR_INVALID
    assert b"cell_mask" in L.bgpu_last_error()
    assert run(is_csr=0, num_genes=5) == _lib.ERR_INVALID
    assert b"fewer genes" in L.bgpu_last_error()
    assert L.bgpu_gene_mean_var(None, 1, None, None, None, None) == _lib.ERR_INVALID


def test_knn_self_argument_checks_before_any_device_work():
    """The knn_self drop-in rejects wrong dtypes, shapes and chunk sizes with
    the reference caller's errors before touching the GPU."""
    import pytest as _pt
    from brisc_gb300 import knn
    n, d, k, cs, nc = 10, 3, 2, 2, 2
    good = dict(X=np.zeros((n, d), np.float32), sorted_order=np.arange(n, dtype=np.uint32),
                centroids=np.zeros((nc, d), np.float32),
                num_cells_per_cluster=np.array([5, 5], np.uint32),
                neighbors=np.zeros((n, k), np.uint32), distances=np.zeros((n, k), np.float32),
                cell_norms=np.zeros(n, np.float32),
                centroid_distances=np.zeros((n, cs), np.float32),
                nearest_clusters=np.zeros((n, cs), np.uint32), num_neighbors=k,
                num_clusters_searched=cs)
    bad = dict(good, X=np.zeros((n, d), np.float64))
    with _pt.raises(TypeError):
        knn.knn_self(**bad)
    bad = dict(good, neighbors=np.zeros((n, k + 1), np.uint32))
    with _pt.raises(ValueError):
        knn.knn_self(**bad)
    with _pt.raises(ValueError, match="chunk_size_search"):
        knn.knn_self(**good, chunk_size_search=0)


def test_harmony_argument_checks_before_any_device_work(built_lib):
    """bgpu_harmony rejects NULL pointers and sizes beyond its limits before
    it touches memory (the pointers below are never dereferenced)."""
    from brisc_gb300 import _lib
    L = _lib.lib()
    it = C.c_uint32(0)
    p = C.c_void_p(256)

    def run(B=3, d=20, nc=50, chunk=256, n=1000, bp=0.05, sigma=0.1, null=False):
        ptrs = [None] * 5 if null else [p] * 5
        return L.bgpu_harmony(*ptrs, B, 10, 5, bp, 0.01, 0, 1e-3, 2.0, 0.0, 0.2, sigma,
                              chunk, 0, n, d, nc, C.byref(it), None)
    assert run(null=True) == _lib.ERR_INVALID
    assert run(B=65) == _lib.ERR_UNSUPPORTED
    assert run(d=129) == _lib.ERR_UNSUPPORTED
    assert run(nc=257) == _lib.ERR_UNSUPPORTED
    assert run(chunk=2000) == _lib.ERR_UNSUPPORTED
    assert run(bp=0.0) == _lib.ERR_INVALID
    assert run(sigma=0.0) == _lib.ERR_INVALID
    assert b"sigma" in L.bgpu_last_error()
    assert L.bgpu_normalize_rows(None, None, 5, 3, None) == _lib.ERR_INVALID
