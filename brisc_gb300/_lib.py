"""ctypes binding of ``libbriscgpu.so`` (the C ABI declared in include/briscgpu.h).

The library is loaded from the package directory. There is no CPU fallback:
if the library is missing, every entry point raises ``RuntimeError`` telling
the caller to build it (``python -m brisc_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libbriscgpu.so"

# status codes (include/briscgpu.h)
(OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_UNSUPPORTED, ERR_CANCELLED, ERR_DEVICE,
 ERR_IO) = range(8)
INDEX_I32, INDEX_I64 = 0, 1
VALUE_U16, VALUE_U32, VALUE_I32, VALUE_F32 = 0, 1, 2, 3
VALUE_I64, VALUE_U64, VALUE_F64 = 4, 5, 6  # the HVG statistics only
NORM_NONE, NORM_LOGCP10K, NORM_LOG1PPF, NORM_PFLOG1PPF = -1, 0, 1, 2
# forced product kernels (bgpu_matrix_desc.kernels)
KERNELS = {"panels": 1, "natural": 2, "words32": 4, "xv_rows": 8, "xv_seg": 16,
           "vector": 32}


class MatrixDesc(C.Structure):
    _fields_ = [
        ("indptr", C.c_void_p),
        ("indices", C.c_void_p),
        ("values", C.c_void_p),
        ("index_type", C.c_int),
        ("value_type", C.c_int),
        ("on_device", C.c_int),
        ("num_cells", C.c_uint64),
        ("num_genes", C.c_uint32),
        ("nnz", C.c_uint64),
        ("norm_method", C.c_int),
        ("inv_size_factors", C.c_void_p),
        ("post_factors", C.c_void_p),
        ("panel_rows", C.c_uint32),
        ("kernels", C.c_uint32),
        ("sell_panel_rows", C.c_uint32),
    ]


class SolveOpts(C.Structure):
    _fields_ = [
        ("k", C.c_uint32),
        ("subspace_size", C.c_uint32),
        ("tolerance", C.c_float),
        ("max_iterations", C.c_uint32),
        ("seed", C.c_uint64),
        ("chunk_size", C.c_uint64),
        ("reorth_passes", C.c_uint32),
        ("rotation_mode", C.c_uint32),
        ("cancel", C.c_void_p),
        ("use_graphs", C.c_int),
        ("profile", C.c_int),
        ("svd_mode", C.c_uint32),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("converged", C.c_int32),
        ("restarts", C.c_uint32),
        ("lanczos_steps", C.c_uint32),
        ("rmatvecs", C.c_uint32),
        ("num_converged", C.c_uint32),
        ("k_current", C.c_uint32),
        ("seconds", C.c_double),
        ("matvec_seconds", C.c_double),
        ("rmatvec_seconds", C.c_double),
        ("svd_seconds", C.c_double),
        ("reorth_seconds", C.c_double),
        ("vstep_seconds", C.c_double),
        ("rotation_seconds", C.c_double),
        ("matvec_bytes", C.c_double),
        ("rmatvec_bytes", C.c_double),
        ("reorth_bytes", C.c_double),
        ("rotation_bytes", C.c_double),
        ("kernel_launches", C.c_uint64),
        ("second_passes", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class HvgInput(C.Structure):
    _fields_ = [
        ("data", C.c_void_p),
        ("value_type", C.c_int),
        ("indices", C.c_void_p),
        ("indptr", C.c_void_p),
        ("index_type", C.c_int),
        ("nnz", C.c_uint64),
        ("num_major", C.c_uint64),
        ("is_csr", C.c_int),
        ("num_genes", C.c_uint32),
        ("cell_indices", C.c_void_p),
        ("num_cell_indices", C.c_uint64),
        ("cell_mask", C.c_void_p),
        ("cell_mask_len", C.c_uint64),
        ("on_device", C.c_int),
    ]


H5_I32, H5_I64, H5_U32, H5_U64 = 0, 1, 2, 3  # index arrays in an .h5ad file
H5_READ = {"auto": 0, "staged": 1, "mapped": 2}


class H5Dataset(C.Structure):
    _fields_ = [
        ("file_offset", C.c_uint64),
        ("num_bytes", C.c_uint64),
        ("num_elements", C.c_uint64),
        ("element_size", C.c_uint32),
        ("type", C.c_int),
    ]


class H5adMatrix(C.Structure):
    _fields_ = [
        ("X_key", C.c_char * 64),
        ("is_csr", C.c_int),
        ("num_rows", C.c_uint64),
        ("num_columns", C.c_uint64),
        ("nnz", C.c_uint64),
        ("data", H5Dataset),
        ("indices", H5Dataset),
        ("indptr", H5Dataset),
    ]


# name -> (restype, argtypes); every symbol include/briscgpu.h declares
_vp, _u32, _u64, _i, _f = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
SIGNATURES = {
    "bgpu_last_error": (C.c_char_p, []),
    "bgpu_version": (C.c_char_p, []),
    "bgpu_matrix_create": (_i, [C.POINTER(_vp), C.POINTER(MatrixDesc), _vp]),
    "bgpu_matrix_create_rows": (_i, [C.POINTER(_vp), C.POINTER(MatrixDesc), _vp, _u64, _vp]),
    "bgpu_matrix_destroy": (_i, [_vp]),
    "bgpu_matrix_bytes": (_i, [_vp, C.POINTER(_u64)]),
    "bgpu_matrix_layout": (_i, [_vp, C.POINTER(C.c_int)]),
    "bgpu_matrix_matvec": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "bgpu_matrix_rmatvec": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "bgpu_matrix_gene_stddev": (_i, [_vp, _vp, _vp]),
    "bgpu_solve_opts_default": (None, [C.POINTER(SolveOpts)]),
    "bgpu_irlba": (_i, [_vp, C.POINTER(SolveOpts), _vp, _i, _vp, _vp,
                        C.POINTER(SolveInfo), _vp]),
    "bgpu_irlba_batch": (_i, [_vp, C.POINTER(SolveOpts), _u32, _vp, _i, _vp,
                              C.POINTER(SolveInfo), C.POINTER(_u64), _vp]),
    "bgpu_irlba_f32": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i, _u64, _u32, _u32,
                            _u32, _f, _u32, _u64, _i, _i, _u32, _u64, _vp,
                            C.POINTER(_i)]),
    "bgpu_start_vector": (_i, [_u64, _u32, _vp]),
    "bgpu_rotate_basis": (_i, [_vp, _u64, _u64, _u32, _vp, _u64, _u32, _vp, _u64, _i, _vp]),
    "bgpu_small_svd": (_i, [_vp, _u32, _vp, _vp, _vp, _vp]),
    "bgpu_small_svd_noalloc": (_i, [_vp, _u32, _vp, _vp, _vp, _vp]),
    "bgpu_size_factors": (_i, [_vp, _i, _vp, _i, _u64, _i, _vp, _vp, _vp, _vp, _vp]),
    "bgpu_normalize_csr": (_i, [_vp, _i, _vp, _i, _u64, _vp, _vp, _vp, _vp]),
    "bgpu_csr_tocsc": (_i, [_u64, _u32, _vp, _vp, _vp, _i, _vp, _vp, _vp, _vp]),
    "bgpu_gene_mean_var": (_i, [C.POINTER(HvgInput), _u64, _vp, _vp, _vp, _vp]),
    "bgpu_clipped_sum": (_i, [C.POINTER(HvgInput), _u64, _vp, _vp, _vp, _vp]),
    "bgpu_knn_self": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _u64, _u32,
                           _u32, _u32, _u32, _vp]),
    "bgpu_kmeans": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _u32, _f, _u32, _u64,
                         _u64, _u32, _u32, C.POINTER(_u32), _vp]),
    "bgpu_normalize_rows": (_i, [_vp, _vp, _u64, _u32, _vp]),
    "bgpu_harmony": (_i, [_vp, _vp, _vp, _vp, _vp, _u32, _u32, _u32, _f, _f, _i, _f, _f,
                          _f, _f, _f, _u32, _u64, _u64, _u32, _u32, C.POINTER(_u32), _vp]),
    "bgpu_h5ad_inspect": (_i, [C.c_char_p, C.c_char_p, C.POINTER(H5adMatrix)]),
    "bgpu_h5ad_read": (_i, [C.c_char_p, C.POINTER(H5adMatrix), _vp, _vp, _vp, _u32, _u32,
                            _vp]),
}

_lock = threading.Lock()
_lib = None


class BriscGPUError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn} failed (status {code}): {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the library once; raise if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: the GPU path has no CPU fallback; "
                    "build it with `python -m brisc_gb300.build`")
            L = C.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(code: int, fn: str) -> None:
    if code != OK:
        msg = lib().bgpu_last_error().decode(errors="replace")
        if code == ERR_INVALID:
            raise ValueError(f"{fn}: {msg}")
        if code == ERR_IO:
            raise OSError(f"{fn}: {msg}")
        raise BriscGPUError(code, fn, msg)


def call(fn: str, *args) -> None:
    check(getattr(lib(), fn)(*args), fn)
