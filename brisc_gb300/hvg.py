"""Highly-variable-gene statistics on the GPU, as brisc/hvg.pyx computes them.

The four functions keep the reference's names, argument order and meaning,
and fill their output arrays in place:

- ``gene_mean_and_variance_csr`` (brisc/hvg.pyx:9-139)
- ``gene_mean_and_variance_csc`` (brisc/hvg.pyx:142-252)
- ``clipped_sum_csr`` (brisc/hvg.pyx:255-403)
- ``clipped_sum_csc`` (brisc/hvg.pyx:406-530)

The counts are summed as 64-bit integers on the device, and the float outputs
follow the reference's expressions rounding for rounding, so every output is
bit-identical to the reference's. ``num_threads`` is accepted for signature
parity and unused.

Arrays are NumPy arrays on the host, or CUDA tensors for a matrix already on
the device. In the second case every array, outputs included, must be a CUDA
tensor. The dtypes are the reference's:
- data: int32, uint32, int64, uint64, float32 or float64, plus uint16;
- indices and indptr: int32 or int64, the same type for both;
- cell_indices: int64; cell_mask: one byte per cell;
- outputs: float32, and uint32 for the nonzero counts (int32 tensors are
  accepted for them on the device).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

_VALUE = {np.dtype(np.uint16): L.VALUE_U16, np.dtype(np.uint32): L.VALUE_U32,
          np.dtype(np.int32): L.VALUE_I32, np.dtype(np.float32): L.VALUE_F32,
          np.dtype(np.int64): L.VALUE_I64, np.dtype(np.uint64): L.VALUE_U64,
          np.dtype(np.float64): L.VALUE_F64}
_INDEX = {np.dtype(np.int32): L.INDEX_I32, np.dtype(np.int64): L.INDEX_I64}


def _is_cuda(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _dtype(a) -> np.dtype:
    if isinstance(a, np.ndarray):
        return a.dtype
    return np.dtype(str(a.dtype).replace("torch.", ""))


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("ndarray is not C-contiguous")
        return a.ctypes.data
    if not a.is_contiguous():
        raise ValueError("tensor is not contiguous")
    return a.data_ptr()


def _len(a) -> int:
    return int(a.shape[0])


def _check(a, name: str, dtypes: tuple, n: int | None = None) -> None:
    if a is None:
        raise TypeError(f"{name} is required")
    if a.ndim != 1:
        raise ValueError(f"{name} must be one-dimensional")
    if _dtype(a) not in tuple(np.dtype(d) for d in dtypes):
        raise TypeError(f"{name} has dtype {_dtype(a)}; expected one of "
                        f"{', '.join(str(np.dtype(d)) for d in dtypes)}")
    if n is not None and _len(a) < n:
        raise ValueError(f"{name} has {_len(a):,} entries; {n:,} are needed")


def _input(data, indices, indptr, is_csr: bool, num_genes: int,
           cell_indices=None, cell_mask=None) -> L.HvgInput:
    arrays = [x for x in (data, indices, indptr, cell_indices, cell_mask)
              if x is not None]
    on_device = _is_cuda(data)
    if any(_is_cuda(x) != on_device for x in arrays):
        raise TypeError("all arrays must be on the host, or all CUDA tensors")
    _check(data, "data", tuple(_VALUE))
    _check(indices, "indices", tuple(_INDEX))
    _check(indptr, "indptr", tuple(_INDEX))
    if _dtype(indices) != _dtype(indptr):
        raise TypeError("indices and indptr must have the same dtype")
    if _len(indices) != _len(data):
        raise ValueError("data and indices must have the same length")
    if _len(indptr) < 1:
        raise ValueError("indptr must have at least one entry")
    h = L.HvgInput()
    h.data, h.value_type = _ptr(data), _VALUE[_dtype(data)]
    h.indices, h.indptr = _ptr(indices), _ptr(indptr)
    h.index_type = _INDEX[_dtype(indptr)]
    h.nnz, h.num_major = _len(data), _len(indptr) - 1
    h.is_csr, h.num_genes = int(is_csr), int(num_genes)
    if cell_indices is not None and _len(cell_indices) > 0:
        _check(cell_indices, "cell_indices", (np.int64,))
        h.cell_indices, h.num_cell_indices = _ptr(cell_indices), _len(cell_indices)
    if cell_mask is not None and _len(cell_mask) > 0:
        _check(cell_mask, "cell_mask", (np.int8, np.uint8, np.bool_))
        h.cell_mask, h.cell_mask_len = _ptr(cell_mask), _len(cell_mask)
    h.on_device = int(on_device)
    return h


def _stream(a):
    if not _is_cuda(a):
        return None
    import torch
    return C.c_void_p(torch.cuda.current_stream(a.device).cuda_stream)


def _mean_var(h: L.HvgInput, num_cells, num_dataset_genes, mean, var,
              nonzero_count, like) -> None:
    # a CUDA tensor of int32 holds the uint32 counts (torch keeps few uint32
    # operations)
    nz_types = (np.uint32, np.int32) if h.on_device else (np.uint32,)
    for a, name, dts in ((mean, "mean", (np.float32,)), (var, "var", (np.float32,)),
                         (nonzero_count, "nonzero_count", nz_types)):
        _check(a, name, dts, int(num_dataset_genes))
        if _is_cuda(a) != bool(h.on_device):
            raise TypeError(f"{name} must live where the inputs live")
    L.call("bgpu_gene_mean_var", C.byref(h), int(num_cells), _ptr(mean), _ptr(var),
           _ptr(nonzero_count), _stream(like))


def _clipped(h: L.HvgInput, num_cells, n_out, clip_val, batch_counts_sum,
             squared_batch_counts_sum, like) -> None:
    for a, name in ((clip_val, "clip_val"), (batch_counts_sum, "batch_counts_sum"),
                    (squared_batch_counts_sum, "squared_batch_counts_sum")):
        _check(a, name, (np.float32,), int(n_out))
        if _is_cuda(a) != bool(h.on_device):
            raise TypeError(f"{name} must live where the inputs live")
    L.call("bgpu_clipped_sum", C.byref(h), int(num_cells), _ptr(clip_val),
           _ptr(batch_counts_sum), _ptr(squared_batch_counts_sum), _stream(like))


def gene_mean_and_variance_csr(data, indices, indptr, cell_indices, num_cells,
                               num_dataset_genes, mean, var, nonzero_count,
                               num_threads=1) -> None:
    """brisc/hvg.pyx:9-139. An empty ``cell_indices`` sums every stored
    entry; otherwise its first ``num_cells`` cells."""
    h = _input(data, indices, indptr, True, num_dataset_genes,
               cell_indices=cell_indices)
    _mean_var(h, num_cells, num_dataset_genes, mean, var, nonzero_count, data)


def gene_mean_and_variance_csc(data, indices, indptr, cell_mask, num_cells,
                               num_dataset_genes, mean, var, nonzero_count,
                               num_threads=1) -> None:
    """brisc/hvg.pyx:142-252. An empty ``cell_mask`` keeps every cell."""
    h = _input(data, indices, indptr, False, num_dataset_genes, cell_mask=cell_mask)
    _mean_var(h, num_cells, num_dataset_genes, mean, var, nonzero_count, data)


def clipped_sum_csr(data, indices, indptr, num_cells, num_dataset_genes,
                    cell_indices, clip_val, batch_counts_sum,
                    squared_batch_counts_sum, num_threads=1) -> None:
    """brisc/hvg.pyx:255-403. An empty ``cell_indices`` sums rows
    [0, num_cells); otherwise every listed cell."""
    h = _input(data, indices, indptr, True, num_dataset_genes,
               cell_indices=cell_indices)
    _clipped(h, num_cells, num_dataset_genes, clip_val, batch_counts_sum,
             squared_batch_counts_sum, data)


def clipped_sum_csc(data, indices, indptr, cell_mask, clip_val, batch_counts_sum,
                    squared_batch_counts_sum, num_threads=1) -> None:
    """brisc/hvg.pyx:406-530, over every gene of ``indptr``."""
    h = _input(data, indices, indptr, False, _len(indptr) - 1, cell_mask=cell_mask)
    _clipped(h, 0, _len(indptr) - 1, clip_val, batch_counts_sum,
             squared_batch_counts_sum, data)


NAMES = ("gene_mean_and_variance_csr", "gene_mean_and_variance_csc",
         "clipped_sum_csr", "clipped_sum_csc")


def install_hvg(module=None) -> dict:
    """Bind the four functions into brisc's ``single_cell`` module, where
    ``import_cython`` puts the reference's (brisc/single_cell.py:34-43) and
    its HVG step calls them (single_cell.py:11330-11391). Returns the
    previous bindings (name -> function), for restoring them."""
    if module is None:
        import brisc.single_cell as module  # pragma: no cover
    previous = {name: getattr(module, name, None) for name in NAMES}
    here = globals()
    for name in NAMES:
        setattr(module, name, here[name])
    return previous
