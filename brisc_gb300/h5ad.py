"""The count matrix of an .h5ad file, read straight into device memory.

SingleCell's reader (brisc/single_cell.py:83-1400) asks h5py where each
dataset of X starts in the file (single_cell.py:1848-1883) and preads the
contiguous bytes into host arrays with OpenMP threads (brisc/hdf5.pyx:163,
``read_all_datasets``). Here the library parses the file's HDF5 metadata
itself (no HDF5 library needed) and streams X's ``data``, ``indices`` and
``indptr`` from the file through pinned staging buffers into CUDA tensors:
the 10M-cell matrix never exists as host arrays. X is chosen as the
reference chooses it, with its messages: ``X_key``, else ``layers/UMIs``,
else ``raw/X``, else ``X``; ``encoding-type`` (or ``h5sparse_format``) must
be csr_matrix or csc_matrix. Only contiguous, uncompressed datasets are
streamed (the reference sends chunked or compressed files to a slower
reader; here they raise NotImplementedError).

``device_matrix`` goes one step further, to the PCA's input: size factors on
the GPU and the solver's layout, for ``DeviceMatrix.solve`` with the
normalisation fused into the products.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _lib as L

_VALUE_DTYPES = {L.VALUE_U16: "uint16", L.VALUE_U32: "uint32", L.VALUE_I32: "int32",
                 L.VALUE_F32: "float32", L.VALUE_I64: "int64", L.VALUE_U64: "uint64",
                 L.VALUE_F64: "float64"}
_INDEX_DTYPES = {L.H5_I32: "int32", L.H5_I64: "int64", L.H5_U32: "uint32",
                 L.H5_U64: "uint64"}


def _info(path, X_key) -> L.H5adMatrix:
    m = L.H5adMatrix()
    code = L.lib().bgpu_h5ad_inspect(os.fsencode(path),
                                     None if X_key is None else X_key.encode(), C.byref(m))
    if code == L.ERR_UNSUPPORTED:
        raise NotImplementedError(L.lib().bgpu_last_error().decode(errors="replace"))
    L.check(code, "bgpu_h5ad_inspect")
    return m


def inspect(path, X_key: str | None = None) -> dict:
    """What the file's sparse X is: the group chosen, csr or csc, shape,
    stored entries, element types and the three datasets' byte ranges."""
    m = _info(path, X_key)

    def ds(d, types):
        return {"file_offset": int(d.file_offset), "num_bytes": int(d.num_bytes),
                "num_elements": int(d.num_elements), "dtype": types[d.type]}
    return {"X_key": m.X_key.decode(), "format": "csr" if m.is_csr else "csc",
            "shape": (int(m.num_rows), int(m.num_columns)), "nnz": int(m.nnz),
            "data": ds(m.data, _VALUE_DTYPES), "indices": ds(m.indices, _INDEX_DTYPES),
            "indptr": ds(m.indptr, _INDEX_DTYPES)}


def _torch_dtype(name: str):
    import torch
    return getattr(torch, name)


def read_X(path, X_key: str | None = None, num_threads: int = 0, device=None,
           stream=None, method: str = "auto") -> dict:
    """X's three arrays as CUDA tensors (element types as stored; unsigned
    index arrays come back as the signed type of the same width, holding the
    same bits), plus ``shape``, ``format`` ('csr' or 'csc') and ``X_key``.
    ``method``: 'mapped' (the file range registered with the driver, copied
    by the copy engines straight from the page cache), 'staged' (``num_threads``
    host threads, 0 = all, pread into pinned buffers) or 'auto' (mapped
    where the driver allows it)."""
    import torch
    m = _info(path, X_key)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None \
        else torch.device(device)
    out = {}
    signed = {"uint32": "int32", "uint64": "int64"}
    for name, types in (("data", _VALUE_DTYPES), ("indices", _INDEX_DTYPES),
                        ("indptr", _INDEX_DTYPES)):
        d = getattr(m, name)
        dt = types[d.type]
        if name != "data":
            dt = signed.get(dt, dt)
        out[name] = torch.empty(int(d.num_elements), dtype=_torch_dtype(dt), device=dev)
    s = torch.cuda.current_stream(dev) if stream is None else stream
    with torch.cuda.device(dev):
        L.call("bgpu_h5ad_read", os.fsencode(path), C.byref(m),
               out["data"].data_ptr() if out["data"].numel() else None,
               out["indices"].data_ptr() if out["indices"].numel() else None,
               out["indptr"].data_ptr(), L.H5_READ[method], int(num_threads),
               C.c_void_p(s.cuda_stream))
    out.update(shape=(int(m.num_rows), int(m.num_columns)),
               format="csr" if m.is_csr else "csc", X_key=m.X_key.decode())
    return out


def device_matrix(path, method: str | None = "logCP10k", X_key: str | None = None,
                  num_threads: int = 0, kernels=()):
    """The file's count matrix as a :class:`~brisc_gb300.pca.DeviceMatrix`
    (cells x genes), without host arrays: X read to the device, transposed
    there if stored csc, per-cell size factors for ``method`` computed on the
    GPU over all genes (brisc/normalize.pyx:36-81), the normalisation fused
    into the products. ``method=None`` takes the stored values as already
    normalised float32."""
    import torch

    from .pca import _METHODS, DeviceMatrix
    X = read_X(path, X_key, num_threads)
    n, g = X["shape"]
    data, indices, indptr = X["data"], X["indices"], X["indptr"]
    if data.dtype == torch.uint64 or data.dtype == torch.float64 or data.dtype == torch.int64:
        data = data.to(torch.float32)  # the solver's value types
    nnz = data.numel()
    itype = torch.int64 if nnz >= 2 ** 31 or max(n, g) >= 2 ** 31 else torch.int32
    indptr, indices = indptr.to(itype), indices.to(itype)
    stream = torch.cuda.current_stream()
    if X["format"] == "csc":  # genes x cells CSR -> its CSC, i.e. cells x genes CSR
        if data.element_size() != 4:
            data = data.to(torch.float32)
        Bp = torch.empty(n + 1, dtype=itype, device=data.device)
        Bi = torch.empty(nnz, dtype=itype, device=data.device)
        Bx = torch.empty_like(data)
        L.call("bgpu_csr_tocsc", g, n, indptr.data_ptr(), indices.data_ptr(),
               data.data_ptr(), L.INDEX_I64 if itype == torch.int64 else L.INDEX_I32,
               Bp.data_ptr(), Bi.data_ptr(), Bx.data_ptr(), C.c_void_p(stream.cuda_stream))
        indptr, indices, data = Bp, Bi, Bx
    isf = post = None
    if method is not None:
        if method not in _METHODS:
            raise ValueError("method must be one of 'PFlog1pPF', 'log1pPF', or 'logCP10k'")
        vt = {torch.uint16: L.VALUE_U16, torch.uint32: L.VALUE_U32,
              torch.int32: L.VALUE_I32, torch.float32: L.VALUE_F32}.get(data.dtype)
        if vt is None:
            data, vt = data.to(torch.float32), L.VALUE_F32
        isf = torch.empty(n, dtype=torch.float32, device=data.device)
        post = torch.empty(n, dtype=torch.float32, device=data.device) \
            if method == "PFlog1pPF" else None
        L.call("bgpu_size_factors", indptr.data_ptr(),
               L.INDEX_I64 if itype == torch.int64 else L.INDEX_I32, data.data_ptr(), vt,
               n, _METHODS[method], None, isf.data_ptr(),
               post.data_ptr() if post is not None else None, None,
               C.c_void_p(stream.cuda_stream))
    elif data.dtype != torch.float32:
        raise TypeError("method=None needs X stored as normalised float32 values")
    return DeviceMatrix(indptr, indices, data, n, g, norm=method, inv_size_factors=isf,
                        post_factors=post, kernels=kernels)
