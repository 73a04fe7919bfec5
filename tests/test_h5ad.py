"""The .h5ad metadata reader (bgpu_h5ad_inspect, brisc_gb300/h5ad.py) on
files written by h5file.py in both of h5py's layouts: superblock 0 with
symbol-table groups and version-1 object headers (h5py's default), and
superblock 2 with version-2 object headers and link messages
(libver='latest'); attributes inline or in continuation blocks.

CPU only: the reader parses metadata on the host. The byte ranges it reports
must hold exactly the arrays written (bit-exact), X must be chosen and
checked as the reference's reader does (brisc/single_cell.py:497-522,
610-657), with its messages.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import h5file

STYLES = [("v0", False), ("v0", True), ("v2", False), ("v2", True)]


def _matrix(n=300, g=50, density=0.1, seed=1, dtype=np.float32):
    X = sp.random(n, g, density=density, format="csr", random_state=seed, dtype=np.float64)
    X.data = np.ceil(X.data * 20).astype(dtype)
    return X


def _check_ranges(path, info, arrays):
    raw = open(path, "rb").read()
    for name, arr in arrays.items():
        d = info[name]
        assert d["dtype"] == np.dtype(arr.dtype).name
        got = np.frombuffer(raw[d["file_offset"]:d["file_offset"] + d["num_bytes"]],
                            dtype=d["dtype"])
        np.testing.assert_array_equal(got, arr)


@pytest.mark.parametrize("style,continuation", STYLES)
@pytest.mark.parametrize("vdt,idt,pdt", [(np.float32, np.int32, np.int64),
                                         (np.uint16, np.int32, np.int32),
                                         (np.int32, np.uint32, np.uint64),
                                         (np.float64, np.int64, np.int64)])
def test_inspect_reports_the_written_arrays(tmp_path, built_lib, style, continuation,
                                            vdt, idt, pdt):
    from brisc_gb300 import h5ad
    X = _matrix(dtype=vdt)
    arrays = {"data": X.data, "indices": X.indices.astype(idt),
              "indptr": X.indptr.astype(pdt)}
    path = str(tmp_path / "x.h5ad")
    h5file.write_h5ad(path, arrays["data"], arrays["indices"], arrays["indptr"], X.shape,
                      style=style, continuation=continuation)
    info = h5ad.inspect(path)
    assert info["X_key"] == "X" and info["format"] == "csr"
    assert info["shape"] == X.shape and info["nnz"] == X.nnz
    _check_ranges(path, info, arrays)


@pytest.mark.parametrize("style,continuation", STYLES)
def test_csc_legacy_attributes_and_many_groups(tmp_path, built_lib, style, continuation):
    """h5sparse_format / h5sparse_shape attributes, a csc X, a root group with
    more members than one symbol-table node holds."""
    from brisc_gb300 import h5ad
    X = _matrix().tocsc()
    tree = h5file.h5ad_tree(X.data, X.indices.astype(np.int32), X.indptr.astype(np.int64),
                            X.shape, fmt="csc_matrix", legacy_attrs=True,
                            continuation=continuation)
    for q in range(13):
        tree.children[f"extra{q:02d}"] = h5file.Group(attrs={"encoding-type": "dict"})
    path = str(tmp_path / "c.h5ad")
    h5file.write(path, tree, style=style)
    info = h5ad.inspect(path)
    assert info["format"] == "csc" and info["shape"] == X.shape
    _check_ranges(path, info, {"data": X.data, "indptr": X.indptr.astype(np.int64)})


@pytest.mark.parametrize("style", ["v0", "v2"])
def test_X_key_choice_as_the_reference(tmp_path, built_lib, style):
    """layers/UMIs, else raw/X, else X (single_cell.py:497-509); an explicit
    X_key wins; both UMIs and raw.X is an error."""
    from brisc_gb300 import h5ad
    A, B = _matrix(seed=2), _matrix(n=200, seed=3)
    for key in ("raw/X", "layers/UMIs"):
        tree = h5file.h5ad_tree(A.data, A.indices, A.indptr, A.shape)
        extra = h5file.h5ad_tree(B.data, B.indices, B.indptr, B.shape, X_key=key)
        for name, node in extra.children.items():
            if name not in tree.children:
                tree.children[name] = node
        path = str(tmp_path / f"k{key.replace('/', '_')}.h5ad")
        h5file.write(path, tree, style=style)
        info = h5ad.inspect(path)
        assert info["X_key"] == key and info["shape"] == B.shape
        assert h5ad.inspect(path, X_key="X")["shape"] == A.shape
    tree = h5file.h5ad_tree(A.data, A.indices, A.indptr, A.shape, X_key="raw/X")
    tree.children["layers"] = h5file.h5ad_tree(B.data, B.indices, B.indptr, B.shape,
                                               X_key="layers/UMIs").children["layers"]
    path = str(tmp_path / "both.h5ad")
    h5file.write(path, tree, style=style)
    with pytest.raises(ValueError, match="both layers\\['UMIs'\\] and raw.X are present"):
        h5ad.inspect(path)
    with pytest.raises(ValueError, match="X_key 'nope' is not present in the .h5ad file"):
        h5ad.inspect(path, X_key="nope")


def test_errors_have_the_references_messages(tmp_path, built_lib):
    from brisc_gb300 import h5ad
    X = _matrix()
    path = str(tmp_path / "e.h5ad")
    h5file.write_h5ad(path, X.data, X.indices, X.indptr, X.shape, fmt="coo_matrix")
    with pytest.raises(ValueError, match="X has unsupported encoding-type 'coo_matrix', but "
                                         "should be 'csr_matrix' or 'csc_matrix'"):
        h5ad.inspect(path)
    h5file.write_h5ad(path, X.data, X.indices, X.indptr[:-1], X.shape)
    with pytest.raises(ValueError, match="X is corrupted: len\\(X.indptr\\) - 1 is 299, but "
                                         "X.shape\\[0\\] is 300"):
        h5ad.inspect(path)
    h5file.write_h5ad(path, X.data, X.indices, X.indptr, X.shape, chunked=True)
    with pytest.raises(NotImplementedError, match="chunked or compressed"):
        h5ad.inspect(path)
    with open(path, "wb") as f:
        f.write(b"not an hdf5 file" * 100)
    with pytest.raises(ValueError, match="not an HDF5 file"):
        h5ad.inspect(path)
    with open(path, "wb") as f:  # a truncated file: metadata points past its end
        h5file.write_h5ad(str(tmp_path / "full.h5ad"), X.data, X.indices, X.indptr, X.shape)
        f.write(open(tmp_path / "full.h5ad", "rb").read()[:2000])
    with pytest.raises(ValueError):
        h5ad.inspect(path)


def test_lookup3_checksum_known_values():
    """The version-2 metadata checksum (Jenkins lookup3 hashlittle) on the
    published test vectors."""
    assert h5file.lookup3(b"", 0) == 0xDEADBEEF
    assert h5file.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert h5file.lookup3(b"Four score and seven years ago", 0) == 0x17770551
    assert h5file.lookup3(b"Four score and seven years ago", 1) == 0xCD628161


def test_reference_reader_at_the_reported_offsets(tmp_path, built_lib):
    """The reference's own contiguous-dataset reader (brisc/hdf5.pyx:163,
    compiled from its sources) given the offsets the metadata reader reports
    returns the arrays written: the offsets are the ones h5py's
    get_offset() would hand it."""
    from oracle import ref
    if ref.load() is None or "hdf5" not in ref.load():
        pytest.skip("the reference's hdf5 module is not built here")
    from brisc_gb300 import h5ad
    X = _matrix(n=5000, g=300)
    path = str(tmp_path / "r.h5ad")
    h5file.write_h5ad(path, X.data, X.indices.astype(np.int32), X.indptr.astype(np.int64),
                      X.shape)
    info = h5ad.inspect(path)
    got = ref.run_read_all_datasets(
        path, [(info[k]["file_offset"], info[k]["dtype"], info[k]["num_elements"])
               for k in ("data", "indices", "indptr")], num_threads=4)
    np.testing.assert_array_equal(got[0], X.data)
    np.testing.assert_array_equal(got[1], X.indices)
    np.testing.assert_array_equal(got[2], X.indptr)
