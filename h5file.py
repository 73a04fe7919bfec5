"""A minimal HDF5 writer for synthetic .h5ad inputs (benchmark and tests).

Neither h5py nor the HDF5 library is installed here, so the benchmark's and the
tests' .h5ad files are written by this module, following the HDF5 File Format
Specification (version 3.0) for the structures h5py writes:

* ``style="v0"`` (h5py's default, ``libver="earliest"``): superblock version 0,
  version-1 object headers, groups as symbol tables (a version-1 B-tree over
  symbol-table nodes, names in a local heap), version-1 attribute messages;
* ``style="v2"`` (``libver="latest"``): superblock version 2, version-2 object
  headers ("OHDR", Jenkins lookup3 checksums), groups as compact link
  messages, version-3 attribute messages.

Datasets are 1-D or 2-D, little-endian integers or IEEE floats, stored
contiguously (layout message version 3) or, to exercise a reader's refusal,
declared chunked. Attributes: scalar variable-length UTF-8 strings (data in a
global heap collection, as h5py stores ``str``), fixed-length strings and
integer arrays. ``continuation=True`` moves a group's or dataset's attributes
to a continuation block, as the HDF5 library does when attributes are added
after the object was created.

An .h5ad file is a tree: ``write_h5ad`` lays out AnnData's sparse ``X``
(``data``, ``indices``, ``indptr`` with ``encoding-type``, ``encoding-version``
and ``shape`` attributes) plus the usual top-level groups.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"


# ---------------------------------------------------------------------------
# Jenkins lookup3 hashlittle (the checksum of version-2 metadata)
def _rot(x, k):
    return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF


def lookup3(data: bytes, initval: int = 0) -> int:
    length = len(data)
    a = b = c = (0xDEADBEEF + length + initval) & 0xFFFFFFFF
    i = 0
    M = 0xFFFFFFFF
    while length > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & M
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & M
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & M
        a = (a - c) & M; a ^= _rot(c, 4); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 6); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 8); b = (b + a) & M
        a = (a - c) & M; a ^= _rot(c, 16); c = (c + b) & M
        b = (b - a) & M; b ^= _rot(a, 19); a = (a + c) & M
        c = (c - b) & M; c ^= _rot(b, 4); b = (b + a) & M
        i += 12
        length -= 12
    if length == 0:
        return c
    tail = data[i:] + b"\0" * (12 - length)
    a = (a + int.from_bytes(tail[0:4], "little")) & M
    b = (b + int.from_bytes(tail[4:8], "little")) & M
    c = (c + int.from_bytes(tail[8:12], "little")) & M
    c ^= b; c = (c - _rot(b, 14)) & M
    a ^= c; a = (a - _rot(c, 11)) & M
    b ^= a; b = (b - _rot(a, 25)) & M
    c ^= b; c = (c - _rot(b, 16)) & M
    a ^= c; a = (a - _rot(c, 4)) & M
    b ^= a; b = (b - _rot(a, 14)) & M
    c ^= b; c = (c - _rot(b, 24)) & M
    return c


# ---------------------------------------------------------------------------
# the tree
@dataclass
class Dataset:
    data: np.ndarray
    attrs: dict = field(default_factory=dict)
    chunked: bool = False          # declare a chunked layout (no chunk index)
    continuation: bool = False


@dataclass
class Group:
    children: dict = field(default_factory=dict)
    attrs: dict = field(default_factory=dict)
    continuation: bool = False


class FixedString(str):
    """An attribute written as a fixed-length (null-padded) string."""


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0x00
        return bytes([0x10, bits, 0, 0]) + struct.pack("<IHH", dt.itemsize, 0,
                                                       dt.itemsize * 8)
    if dt.kind == "f":
        if dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        else:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        return bytes([0x11, 0x20, dt.itemsize * 8 - 1, 0]) + \
            struct.pack("<I", dt.itemsize) + props
    raise TypeError(f"unsupported dtype {dt}")


def _vlen_str_type() -> bytes:
    base = bytes([0x10, 0, 0, 0]) + struct.pack("<IHH", 1, 0, 8)
    return bytes([0x19, 0x01, 0x01, 0]) + struct.pack("<I", 16) + base


def _fixed_str_type(n: int) -> bytes:
    return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", n)


def _space_v1(shape) -> bytes:
    out = bytes([1, len(shape), 0, 0]) + b"\0" * 4
    for s in shape:
        out += struct.pack("<Q", s)
    return out


def _space_v2(shape) -> bytes:
    out = bytes([2, len(shape), 0, 1 if len(shape) else 0])
    for s in shape:
        out += struct.pack("<Q", s)
    return out


class _Writer:
    def __init__(self, style: str):
        assert style in ("v0", "v2")
        self.style = style
        self.buf = bytearray()
        self.strings = []      # vlen attribute strings, in order
        self.gcol_addr = 0

    def alloc(self, payload: bytes, align: int = 8) -> int:
        self.buf += b"\0" * (-len(self.buf) % align)
        at = len(self.buf)
        self.buf += payload
        return at

    # -- attributes ----------------------------------------------------------
    def _collect_strings(self, node):
        for v in node.attrs.values():
            if isinstance(v, str) and not isinstance(v, FixedString):
                self.strings.append(v.encode())
        if isinstance(node, Group):
            for c in node.children.values():
                self._collect_strings(c)

    def _write_gcol(self):
        objs = b""
        for i, s in enumerate(self.strings, start=1):
            objs += struct.pack("<HHIQ", i, 1, 0, len(s)) + _pad8(s)
        size = 16 + len(objs) + 16
        size = max(size, 4096)
        body = b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", size) + objs
        free = size - len(body)
        body += struct.pack("<HHIQ", 0, 0, 0, free) if free >= 16 else b""
        body += b"\0" * (size - len(body))
        self.gcol_addr = self.alloc(body)
        self._string_index = {s: i for i, s in enumerate(self.strings, start=1)}

    def _attr_parts(self, value):
        """(datatype, dataspace shape, raw data) of an attribute value."""
        if isinstance(value, FixedString):
            b = value.encode()
            return _fixed_str_type(len(b) + 1), (), b + b"\0"
        if isinstance(value, str):
            b = value.encode()
            heap_id = struct.pack("<IQI", len(b), self.gcol_addr, self._string_index[b])
            return _vlen_str_type(), (), heap_id
        a = np.ascontiguousarray(value)
        if a.dtype.kind in "iuf":
            a = a.astype(a.dtype.newbyteorder("<"))
            return _dtype_msg(a.dtype), a.shape, a.tobytes()
        raise TypeError(f"unsupported attribute {value!r}")

    def _attr_msg(self, name: str, value) -> bytes:
        dtm, shape, raw = self._attr_parts(value)
        nm = name.encode() + b"\0"
        if self.style == "v0":
            sp = _space_v1(shape)
            return struct.pack("<BBHHH", 1, 0, len(nm), len(dtm), len(sp)) + \
                _pad8(nm) + _pad8(dtm) + _pad8(sp) + raw
        sp = _space_v2(shape)
        return struct.pack("<BBHHHB", 3, 0, len(nm), len(dtm), len(sp), 1) + nm + dtm + \
            sp + raw

    # -- object headers ------------------------------------------------------
    def _ohdr(self, msgs, cont_msgs=None) -> int:
        """Writes an object header with messages [(type, body)]; cont_msgs go
        to a continuation block."""
        cont_addr, cont_len = None, 0
        if cont_msgs:
            if self.style == "v0":
                block = b"".join(self._msg_v1(t, b) for t, b in cont_msgs)
            else:
                body = b"OCHK" + b"".join(self._msg_v2(t, b) for t, b in cont_msgs)
                block = body + struct.pack("<I", lookup3(body))
            cont_addr = self.alloc(block)
            cont_len = len(block)
            msgs = list(msgs) + [(0x10, struct.pack("<QQ", cont_addr, cont_len))]
        if self.style == "v0":
            area = b"".join(self._msg_v1(t, b) for t, b in msgs)
            head = struct.pack("<BBHII", 1, 0, len(msgs) + (len(cont_msgs or [])),
                               1, len(area)) + b"\0" * 4
            return self.alloc(head + area)
        area = b"".join(self._msg_v2(t, b) for t, b in msgs)
        body = b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(area)) + area
        return self.alloc(body + struct.pack("<I", lookup3(body)))

    @staticmethod
    def _msg_v1(t: int, body: bytes) -> bytes:
        body = _pad8(body)
        return struct.pack("<HHB", t, len(body), 0) + b"\0" * 3 + body

    @staticmethod
    def _msg_v2(t: int, body: bytes) -> bytes:
        return struct.pack("<BHB", t, len(body), 0) + body

    # -- objects ---------------------------------------------------------------
    def dataset(self, ds: Dataset) -> int:
        a = np.ascontiguousarray(ds.data)
        a = a.astype(a.dtype.newbyteorder("<"))
        raw_addr = self.alloc(a.tobytes(), align=16) if not ds.chunked else UNDEF
        space = _space_v1(a.shape) if self.style == "v0" else _space_v2(a.shape)
        if ds.chunked:
            rank = a.ndim + 1
            dims = [min(1024, s) for s in a.shape] + [a.itemsize]
            layout = struct.pack("<BBBQ", 3, 2, rank, UNDEF) + \
                b"".join(struct.pack("<I", x) for x in dims)
        else:
            layout = struct.pack("<BBQQ", 3, 1, raw_addr, a.nbytes)
        msgs = [(0x01, space), (0x03, _dtype_msg(a.dtype))]
        if self.style == "v0":  # fill value (new style, version 2): allocation late, no fill
            msgs.append((0x05, bytes([2, 2, 2, 0])))
        msgs.append((0x08, layout))
        attrs = [(0x0C, self._attr_msg(k, v)) for k, v in ds.attrs.items()]
        if ds.continuation:
            return self._ohdr(msgs, attrs)
        return self._ohdr(msgs + attrs)

    def group(self, g: Group) -> int:
        kids = {name: (self.group(c) if isinstance(c, Group) else self.dataset(c))
                for name, c in sorted(g.children.items())}
        attrs = [(0x0C, self._attr_msg(k, v)) for k, v in g.attrs.items()]
        if self.style == "v0":
            btree, heap = self._symbol_table(kids)
            msgs = [(0x11, struct.pack("<QQ", btree, heap))]
        else:
            msgs = [(0x02, bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF)),
                    (0x0A, bytes([0, 0]))]
            for name, addr in kids.items():
                nm = name.encode()
                msgs.append((0x06, bytes([1, 0x00, len(nm)]) + nm + struct.pack("<Q", addr)))
        if g.continuation:
            return self._ohdr(msgs, attrs)
        return self._ohdr(msgs + attrs)

    def _symbol_table(self, kids: dict):
        """A local heap of the names and a one-level v1 B-tree over symbol
        table nodes of up to 8 entries (group leaf node K = 4)."""
        heap_data = bytearray(b"\0" * 8)  # offset 0: the empty string
        offsets = {}
        for name in kids:
            offsets[name] = len(heap_data)
            heap_data += _pad8(name.encode() + b"\0")
        data_addr = self.alloc(bytes(heap_data))
        heap = self.alloc(b"HEAP" + bytes([0, 0, 0, 0]) +
                          struct.pack("<QQQ", len(heap_data), UNDEF, data_addr))
        names = list(kids)
        snods, last_names = [], []
        for i in range(0, max(len(names), 1), 8):
            part = names[i:i + 8]
            entries = b"".join(struct.pack("<QQII", offsets[nm], kids[nm], 0, 0) + b"\0" * 16
                               for nm in part)
            entries += b"\0" * (40 * (8 - len(part)))
            snods.append(self.alloc(b"SNOD" + bytes([1, 0]) +
                                    struct.pack("<H", len(part)) + entries))
            last_names.append(offsets[part[-1]] if part else 0)
        node = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(snods), UNDEF, UNDEF)
        node += struct.pack("<Q", 0)
        for addr, key in zip(snods, last_names):
            node += struct.pack("<QQ", addr, key)
        node += b"\0" * ((2 * 16 - len(snods)) * 16)  # room for 2K children, K = 16
        return self.alloc(node), heap

    def finish(self, root: Group) -> bytes:
        self._collect_strings(root)
        if self.style == "v0":
            self.alloc(b"\0" * 96)  # superblock, patched below
        else:
            self.alloc(b"\0" * 48)
        if self.strings:
            self._write_gcol()
        root_addr = self.group(root)
        eof = len(self.buf)
        if self.style == "v0":
            sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
            sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
            sb += struct.pack("<QQII", 0, root_addr, 0, 0) + b"\0" * 16
            assert len(sb) == 96
        else:
            sb = SIGNATURE + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, UNDEF, eof, root_addr)
            sb += struct.pack("<I", lookup3(sb))
            assert len(sb) == 48
        self.buf[0:len(sb)] = sb
        return bytes(self.buf)


def write(path: str, root: Group, style: str = "v0") -> None:
    with open(path, "wb") as f:
        f.write(_Writer(style).finish(root))


def h5ad_tree(data, indices, indptr, shape, *, fmt: str = "csr_matrix",
              X_key: str = "X", legacy_attrs: bool = False,
              continuation: bool = False, chunked: bool = False,
              obs_names=None, var_names=None) -> Group:
    """AnnData's layout with a sparse matrix at X_key ('X', 'raw/X' or
    'layers/UMIs'): a group of data / indices / indptr with encoding-type and
    shape attributes (or, with legacy_attrs, h5sparse_format and
    h5sparse_shape)."""
    n, g = shape
    if legacy_attrs:
        xattrs = {"h5sparse_format": fmt.split("_")[0],
                  "h5sparse_shape": np.array(shape, dtype=np.int64)}
    else:
        xattrs = {"encoding-type": fmt, "encoding-version": "0.1.0",
                  "shape": np.array(shape, dtype=np.int64)}
    Xg = Group({"data": Dataset(np.asarray(data), chunked=chunked),
                "indices": Dataset(np.asarray(indices)),
                "indptr": Dataset(np.asarray(indptr))}, xattrs, continuation=continuation)
    obs_index = np.arange(n, dtype=np.int64) if obs_names is None else obs_names
    var_index = np.arange(g, dtype=np.int64) if var_names is None else var_names
    df = lambda idx: Group({"_index": Dataset(idx)},  # noqa: E731
                           {"_index": "_index", "column-order": np.zeros(0, np.int64),
                            "encoding-type": "dataframe", "encoding-version": "0.2.0"})
    root = Group({"obs": df(obs_index), "var": df(var_index),
                  "obsm": Group(attrs={"encoding-type": "dict", "encoding-version": "0.1.0"}),
                  "uns": Group(attrs={"encoding-type": "dict", "encoding-version": "0.1.0"})},
                 {"encoding-type": "anndata", "encoding-version": "0.1.0"})
    parts = X_key.split("/")
    node = root
    for p in parts[:-1]:
        node = node.children.setdefault(p, Group(attrs={"encoding-type": "dict",
                                                        "encoding-version": "0.1.0"}))
    node.children[parts[-1]] = Xg
    return root


def write_h5ad(path: str, data, indices, indptr, shape, *, style: str = "v0",
               **kw) -> None:
    write(path, h5ad_tree(data, indices, indptr, shape, **kw), style=style)
