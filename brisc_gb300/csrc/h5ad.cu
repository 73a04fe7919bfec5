// The count matrix of an .h5ad file, read straight into device memory: the
// reference's fast path for AnnData files (brisc/single_cell.py:83-1400 with
// brisc/hdf5.pyx:163 read_all_datasets) without the host-side arrays.
//
// The reference asks h5py for each dataset's byte offset in the file
// (single_cell.py:1848-1883, `dataset.id.get_offset()`; None when the dataset
// is chunked or compressed) and then preads the contiguous bytes with OpenMP
// threads into NumPy arrays. Here the HDF5 metadata is parsed directly
// (HDF5 File Format Specification 3.0: superblock versions 0-3, version-1 and
// version-2 object headers with continuation blocks, groups stored as symbol
// tables (v1 B-tree, symbol-table nodes, local heap) or as compact link
// messages, dataspace, datatype, data-layout and attribute messages,
// variable-length string attributes in global heap collections), and the
// three datasets of the sparse X (data, indices, indptr) are streamed by
// host threads: pread into pinned staging buffers, cudaMemcpyAsync into the
// caller's device arrays, two buffers per thread so reading and copying
// overlap. Dense-link groups (fractal heaps), shared messages, chunked or
// filtered datasets are not read (BGPU_ERR_UNSUPPORTED), as the reference
// sends chunked/compressed files to a slower reader.
//
// X is chosen as the reference chooses it (single_cell.py:497-522, 610-657):
// X_key, or 'layers/UMIs' when present, else 'raw/X' when present, else 'X';
// the matrix class from the 'encoding-type' attribute, else
// 'h5sparse_format' + '_matrix'; the shape from 'shape', else
// 'h5sparse_shape'.
#include <fcntl.h>
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace bgpu {
namespace {

constexpr uint64_t kUndef = ~0ull;

struct H5Error {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& m) { throw H5Error{code, m}; }

// Little-endian field reader over a byte buffer, bounds-checked.
struct Cursor {
  const uint8_t* p;
  size_t n, i = 0;
  Cursor(const uint8_t* p_, size_t n_) : p(p_), n(n_) {}
  void need(size_t k) const {
    if (i + k > n) fail(BGPU_ERR_INVALID, "HDF5: truncated metadata structure");
  }
  uint64_t u(int bytes) {
    need(bytes);
    uint64_t v = 0;
    for (int b = 0; b < bytes; ++b) v |= (uint64_t)p[i + b] << (8 * b);
    i += bytes;
    return v;
  }
  void skip(size_t k) {
    need(k);
    i += k;
  }
  const uint8_t* here() const { return p + i; }
  size_t left() const { return n - i; }
};

struct Datatype {
  int cls = -1;       // 0 fixed-point, 1 float, 3 string, 9 variable-length
  uint32_t size = 0;
  bool is_signed = false;
  bool big_endian = false;
  bool vlen_string = false;
};

struct Dataspace {
  std::vector<uint64_t> dims;  // empty: scalar
  bool null = false;
  uint64_t elements() const {
    uint64_t e = 1;
    for (uint64_t d : dims) e *= d;
    return null ? 0 : e;
  }
};

struct Attribute {
  Datatype type;
  Dataspace space;
  std::vector<uint8_t> data;
};

struct Object {
  bool has_symbol_table = false;
  uint64_t btree = kUndef, heap = kUndef;
  bool has_link_info = false;
  uint64_t fractal_heap = kUndef;
  std::map<std::string, uint64_t> links;  // compact links
  bool has_space = false, has_type = false, has_layout = false;
  Dataspace space;
  Datatype type;
  int layout_class = -1;  // 0 compact, 1 contiguous, 2 chunked, 3 virtual
  uint64_t data_addr = kUndef, data_size = 0;
  bool filtered = false;
  std::map<std::string, Attribute> attrs;
};

class H5File {
 public:
  explicit H5File(const std::string& path) {
    fd_ = ::open(path.c_str(), O_RDONLY);
    if (fd_ < 0) fail(BGPU_ERR_INVALID, "cannot open " + path + ": " + std::strerror(errno));
    size_ = (uint64_t)::lseek(fd_, 0, SEEK_END);
    read_superblock();
  }
  ~H5File() {
    if (fd_ >= 0) ::close(fd_);
  }
  H5File(const H5File&) = delete;
  H5File& operator=(const H5File&) = delete;

  int offset_size() const { return so_; }
  int length_size() const { return sl_; }

  std::vector<uint8_t> read(uint64_t addr, uint64_t len) const {
    if (addr == kUndef || addr + base_ > size_ || len > size_ - (addr + base_))
      fail(BGPU_ERR_INVALID, "HDF5: an address points outside the file");
    std::vector<uint8_t> b(len);
    uint64_t got = 0;
    while (got < len) {
      const ssize_t r = ::pread(fd_, b.data() + got, len - got, (off_t)(base_ + addr + got));
      if (r < 0 && errno == EINTR) continue;
      if (r <= 0) fail(BGPU_ERR_INVALID, "HDF5: read failed inside the file");
      got += (uint64_t)r;
    }
    return b;
  }
  // Up to `len` bytes (fewer at the end of the file).
  std::vector<uint8_t> read_upto(uint64_t addr, uint64_t len) const {
    if (addr == kUndef || addr + base_ >= size_)
      fail(BGPU_ERR_INVALID, "HDF5: an address points outside the file");
    return read(addr, std::min<uint64_t>(len, size_ - base_ - addr));
  }
  uint64_t file_offset(uint64_t addr) const { return base_ + addr; }

  Object object(uint64_t addr) const;
  // Resolves a '/'-separated path from the root; kUndef when absent.
  uint64_t lookup(const std::string& path) const;
  std::map<std::string, uint64_t> members(const Object& g) const;

 private:
  void read_superblock();
  void parse_messages(Object& o, Cursor& c, int ohv, uint8_t oh_flags,
                      std::vector<std::pair<uint64_t, uint64_t>>& cont) const;
  void message(Object& o, int type, const uint8_t* p, size_t n, uint8_t flags) const;
  Datatype parse_type(Cursor& c) const;
  Dataspace parse_space(Cursor& c) const;
  void symbol_table_members(uint64_t btree, uint64_t heap,
                            std::map<std::string, uint64_t>& out, int depth) const;

  int fd_ = -1;
  uint64_t size_ = 0, base_ = 0, root_ = kUndef;
  int so_ = 8, sl_ = 8;
};

void H5File::read_superblock() {
  static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  uint64_t at = 0;
  for (;; at = at ? at * 2 : 512) {
    if (at + 8 > size_) fail(BGPU_ERR_INVALID, "not an HDF5 file (no superblock signature)");
    uint8_t b[8];
    if (::pread(fd_, b, 8, (off_t)at) != 8) fail(BGPU_ERR_INVALID, "HDF5: read failed");
    if (std::memcmp(b, sig, 8) == 0) break;
  }
  uint8_t hdr[256];
  const ssize_t r = ::pread(fd_, hdr, sizeof hdr, (off_t)at);
  if (r < 16) fail(BGPU_ERR_INVALID, "HDF5: truncated superblock");
  Cursor c(hdr, (size_t)r);
  c.skip(8);
  const int version = (int)c.u(1);
  if (version == 0 || version == 1) {
    c.skip(4);  // free-space, root symbol table entry, reserved, shared header versions
    so_ = (int)c.u(1);
    sl_ = (int)c.u(1);
    c.skip(1);
    c.skip(4);  // group leaf / internal node K
    c.skip(4);  // consistency flags
    if (version == 1) c.skip(4);
    if (so_ != 2 && so_ != 4 && so_ != 8) fail(BGPU_ERR_UNSUPPORTED, "HDF5: offset size");
    if (sl_ != 2 && sl_ != 4 && sl_ != 8) fail(BGPU_ERR_UNSUPPORTED, "HDF5: length size");
    base_ = c.u(so_);
    c.skip(3 * (size_t)so_);  // free-space info, end of file, driver information block
    c.skip(so_);               // root entry: link name offset
    root_ = c.u(so_);          // root entry: object header address
  } else if (version == 2 || version == 3) {
    so_ = (int)c.u(1);
    sl_ = (int)c.u(1);
    if (so_ != 2 && so_ != 4 && so_ != 8) fail(BGPU_ERR_UNSUPPORTED, "HDF5: offset size");
    if (sl_ != 2 && sl_ != 4 && sl_ != 8) fail(BGPU_ERR_UNSUPPORTED, "HDF5: length size");
    c.skip(1);  // flags
    base_ = c.u(so_);
    c.skip(2 * (size_t)so_);  // superblock extension, end of file
    root_ = c.u(so_);
  } else {
    fail(BGPU_ERR_UNSUPPORTED, "HDF5: superblock version " + std::to_string(version));
  }
  if (base_ == kUndef) base_ = 0;
  if (so_ < 8 && root_ == ((1ull << (8 * so_)) - 1)) root_ = kUndef;
  if (base_ == 0 && at != 0) base_ = at;  // a user block before the superblock
}

Datatype H5File::parse_type(Cursor& c) const {
  Datatype t;
  const uint8_t cv = (uint8_t)c.u(1);
  t.cls = cv & 0x0F;
  const uint32_t bits = (uint32_t)c.u(3);
  t.size = (uint32_t)c.u(4);
  switch (t.cls) {
    case 0:  // fixed-point
      t.big_endian = bits & 1;
      t.is_signed = (bits >> 3) & 1;
      c.skip(4);
      break;
    case 1:  // floating-point
      t.big_endian = bits & 1;
      c.skip(12);
      break;
    case 3:  // string
      break;
    case 9: {  // variable-length: a sequence or a string; its base type follows
      t.vlen_string = (bits & 0x0F) == 1;
      parse_type(c);
      break;
    }
    default:
      // other classes (bitfield, opaque, compound, reference, enum, array)
      // are not needed for the sparse matrix; their properties are not parsed
      c.skip(c.left());
      break;
  }
  return t;
}

Dataspace H5File::parse_space(Cursor& c) const {
  Dataspace s;
  const int version = (int)c.u(1);
  const int rank = (int)c.u(1);
  const int flags = (int)c.u(1);
  if (version == 1) {
    c.skip(5);
  } else if (version == 2) {
    const int type = (int)c.u(1);
    s.null = type == 2;
  } else {
    fail(BGPU_ERR_UNSUPPORTED, "HDF5: dataspace message version " + std::to_string(version));
  }
  for (int r = 0; r < rank; ++r) s.dims.push_back(c.u(sl_));
  if (flags & 1) c.skip((size_t)rank * sl_);
  return s;
}

void H5File::message(Object& o, int type, const uint8_t* p, size_t n, uint8_t flags) const {
  if (flags & 0x02) {
    // a shared message: only the ones the sparse matrix needs matter
    if (type == 0x01 || type == 0x03 || type == 0x08 || type == 0x0C)
      fail(BGPU_ERR_UNSUPPORTED, "HDF5: shared (committed) messages are not read");
    return;
  }
  Cursor c(p, n);
  switch (type) {
    case 0x01:
      o.space = parse_space(c);
      o.has_space = true;
      break;
    case 0x02: {  // link info
      c.skip(1);
      const int f = (int)c.u(1);
      if (f & 1) c.skip(8);
      o.fractal_heap = c.u(so_);
      o.has_link_info = true;
      break;
    }
    case 0x03:
      o.type = parse_type(c);
      o.has_type = true;
      break;
    case 0x06: {  // link
      const int version = (int)c.u(1);
      if (version != 1) fail(BGPU_ERR_UNSUPPORTED, "HDF5: link message version");
      const int f = (int)c.u(1);
      int ltype = 0;
      if (f & 0x08) ltype = (int)c.u(1);
      if (f & 0x04) c.skip(8);
      if (f & 0x10) c.skip(1);
      const uint64_t len = c.u(1 << (f & 3));
      c.need(len);
      std::string name((const char*)c.here(), len);
      c.skip(len);
      if (ltype == 0) o.links[name] = c.u(so_);  // soft / external links are skipped
      break;
    }
    case 0x08: {  // data layout
      const int version = (int)c.u(1);
      if (version == 3 || version == 4) {
        o.layout_class = (int)c.u(1);
        if (o.layout_class == 1) {
          o.data_addr = c.u(so_);
          o.data_size = c.u(sl_);
        } else if (o.layout_class == 0) {
          o.data_size = c.u(2);
          o.data_addr = kUndef;
        }
      } else if (version == 1 || version == 2) {
        const int rank = (int)c.u(1);
        o.layout_class = (int)c.u(1);
        c.skip(5);
        if (o.layout_class != 0) o.data_addr = c.u(so_);
        uint64_t elems = 1;
        for (int r = 0; r < rank; ++r) elems *= c.u(4);
        o.data_size = elems;  // in elements for these versions; fixed below
        if (o.layout_class == 1) o.data_size = kUndef;  // size from the dataspace
      } else {
        fail(BGPU_ERR_UNSUPPORTED, "HDF5: data layout message version");
      }
      o.has_layout = true;
      break;
    }
    case 0x0B:
      o.filtered = true;
      break;
    case 0x0C: {  // attribute
      const int version = (int)c.u(1);
      int f = 0;
      if (version == 1) {
        c.skip(1);
      } else {
        f = (int)c.u(1);
      }
      if (version < 1 || version > 3) fail(BGPU_ERR_UNSUPPORTED, "HDF5: attribute version");
      if (f & 0x03) fail(BGPU_ERR_UNSUPPORTED, "HDF5: shared attribute datatype/dataspace");
      const uint64_t nsz = c.u(2), tsz = c.u(2), ssz = c.u(2);
      if (version == 3) c.skip(1);
      auto pad = [&](uint64_t k) { return version == 1 ? (k + 7) & ~7ull : k; };
      c.need(pad(nsz));
      std::string name((const char*)c.here(), nsz ? nsz - 1 : 0);
      name = name.c_str();
      c.skip(pad(nsz));
      Attribute a;
      {
        c.need(pad(tsz));
        Cursor t(c.here(), tsz);
        a.type = parse_type(t);
        c.skip(pad(tsz));
      }
      {
        c.need(pad(ssz));
        Cursor s(c.here(), ssz);
        a.space = parse_space(s);
        c.skip(pad(ssz));
      }
      a.data.assign(c.here(), c.here() + c.left());
      o.attrs[name] = std::move(a);
      break;
    }
    case 0x11:  // symbol table
      o.btree = c.u(so_);
      o.heap = c.u(so_);
      o.has_symbol_table = true;
      break;
    default:
      break;
  }
}

void H5File::parse_messages(Object& o, Cursor& c, int ohv, uint8_t oh_flags,
                            std::vector<std::pair<uint64_t, uint64_t>>& cont) const {
  while (c.left() > 0) {
    int type;
    uint64_t size;
    uint8_t flags;
    if (ohv == 1) {
      if (c.left() < 8) break;
      type = (int)c.u(2);
      size = c.u(2);
      flags = (uint8_t)c.u(1);
      c.skip(3);
    } else {
      if (c.left() < 4) break;  // a gap at the end of the chunk
      type = (int)c.u(1);
      size = c.u(2);
      flags = (uint8_t)c.u(1);
      if (oh_flags & 0x04) c.skip(2);
    }
    c.need(size);
    if (type == 0x10) {
      Cursor k(c.here(), size);
      const uint64_t addr = k.u(so_), len = k.u(sl_);
      cont.emplace_back(addr, len);
    } else {
      message(o, type, c.here(), size, flags);
    }
    c.skip(size);
  }
}

Object H5File::object(uint64_t addr) const {
  Object o;
  std::vector<std::pair<uint64_t, uint64_t>> cont;
  std::vector<uint8_t> head = read_upto(addr, 16);
  int ohv;
  uint8_t oh_flags = 0;
  if (head.size() >= 4 && std::memcmp(head.data(), "OHDR", 4) == 0) {
    ohv = 2;
    std::vector<uint8_t> pre = read_upto(addr, 64);
    Cursor c(pre.data(), pre.size());
    c.skip(4);
    if (c.u(1) != 2) fail(BGPU_ERR_UNSUPPORTED, "HDF5: object header version");
    oh_flags = (uint8_t)c.u(1);
    if (oh_flags & 0x20) c.skip(16);
    if (oh_flags & 0x10) c.skip(4);
    const uint64_t chunk = c.u(1 << (oh_flags & 3));
    const uint64_t start = c.i;
    std::vector<uint8_t> body = read(addr + start, chunk);
    Cursor m(body.data(), body.size());
    parse_messages(o, m, 2, oh_flags, cont);
  } else {
    if (head.size() < 16 || head[0] != 1)
      fail(BGPU_ERR_INVALID, "HDF5: not an object header at an object's address");
    ohv = 1;
    Cursor c(head.data(), head.size());
    c.skip(8);
    const uint64_t hsize = c.u(4);
    std::vector<uint8_t> body = read(addr + 16, hsize);
    Cursor m(body.data(), body.size());
    parse_messages(o, m, 1, 0, cont);
  }
  for (size_t q = 0; q < cont.size(); ++q) {
    if (q > 4096) fail(BGPU_ERR_INVALID, "HDF5: too many continuation blocks");
    std::vector<uint8_t> blk = read(cont[q].first, cont[q].second);
    if (ohv == 2) {
      if (blk.size() < 8 || std::memcmp(blk.data(), "OCHK", 4) != 0)
        fail(BGPU_ERR_INVALID, "HDF5: bad continuation block");
      Cursor m(blk.data() + 4, blk.size() - 8);
      parse_messages(o, m, 2, oh_flags, cont);
    } else {
      Cursor m(blk.data(), blk.size());
      parse_messages(o, m, 1, 0, cont);
    }
  }
  return o;
}

void H5File::symbol_table_members(uint64_t btree, uint64_t heap,
                                  std::map<std::string, uint64_t>& out, int depth) const {
  if (depth > 64) fail(BGPU_ERR_INVALID, "HDF5: group B-tree too deep");
  std::vector<uint8_t> hh = read(heap, 8 + 2 * (uint64_t)sl_ + so_);
  if (std::memcmp(hh.data(), "HEAP", 4) != 0) fail(BGPU_ERR_INVALID, "HDF5: bad local heap");
  Cursor hc(hh.data(), hh.size());
  hc.skip(8);
  const uint64_t dsize = hc.u(sl_);
  hc.skip(sl_);
  const uint64_t daddr = hc.u(so_);
  const std::vector<uint8_t> names = read(daddr, dsize);
  auto name_at = [&](uint64_t off) {
    if (off >= names.size()) fail(BGPU_ERR_INVALID, "HDF5: bad name offset");
    const char* s = (const char*)names.data() + off;
    return std::string(s, strnlen(s, names.size() - off));
  };
  std::vector<uint8_t> nh = read(btree, 8 + 2 * (uint64_t)so_);
  if (std::memcmp(nh.data(), "TREE", 4) != 0) fail(BGPU_ERR_INVALID, "HDF5: bad group B-tree");
  Cursor nc(nh.data(), nh.size());
  nc.skip(4);
  if (nc.u(1) != 0) fail(BGPU_ERR_INVALID, "HDF5: not a group B-tree node");
  const int level = (int)nc.u(1);
  const uint64_t used = nc.u(2);
  const uint64_t klen = (uint64_t)sl_;
  std::vector<uint8_t> body = read(btree + 8 + 2 * (uint64_t)so_,
                                   klen + used * ((uint64_t)so_ + klen));
  Cursor bc(body.data(), body.size());
  bc.skip(klen);
  for (uint64_t e = 0; e < used; ++e) {
    const uint64_t child = bc.u(so_);
    bc.skip(klen);
    if (level > 0) {
      symbol_table_members(child, heap, out, depth + 1);
      continue;
    }
    std::vector<uint8_t> sh = read(child, 8);
    if (std::memcmp(sh.data(), "SNOD", 4) != 0) fail(BGPU_ERR_INVALID, "HDF5: bad symbol node");
    const uint64_t nsym = (uint64_t)sh[6] | ((uint64_t)sh[7] << 8);
    const uint64_t esz = 2 * (uint64_t)so_ + 24;
    std::vector<uint8_t> ents = read(child + 8, nsym * esz);
    Cursor ec(ents.data(), ents.size());
    for (uint64_t s = 0; s < nsym; ++s) {
      const uint64_t name_off = ec.u(so_), oh = ec.u(so_);
      ec.skip(24);
      out[name_at(name_off)] = oh;
    }
  }
}

std::map<std::string, uint64_t> H5File::members(const Object& g) const {
  std::map<std::string, uint64_t> out;
  if (g.has_symbol_table) {
    symbol_table_members(g.btree, g.heap, out, 0);
  } else {
    if (g.has_link_info && g.fractal_heap != kUndef)
      fail(BGPU_ERR_UNSUPPORTED,
           "HDF5: groups with dense link storage (fractal heaps) are not read");
    out = g.links;
  }
  return out;
}

uint64_t H5File::lookup(const std::string& path) const {
  uint64_t addr = root_;
  size_t at = 0;
  while (at < path.size()) {
    size_t slash = path.find('/', at);
    if (slash == std::string::npos) slash = path.size();
    const std::string part = path.substr(at, slash - at);
    at = slash + 1;
    if (part.empty()) continue;
    const Object g = object(addr);
    if (!g.has_symbol_table && !g.has_link_info && g.links.empty()) return kUndef;
    const auto kids = members(g);
    const auto it = kids.find(part);
    if (it == kids.end()) return kUndef;
    addr = it->second;
  }
  return addr;
}

// An attribute's value as a string (fixed or variable length, scalar).
bool attr_string(const H5File& f, const Object& o, const std::string& name, std::string* out) {
  const auto it = o.attrs.find(name);
  if (it == o.attrs.end()) return false;
  const Attribute& a = it->second;
  if (a.type.cls == 3) {
    const size_t n = std::min<size_t>(a.type.size, a.data.size());
    *out = std::string((const char*)a.data.data(), strnlen((const char*)a.data.data(), n));
    return true;
  }
  if (a.type.cls == 9 && a.type.vlen_string) {
    Cursor c(a.data.data(), a.data.size());
    const uint64_t len = c.u(4), coll = c.u(f.offset_size()), index = c.u(4);
    std::vector<uint8_t> hdr = f.read(coll, 8 + (uint64_t)f.length_size());
    if (std::memcmp(hdr.data(), "GCOL", 4) != 0)
      fail(BGPU_ERR_INVALID, "HDF5: bad global heap collection");
    Cursor hc(hdr.data(), hdr.size());
    hc.skip(8);
    const uint64_t csize = hc.u(f.length_size());
    std::vector<uint8_t> col = f.read(coll, csize);
    Cursor cc(col.data(), col.size());
    cc.skip(8 + (size_t)f.length_size());
    while (cc.left() >= 8 + (size_t)f.length_size()) {
      const uint64_t idx = cc.u(2);
      cc.skip(6);
      const uint64_t osz = cc.u(f.length_size());
      if (idx == 0) break;
      cc.need(osz);
      if (idx == index) {
        *out = std::string((const char*)cc.here(), std::min<uint64_t>(osz, len));
        return true;
      }
      cc.skip((osz + 7) & ~7ull);
    }
    fail(BGPU_ERR_INVALID, "HDF5: a string attribute's heap object is missing");
  }
  return false;
}

// An attribute's value as integers (a 1-D or scalar integer attribute).
bool attr_ints(const Object& o, const std::string& name, std::vector<int64_t>* out) {
  const auto it = o.attrs.find(name);
  if (it == o.attrs.end()) return false;
  const Attribute& a = it->second;
  if (a.type.cls != 0 || a.type.big_endian || (a.type.size != 4 && a.type.size != 8))
    return false;
  const uint64_t n = a.space.elements();
  if (a.data.size() < n * a.type.size) fail(BGPU_ERR_INVALID, "HDF5: short attribute data");
  out->clear();
  Cursor c(a.data.data(), a.data.size());
  for (uint64_t e = 0; e < n; ++e) {
    uint64_t v = c.u((int)a.type.size);
    if (a.type.size == 4 && a.type.is_signed && (v & 0x80000000u)) v |= 0xFFFFFFFF00000000ull;
    out->push_back((int64_t)v);
  }
  return true;
}

// Element type code of a numeric dataset (BGPU_VALUE_* for data,
// BGPU_INDEX_* for index arrays).
int value_code(const Datatype& t) {
  if (t.big_endian) return -1;
  if (t.cls == 1) return t.size == 4 ? BGPU_VALUE_F32 : t.size == 8 ? BGPU_VALUE_F64 : -1;
  if (t.cls != 0) return -1;
  if (t.size == 2 && !t.is_signed) return BGPU_VALUE_U16;
  if (t.size == 4) return t.is_signed ? BGPU_VALUE_I32 : BGPU_VALUE_U32;
  if (t.size == 8) return t.is_signed ? BGPU_VALUE_I64 : BGPU_VALUE_U64;
  return -1;
}
int index_code(const Datatype& t) {
  if (t.big_endian || t.cls != 0) return -1;
  if (t.size == 4) return t.is_signed ? BGPU_H5_I32 : BGPU_H5_U32;
  if (t.size == 8) return t.is_signed ? BGPU_H5_I64 : BGPU_H5_U64;
  return -1;
}

void describe(const H5File& f, uint64_t addr, const char* what, bgpu_h5_dataset* out,
              bool numeric_value) {
  const Object o = f.object(addr);
  if (!o.has_layout || !o.has_type || !o.has_space)
    fail(BGPU_ERR_INVALID, std::string("X/") + what + " is not a dataset");
  if (o.space.dims.size() != 1)
    fail(BGPU_ERR_INVALID, std::string("X/") + what + " is not one-dimensional");
  const int code = numeric_value ? value_code(o.type) : index_code(o.type);
  if (code < 0)
    fail(BGPU_ERR_UNSUPPORTED, std::string("X/") + what + " has an unsupported element type");
  const uint64_t elems = o.space.elements();
  const uint64_t bytes = elems * o.type.size;
  out->num_elements = elems;
  out->element_size = o.type.size;
  out->type = code;
  if (o.layout_class == 0) {
    fail(BGPU_ERR_UNSUPPORTED, std::string("X/") + what +
                                   " is stored compact (inside its object header)");
  }
  if (o.layout_class != 1 || o.filtered)
    fail(BGPU_ERR_UNSUPPORTED, std::string("X/") + what +
                                   " is chunked or compressed (only contiguous datasets "
                                   "are read straight to the device)");
  if (elems == 0) {
    out->file_offset = 0;
    out->num_bytes = 0;
    return;
  }
  if (o.data_addr == kUndef) fail(BGPU_ERR_INVALID, std::string("X/") + what + ": no storage");
  if (o.data_size != kUndef && o.data_size < bytes)
    fail(BGPU_ERR_INVALID, std::string("X/") + what + ": storage smaller than its dataspace");
  out->file_offset = f.file_offset(o.data_addr);
  out->num_bytes = bytes;
  f.read(o.data_addr + bytes - 1, 1);  // the storage lies inside the file
}

int inspect(const char* path, const char* X_key, bgpu_h5ad_matrix* out) {
  H5File f(path);
  std::string key;
  if (X_key && *X_key) {
    key = X_key;
    if (f.lookup(key) == kUndef)
      fail(BGPU_ERR_INVALID, "X_key '" + key + "' is not present in the .h5ad file");
  } else {
    const bool umis = f.lookup("layers/UMIs") != kUndef, raw = f.lookup("raw/X") != kUndef;
    if (umis && raw)
      fail(BGPU_ERR_INVALID, "both layers['UMIs'] and raw.X are present; this should never "
                             "happen in well-formed .h5ad files");
    key = umis ? "layers/UMIs" : raw ? "raw/X" : "X";
  }
  const uint64_t xaddr = f.lookup(key);
  if (xaddr == kUndef) fail(BGPU_ERR_INVALID, "the .h5ad file has no X");
  const Object X = f.object(xaddr);
  if (X.has_layout)
    fail(BGPU_ERR_UNSUPPORTED, "'" + key + "' is stored as a dense matrix; only sparse X "
                               "is read straight to the device");
  std::string cls;
  if (!attr_string(f, X, "encoding-type", &cls)) {
    std::string fmt;
    if (!attr_string(f, X, "h5sparse_format", &fmt))
      fail(BGPU_ERR_INVALID, "X has neither an encoding-type nor an h5sparse_format attribute");
    cls = fmt + "_matrix";
  }
  if (cls != "csr_matrix" && cls != "csc_matrix")
    fail(BGPU_ERR_INVALID, "X has unsupported encoding-type '" + cls +
                               "', but should be 'csr_matrix' or 'csc_matrix'");
  std::vector<int64_t> shape;
  if (!attr_ints(X, "shape", &shape) && !attr_ints(X, "h5sparse_shape", &shape))
    fail(BGPU_ERR_INVALID, "X has no shape attribute");
  if (shape.size() != 2 || shape[0] < 0 || shape[1] < 0)
    fail(BGPU_ERR_INVALID, "X's shape attribute is not two non-negative integers");
  const auto kids = f.members(X);
  auto need = [&](const char* name) {
    const auto it = kids.find(name);
    if (it == kids.end()) fail(BGPU_ERR_INVALID, std::string("X has no '") + name + "'");
    return it->second;
  };
  std::memset(out, 0, sizeof *out);
  std::snprintf(out->X_key, sizeof out->X_key, "%s", key.c_str());
  out->is_csr = cls == "csr_matrix";
  out->num_rows = (uint64_t)shape[0];
  out->num_columns = (uint64_t)shape[1];
  describe(f, need("data"), "data", &out->data, true);
  describe(f, need("indices"), "indices", &out->indices, false);
  describe(f, need("indptr"), "indptr", &out->indptr, false);
  const uint64_t major = out->is_csr ? out->num_rows : out->num_columns;
  if (out->indptr.num_elements != major + 1)
    fail(BGPU_ERR_INVALID, "X is corrupted: len(X.indptr) - 1 is " +
                               std::to_string(out->indptr.num_elements - 1) +
                               ", but X.shape[" + std::to_string(out->is_csr ? 0 : 1) +
                               "] is " + std::to_string(major));
  if (out->indices.num_elements != out->data.num_elements)
    fail(BGPU_ERR_INVALID, "X is corrupted: X.indices and X.data differ in length");
  out->nnz = out->data.num_elements;
  return BGPU_OK;
}

// ---------------------------------------------------------------------------
// streaming reader
constexpr uint64_t kPiece = 4ull << 20;  // bytes per pread / copy
constexpr int kMaxThreads = 64;

struct Staging {
  std::mutex mu;
  std::vector<void*> bufs;  // 2 per thread, kPiece bytes each, pinned
};
Staging& staging() {
  static Staging s;
  return s;
}

struct Piece {
  uint64_t offset, bytes;
  char* dst;
};

int read_pieces(const char* path, const std::vector<Piece>& pieces, int threads,
                cudaStream_t caller) {
  const int fd = ::open(path, O_RDONLY);
  BGPU_REQUIRE(fd >= 0, BGPU_ERR_IO, std::string("cannot open ") + path);
  Staging& st = staging();
  std::lock_guard<std::mutex> lock(st.mu);  // one streaming read at a time per process
  while ((int)st.bufs.size() < 2 * threads) {
    void* p = nullptr;
    const cudaError_t e = cudaHostAlloc(&p, kPiece, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      ::close(fd);
      set_error(std::string("cudaHostAlloc of a staging buffer failed: ") +
                cudaGetErrorString(e));
      return BGPU_ERR_ALLOC;
    }
    st.bufs.push_back(p);
  }
  // the caller's earlier work on its stream (e.g. allocating the outputs)
  // comes first
  {
    const cudaError_t e = cudaStreamSynchronize(caller);
    if (e != cudaSuccess) {
      ::close(fd);
      set_error(std::string("cudaStreamSynchronize failed: ") + cudaGetErrorString(e));
      return BGPU_ERR_CUDA;
    }
  }
  std::atomic<int> status{BGPU_OK};
  std::atomic<uint64_t> next{0};
  std::mutex emu;
  std::string emsg;
  auto set_fail = [&](int code, const std::string& m) {
    int ok = BGPU_OK;
    if (status.compare_exchange_strong(ok, code)) {
      std::lock_guard<std::mutex> g(emu);
      emsg = m;
    }
  };
  auto worker = [&](int t) {
    cudaStream_t s = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool live[2] = {false, false};
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming) != cudaSuccess) {
      set_fail(BGPU_ERR_CUDA, "creating a copy stream failed");
    }
    for (uint64_t k = 0; status.load() == BGPU_OK; ++k) {
      const uint64_t q = next.fetch_add(1);
      if (q >= pieces.size()) break;
      const int b = (int)(k & 1);
      char* buf = (char*)st.bufs[2 * t + b];
      if (live[b] && cudaEventSynchronize(ev[b]) != cudaSuccess) {
        set_fail(BGPU_ERR_CUDA, "a host-to-device copy failed");
        break;
      }
      const Piece& p = pieces[q];
      uint64_t got = 0;
      while (got < p.bytes) {
        const ssize_t r = ::pread(fd, buf + got, p.bytes - got, (off_t)(p.offset + got));
        if (r < 0 && (errno == EINTR || errno == EAGAIN)) continue;
        if (r <= 0) {
          set_fail(BGPU_ERR_IO, r == 0 ? "the .h5ad file ends before its data"
                                       : std::string("pread failed: ") + std::strerror(errno));
          break;
        }
        got += (uint64_t)r;
      }
      if (got < p.bytes) break;
      if (cudaMemcpyAsync(p.dst, buf, p.bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
          cudaEventRecord(ev[b], s) != cudaSuccess) {
        set_fail(BGPU_ERR_CUDA, "cudaMemcpyAsync to the device failed");
        break;
      }
      live[b] = true;
    }
    if (s) cudaStreamSynchronize(s);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (s) cudaStreamDestroy(s);
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) pool.emplace_back(worker, t);
  for (auto& th : pool) th.join();
  ::close(fd);
  if (status.load() != BGPU_OK) {
    set_error(emsg);
    return status.load();
  }
  return BGPU_OK;
}

}  // namespace
}  // namespace bgpu

using namespace bgpu;

extern "C" int bgpu_h5ad_inspect(const char* path, const char* X_key, bgpu_h5ad_matrix* out) {
  BGPU_REQUIRE(path && out, BGPU_ERR_INVALID, "h5ad: NULL argument");
  try {
    return inspect(path, X_key, out);
  } catch (const H5Error& e) {
    set_error(e.msg);
    return e.code;
  } catch (const std::bad_alloc&) {
    set_error("h5ad: host allocation failed while parsing the file's metadata");
    return BGPU_ERR_ALLOC;
  }
}

// Zero-copy: the byte range of the three datasets mapped read-only and
// registered with the driver (cudaHostRegisterReadOnly, the registration made
// for read-only file mappings), so the copy engines read the page-cache pages
// directly and no host thread copies a byte. *refused is set (and nothing is
// copied) when the mapping or the registration is not possible here.
int read_mapped(const char* path, const bgpu_h5_dataset* const ds[3], void* const dst[3],
                cudaStream_t s, bool* refused) {
  *refused = true;
  int dev = 0, ro = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&ro, cudaDevAttrHostRegisterReadOnlySupported, dev) !=
          cudaSuccess || !ro) {
    cudaGetLastError();
    return BGPU_OK;
  }
  uint64_t lo = ~0ull, hi = 0;
  for (int q = 0; q < 3; ++q)
    if (ds[q]->num_bytes) {
      lo = std::min(lo, ds[q]->file_offset);
      hi = std::max(hi, ds[q]->file_offset + ds[q]->num_bytes);
    }
  if (hi == 0) {
    *refused = false;
    return BGPU_OK;
  }
  const int fd = ::open(path, O_RDONLY);
  BGPU_REQUIRE(fd >= 0, BGPU_ERR_IO, std::string("cannot open ") + path);
  const off_t fsize = ::lseek(fd, 0, SEEK_END);
  if (fsize < 0 || (uint64_t)fsize < hi) {
    ::close(fd);
    BGPU_REQUIRE(false, BGPU_ERR_IO, "the .h5ad file ends before its data");
  }
  const uint64_t page = (uint64_t)sysconf(_SC_PAGESIZE);
  const uint64_t start = lo & ~(page - 1), len = hi - start;
  void* map = ::mmap(nullptr, len, PROT_READ, MAP_SHARED, fd, (off_t)start);
  if (map == MAP_FAILED) {
    ::close(fd);
    return BGPU_OK;
  }
  if (cudaHostRegister(map, len, cudaHostRegisterReadOnly) != cudaSuccess) {
    cudaGetLastError();
    ::munmap(map, len);
    ::close(fd);
    return BGPU_OK;
  }
  *refused = false;
  int rc = BGPU_OK;
  cudaError_t e = cudaStreamSynchronize(s);  // the caller's earlier work first
  for (int q = 0; q < 3 && e == cudaSuccess; ++q)
    if (ds[q]->num_bytes)
      e = cudaMemcpyAsync(dst[q], (const char*)map + (ds[q]->file_offset - start),
                          ds[q]->num_bytes, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    set_error(std::string("copying the mapped .h5ad data failed: ") + cudaGetErrorString(e));
    rc = BGPU_ERR_CUDA;
  }
  cudaHostUnregister(map);
  ::munmap(map, len);
  ::close(fd);
  return rc;
}

extern "C" int bgpu_h5ad_read(const char* path, const bgpu_h5ad_matrix* m, void* data,
                              void* indices, void* indptr, uint32_t method,
                              uint32_t num_threads, void* stream) {
  BGPU_REQUIRE(path && m, BGPU_ERR_INVALID, "h5ad: NULL argument");
  BGPU_REQUIRE(method <= BGPU_H5_READ_MAPPED, BGPU_ERR_INVALID, "h5ad: unknown read method");
  const bgpu_h5_dataset* ds[3] = {&m->data, &m->indices, &m->indptr};
  void* dst[3] = {data, indices, indptr};
  for (int q = 0; q < 3; ++q)
    BGPU_REQUIRE(ds[q]->num_bytes == 0 || dst[q], BGPU_ERR_INVALID,
                 "h5ad: NULL destination for a non-empty dataset");
  if (method != BGPU_H5_READ_STAGED) {
    bool refused = true;
    BGPU_TRY(read_mapped(path, ds, dst, (cudaStream_t)stream, &refused));
    if (!refused) return BGPU_OK;
    BGPU_REQUIRE(method != BGPU_H5_READ_MAPPED, BGPU_ERR_UNSUPPORTED,
                 "h5ad: the file cannot be mapped and registered with the driver here");
  }
  std::vector<Piece> pieces;
  for (int q = 0; q < 3; ++q) {
    for (uint64_t o = 0; o < ds[q]->num_bytes; o += kPiece)
      pieces.push_back({ds[q]->file_offset + o, std::min(kPiece, ds[q]->num_bytes - o),
                        (char*)dst[q] + o});
  }
  // larger datasets first interleaved by piece index: all threads busy to the end
  int threads = (int)(num_threads ? num_threads : std::thread::hardware_concurrency());
  threads = std::max(1, std::min(threads, kMaxThreads));
  threads = (int)std::min<uint64_t>((uint64_t)threads, std::max<size_t>(pieces.size(), 1));
  if (pieces.empty()) return BGPU_OK;
  return read_pieces(path, pieces, threads, (cudaStream_t)stream);
}
