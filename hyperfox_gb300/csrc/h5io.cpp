// HDF5 mesh and field files without the HDF5 library: a reader and a writer for
// the subset of the format that HDF5Io produces and consumes
// (src/io/HDF5Io.cpp:13-62 load, :64-109 write, :111-152 loadMesh,
// :154-191 loadFields, :193-304 writeMesh, :306-393 writeFields):
//
//   /Mesh/Nodes       float64 [nNodes][nodeDim]
//   /Mesh/Cells       int32   [nCells][nodesPerCell]
//   /FieldData/<name> float64 [nEntities][objsPerEntity][valsPerObj], int attribute "ftype"
//
// Reader: superblock version 0/1, version-1 object headers (with continuation
// blocks), groups as symbol tables (version-1 B-trees of symbol nodes plus a
// local heap) or as link messages, dataspace v1/v2, fixed-point and IEEE
// floating-point little-endian datatypes, contiguous and compact layouts
// (v1-v3), attribute messages v1-v3. Chunked or filtered datasets and the
// newer superblocks (v2/v3, "OHDR" headers, fractal heaps) are refused with a
// message naming what was found.
//
// Writer: the same on-disk forms the library writes with default properties
// (superblock v0, v1 object headers, symbol-table groups with a trailing free
// block in each local heap, contiguous datasets with dataspace, datatype,
// fill-value, layout and modification-time messages, the "ftype" attribute
// as a scalar 32-bit integer).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "hfx_gb300.h"

namespace hfx {
void set_io_error(const std::string& m);  // mesh_io.cpp

namespace {

constexpr uint64_t UNDEF = ~0ull;

struct H5Error {
  std::string msg;
};

[[noreturn]] void fail(const std::string& m) { throw H5Error{"hdf5: " + m}; }

// ------------------------------------------------------------------ reader
struct Reader {
  std::vector<uint8_t> d;
  int so = 8, sl = 8;  // sizes of offsets and lengths

  void need(uint64_t off, uint64_t n) const {
    if (off > d.size() || n > d.size() - off) fail("truncated file or bad address");
  }
  uint64_t u(uint64_t off, int n) const {
    need(off, (uint64_t)n);
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)d[off + i] << (8 * i);
    return v;
  }
  uint64_t addr(uint64_t off) const {
    uint64_t v = u(off, so);
    if (so < 8 && v == (1ull << (8 * so)) - 1) return UNDEF;
    return v;
  }
  bool sig(uint64_t off, const char* s) const {
    need(off, 4);
    return std::memcmp(&d[off], s, 4) == 0;
  }

  struct Msg {
    int type;
    uint64_t body, size;
  };
  struct Dataset {
    std::vector<uint64_t> dims;
    int tclass = -1, tsize = 0;
    bool tsigned = false;
    int layoutClass = -1;  // 0 compact, 1 contiguous, 2 chunked
    uint64_t dataAddr = UNDEF, dataSize = 0;
    bool filtered = false;
  };

  uint64_t rootHeader = UNDEF;

  void open(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) fail("cannot open " + path);
    d.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    // the signature may sit at 0, 512, 1024, ... (user block)
    static const uint8_t S[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    uint64_t base = UNDEF;
    for (uint64_t o = 0; o + 8 <= d.size(); o = o ? o * 2 : 512)
      if (std::memcmp(&d[o], S, 8) == 0) {
        base = o;
        break;
      }
    if (base == UNDEF) fail(path + " is not an HDF5 file");
    const int ver = (int)u(base + 8, 1);
    if (ver > 1)
      fail("superblock version " + std::to_string(ver) +
           " is not read (files written with the library's default settings use version 0)");
    so = (int)u(base + 13, 1);
    sl = (int)u(base + 14, 1);
    if ((so != 4 && so != 8) || (sl != 4 && sl != 8)) fail("unsupported offset/length sizes");
    uint64_t p = base + 24 + (ver == 1 ? 4 : 0);
    const uint64_t baseAddr = addr(p);
    if (baseAddr != base && baseAddr != 0) fail("unexpected base address");
    p += 4 * (uint64_t)so;  // base, free-space, end-of-file, driver-info addresses
    rootHeader = addr(p + so);  // root symbol table entry: link-name offset, header address
    if (base != 0) fail("files with a user block are not read");
  }

  std::vector<Msg> messages(uint64_t oh) const {
    need(oh, 16);
    if (sig(oh, "OHDR")) fail("version-2 object headers are not read");
    if (d[oh] != 1) fail("unknown object header version " + std::to_string(d[oh]));
    const uint64_t nmsg = u(oh + 2, 2);
    const uint64_t size = u(oh + 8, 4);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{oh + 16, size}};
    std::vector<Msg> out;
    for (size_t b = 0; b < blocks.size() && out.size() < nmsg; ++b) {
      uint64_t p = blocks[b].first;
      const uint64_t end = p + blocks[b].second;
      need(blocks[b].first, blocks[b].second);
      while (p + 8 <= end && out.size() < nmsg) {
        Msg m{(int)u(p, 2), p + 8, u(p + 2, 2)};
        if (m.body + m.size > end) fail("object header message overruns its block");
        out.push_back(m);
        if (m.type == 0x10) blocks.push_back({addr(m.body), u(m.body + so, sl)});
        if (blocks.size() > 4096) fail("too many continuation blocks");
        p = m.body + m.size;
      }
    }
    return out;
  }

  std::string heap_name(uint64_t heap, uint64_t off) const {
    if (!sig(heap, "HEAP")) fail("bad local heap signature");
    const uint64_t dsize = u(heap + 8, sl);
    const uint64_t dseg = addr(heap + 8 + 2 * (uint64_t)sl);
    if (off >= dsize) fail("name offset outside the local heap");
    need(dseg, dsize);
    std::string s;
    for (uint64_t i = dseg + off; i < dseg + dsize && d[i]; ++i) s.push_back((char)d[i]);
    return s;
  }

  // name -> object header address of every link in a group
  std::map<std::string, uint64_t> links(uint64_t oh) const {
    std::map<std::string, uint64_t> out;
    for (const Msg& m : messages(oh)) {
      if (m.type == 0x11) {
        const uint64_t btree = addr(m.body), heap = addr(m.body + so);
        walk_btree(btree, heap, &out, 0);
      } else if (m.type == 0x06) {
        read_link(m, &out);
      } else if (m.type == 0x02) {
        fail("groups with dense link storage are not read");
      }
    }
    return out;
  }

  void walk_btree(uint64_t node, uint64_t heap, std::map<std::string, uint64_t>* out, int depth) const {
    if (depth > 64) fail("group B-tree too deep");
    if (!sig(node, "TREE")) fail("bad group B-tree signature");
    if (u(node + 4, 1) != 0) fail("group B-tree of the wrong node type");
    const int level = (int)u(node + 5, 1);
    const uint64_t used = u(node + 6, 2);
    uint64_t p = node + 8 + 2 * (uint64_t)so + sl;  // after left/right siblings and key 0
    for (uint64_t i = 0; i < used; ++i) {
      const uint64_t child = addr(p);
      p += so + sl;
      if (level > 0) {
        walk_btree(child, heap, out, depth + 1);
      } else {
        if (!sig(child, "SNOD")) fail("bad symbol node signature");
        const uint64_t ns = u(child + 6, 2);
        const uint64_t esz = 2 * (uint64_t)so + 4 + 4 + 16;
        for (uint64_t k = 0; k < ns; ++k) {
          const uint64_t e = child + 8 + k * esz;
          (*out)[heap_name(heap, u(e, so))] = addr(e + so);
        }
      }
    }
  }

  void read_link(const Msg& m, std::map<std::string, uint64_t>* out) const {
    uint64_t p = m.body;
    if (u(p, 1) != 1) fail("unknown link message version");
    const int flags = (int)u(p + 1, 1);
    p += 2;
    int ltype = 0;
    if (flags & 0x8) ltype = (int)u(p++, 1);
    if (flags & 0x4) p += 8;
    if (flags & 0x10) p += 1;
    const int lsz = 1 << (flags & 3);
    const uint64_t nlen = u(p, lsz);
    p += lsz;
    need(p, nlen);
    std::string name((const char*)&d[p], (size_t)nlen);
    p += nlen;
    if (ltype == 0) (*out)[name] = addr(p);
  }

  uint64_t resolve(const std::string& path) const {
    uint64_t oh = rootHeader;
    size_t s = 0;
    while (s < path.size()) {
      size_t e = path.find('/', s);
      if (e == std::string::npos) e = path.size();
      if (e > s) {
        auto ls = links(oh);
        auto it = ls.find(path.substr(s, e - s));
        if (it == ls.end()) return UNDEF;
        oh = it->second;
      }
      s = e + 1;
    }
    return oh;
  }

  void parse_type(uint64_t b, int* cls, int* size, bool* sgn) const {
    const int cv = (int)u(b, 1);
    *cls = cv & 15;
    const uint64_t bits = u(b + 1, 3);
    *size = (int)u(b + 4, 4);
    if (*cls != 0 && *cls != 1) fail("datatype class " + std::to_string(*cls) + " is not read (integers and floats only)");
    if (bits & 1) fail("big-endian data is not read");
    *sgn = *cls == 0 ? (bits & 8) != 0 : true;
    if (*cls == 1 && *size != 4 && *size != 8) fail("floating-point size " + std::to_string(*size));
    if (*cls == 0 && *size != 1 && *size != 2 && *size != 4 && *size != 8)
      fail("integer size " + std::to_string(*size));
  }

  std::vector<uint64_t> parse_space(uint64_t b) const {
    const int v = (int)u(b, 1), nd = (int)u(b + 1, 1);
    std::vector<uint64_t> dims(nd);
    uint64_t p;
    if (v == 1) p = b + 8;
    else if (v == 2) {
      if (u(b + 3, 1) == 2) return {0};  // null dataspace
      p = b + 4;
    } else fail("dataspace version " + std::to_string(v));
    for (int i = 0; i < nd; ++i) dims[i] = u(p + (uint64_t)i * sl, sl);
    return dims;
  }

  Dataset dataset(uint64_t oh) const {
    Dataset ds;
    bool haveSpace = false;
    for (const Msg& m : messages(oh)) {
      if (m.type == 0x01) {
        ds.dims = parse_space(m.body);
        haveSpace = true;
      } else if (m.type == 0x03) {
        parse_type(m.body, &ds.tclass, &ds.tsize, &ds.tsigned);
      } else if (m.type == 0x0B) {
        ds.filtered = true;
      } else if (m.type == 0x08) {
        const int v = (int)u(m.body, 1);
        if (v == 3) {
          ds.layoutClass = (int)u(m.body + 1, 1);
          if (ds.layoutClass == 0) {
            ds.dataSize = u(m.body + 2, 2);
            ds.dataAddr = m.body + 4;
          } else if (ds.layoutClass == 1) {
            ds.dataAddr = addr(m.body + 2);
            ds.dataSize = u(m.body + 2 + so, sl);
          }
        } else if (v == 1 || v == 2) {
          const int nd = (int)u(m.body + 1, 1);
          ds.layoutClass = (int)u(m.body + 2, 1);
          uint64_t p = m.body + 8;
          if (ds.layoutClass != 0) {
            ds.dataAddr = addr(p);
            p += so;
          }
          p += 4 * (uint64_t)nd;
          if (ds.layoutClass == 0) {
            ds.dataSize = u(p, 4);
            ds.dataAddr = p + 4;
          } else if (ds.layoutClass == 1) {
            ds.dataSize = UNDEF;  // implied by the dataspace
          }
        } else {
          fail("layout version " + std::to_string(v));
        }
      }
    }
    if (!haveSpace || ds.tclass < 0 || ds.layoutClass < 0) fail("object is not a dataset");
    if (ds.layoutClass == 2) fail("chunked datasets are not read");
    if (ds.filtered) fail("filtered datasets are not read");
    return ds;
  }

  static uint64_t count(const std::vector<uint64_t>& dims) {
    uint64_t n = 1;
    for (uint64_t v : dims) {
      if (v && n > UNDEF / v) fail("dataset too large");
      n *= v;
    }
    return n;
  }

  // element i of raw storage at p, converted to T
  template <typename T>
  T element(uint64_t p, int cls, int size, bool sgn) const {
    if (cls == 1) {
      if (size == 8) {
        uint64_t v = u(p, 8);
        double x;
        std::memcpy(&x, &v, 8);
        return (T)x;
      }
      uint32_t v = (uint32_t)u(p, 4);
      float x;
      std::memcpy(&x, &v, 4);
      return (T)x;
    }
    uint64_t v = u(p, size);
    if (sgn && size < 8 && (v >> (8 * size - 1)) & 1) v |= ~0ull << (8 * size);
    return sgn ? (T)(int64_t)v : (T)v;
  }

  template <typename T>
  void read(const Dataset& ds, T* out) const {
    const uint64_t n = count(ds.dims);
    const uint64_t bytes = n * (uint64_t)ds.tsize;
    if (ds.dataAddr == UNDEF) {  // never written: the default fill value
      std::fill(out, out + n, (T)0);
      return;
    }
    if (ds.dataSize != UNDEF && ds.dataSize < bytes) fail("dataset storage smaller than its dataspace");
    need(ds.dataAddr, bytes);
    for (uint64_t i = 0; i < n; ++i) out[i] = element<T>(ds.dataAddr + i * ds.tsize, ds.tclass, ds.tsize, ds.tsigned);
  }

  // integer attribute `name` of the object at oh; false when absent
  bool int_attribute(uint64_t oh, const std::string& name, int64_t* value) const {
    for (const Msg& m : messages(oh)) {
      if (m.type != 0x0C) continue;
      const int v = (int)u(m.body, 1);
      const uint64_t nlen = u(m.body + 2, 2), tlen = u(m.body + 4, 2), slen = u(m.body + 6, 2);
      uint64_t p = m.body + (v == 3 ? 9 : 8);
      auto pad = [&](uint64_t x) { return v == 1 ? (x + 7) / 8 * 8 : x; };
      need(p, nlen);
      std::string an;
      for (uint64_t i = 0; i < nlen && d[p + i]; ++i) an.push_back((char)d[p + i]);
      p += pad(nlen);
      const uint64_t tp = p;
      p += pad(tlen);
      p += pad(slen);
      if (an != name) continue;
      int cls, size;
      bool sgn;
      parse_type(tp, &cls, &size, &sgn);
      *value = element<int64_t>(p, cls, size, sgn);
      return true;
    }
    return false;
  }
};

// ------------------------------------------------------------------ writer
struct Writer {
  std::vector<uint8_t> b;
  uint64_t pos() const { return b.size(); }
  void put(uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b.push_back((uint8_t)(v >> (8 * i)));
  }
  void patch(uint64_t at, uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b[at + i] = (uint8_t)(v >> (8 * i));
  }
  void bytes(const void* p, size_t n) {
    const uint8_t* c = (const uint8_t*)p;
    b.insert(b.end(), c, c + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void align8() { zeros((8 - b.size() % 8) % 8); }
};

constexpr int K_LEAF = 4, K_INTERNAL = 16;  // group B-tree and symbol node capacities

struct Child {
  std::string name;
  uint64_t header;
  bool group;
  uint64_t btree = 0, heap = 0;  // cached in the symbol table entry of a group
};

// v1 object header prefix; returns the offset of the header-size field
uint64_t header_prefix(Writer& w, int nmsg) {
  w.put(1, 1);
  w.put(0, 1);
  w.put(nmsg, 2);
  w.put(1, 4);
  const uint64_t at = w.pos();
  w.put(0, 4);
  w.put(0, 4);
  return at;
}

void msg_header(Writer& w, int type, int size, int flags) {
  w.put(type, 2);
  w.put(size, 2);
  w.put(flags, 1);
  w.zeros(3);
}

// a group: object header with a symbol table message, a B-tree of symbol
// nodes and a local heap holding the names; returns the header address
struct GroupAddr {
  uint64_t header, btree, heap;
};

GroupAddr write_group(Writer& w, std::vector<Child> kids) {
  std::sort(kids.begin(), kids.end(), [](const Child& a, const Child& c) { return a.name < c.name; });
  const size_t perNode = 2 * K_LEAF;
  const size_t nNodes = std::max<size_t>(1, (kids.size() + perNode - 1) / perNode);
  if (nNodes > 2 * (size_t)K_INTERNAL) fail("more than 256 entries in one group");
  GroupAddr g;
  // object header
  g.header = w.pos();
  const uint64_t hs = header_prefix(w, 1);
  msg_header(w, 0x11, 16, 0);
  const uint64_t stAt = w.pos();
  w.put(0, 8);
  w.put(0, 8);
  w.patch(hs, w.pos() - (hs + 8), 4);
  // local heap: "" at 0, the names, then one free block (next = 1 ends the list)
  std::vector<uint64_t> nameOff(kids.size());
  std::vector<uint8_t> seg(8, 0);
  for (size_t i = 0; i < kids.size(); ++i) {
    nameOff[i] = seg.size();
    seg.insert(seg.end(), kids[i].name.begin(), kids[i].name.end());
    seg.push_back(0);
    while (seg.size() % 8) seg.push_back(0);
  }
  const uint64_t freeOff = seg.size();
  const uint64_t freeSize = 16 + 8 * 8;
  seg.resize(seg.size() + freeSize, 0);
  for (int i = 0; i < 8; ++i) {
    seg[freeOff + i] = (uint8_t)((1ull >> (8 * i)) & 0xff);
    seg[freeOff + 8 + i] = (uint8_t)((freeSize >> (8 * i)) & 0xff);
  }
  g.heap = w.pos();
  w.bytes("HEAP", 4);
  w.put(0, 1);
  w.zeros(3);
  w.put(seg.size(), 8);
  w.put(freeOff, 8);
  w.put(w.pos() + 8, 8);  // the data segment follows this field
  w.bytes(seg.data(), seg.size());
  // symbol nodes
  std::vector<uint64_t> snod(nNodes);
  for (size_t n = 0; n < nNodes; ++n) {
    snod[n] = w.pos();
    const size_t lo = n * perNode, hi = std::min(kids.size(), lo + perNode);
    w.bytes("SNOD", 4);
    w.put(1, 1);
    w.put(0, 1);
    w.put(hi - lo, 2);
    for (size_t i = lo; i < hi; ++i) {
      w.put(nameOff[i], 8);
      w.put(kids[i].header, 8);
      w.put(kids[i].group ? 1 : 0, 4);
      w.put(0, 4);
      if (kids[i].group) {
        w.put(kids[i].btree, 8);
        w.put(kids[i].heap, 8);
      } else {
        w.zeros(16);
      }
    }
    w.zeros((perNode - (hi - lo)) * 40);
  }
  // B-tree node (level 0), sized for 2K children like the library's
  g.btree = w.pos();
  w.bytes("TREE", 4);
  w.put(0, 1);
  w.put(0, 1);
  w.put(kids.empty() ? 0 : nNodes, 2);
  w.put(UNDEF, 8);
  w.put(UNDEF, 8);
  w.put(0, 8);  // key 0: the empty name
  size_t written = 0;
  if (!kids.empty())
    for (size_t n = 0; n < nNodes; ++n) {
      const size_t hi = std::min(kids.size(), (n + 1) * perNode);
      w.put(snod[n], 8);
      w.put(nameOff[hi - 1], 8);  // key n+1: the last name under child n
      ++written;
    }
  w.zeros((2 * K_INTERNAL - written) * 16);
  w.patch(stAt, g.btree, 8);
  w.patch(stAt + 8, g.heap, 8);
  return g;
}

void put_space(Writer& w, const std::vector<uint64_t>& dims) {
  w.put(1, 1);
  w.put(dims.size(), 1);
  w.put(1, 1);  // maximum dimensions present (equal to the current ones)
  w.zeros(5);
  for (uint64_t v : dims) w.put(v, 8);
  for (uint64_t v : dims) w.put(v, 8);
}

void put_type_f64(Writer& w) {
  w.put(0x11, 1);  // version 1, floating point
  w.put(0x20, 1);  // little endian, implied mantissa msb
  w.put(63, 1);    // sign bit position
  w.put(0, 1);
  w.put(8, 4);
  w.put(0, 2);   // bit offset
  w.put(64, 2);  // precision
  w.put(52, 1);  // exponent location
  w.put(11, 1);  // exponent size
  w.put(0, 1);   // mantissa location
  w.put(52, 1);  // mantissa size
  w.put(1023, 4);
}

void put_type_i32(Writer& w) {
  w.put(0x10, 1);  // version 1, fixed point
  w.put(0x08, 1);  // little endian, signed
  w.put(0, 2);
  w.put(4, 4);
  w.put(0, 2);
  w.put(32, 2);
}

// contiguous dataset with an optional scalar int32 attribute; returns the header address
uint64_t write_dataset(Writer& w, const std::vector<uint64_t>& dims, bool isDouble, const void* data,
                       const char* attrName, int attrValue) {
  const uint64_t nelem = Reader::count(dims);
  const uint64_t bytes = nelem * (isDouble ? 8 : 4);
  const uint64_t h = w.pos();
  const int nmsg = attrName ? 6 : 5;
  const uint64_t hs = header_prefix(w, nmsg);
  const int spaceSize = 8 + 16 * (int)dims.size();
  msg_header(w, 0x01, spaceSize, 0);
  put_space(w, dims);
  msg_header(w, 0x03, isDouble ? 24 : 16, 1);
  const uint64_t t0 = w.pos();
  if (isDouble) put_type_f64(w);
  else put_type_i32(w);
  w.zeros((isDouble ? 24 : 16) - (w.pos() - t0));
  msg_header(w, 0x05, 8, 1);  // fill value v2: late allocation, fill if set, default value
  w.put(2, 1);
  w.put(2, 1);
  w.put(2, 1);
  w.put(1, 1);
  w.put(0, 4);
  msg_header(w, 0x08, 24, 0);
  w.put(3, 1);
  w.put(1, 1);
  const uint64_t addrAt = w.pos();
  w.put(0, 8);
  w.put(bytes, 8);
  w.zeros(6);
  msg_header(w, 0x12, 8, 0);
  w.put(1, 1);
  w.zeros(3);
  w.put((uint64_t)std::time(nullptr) & 0xffffffffull, 4);
  if (attrName) {
    const size_t nlen = std::strlen(attrName) + 1;
    const size_t npad = (nlen + 7) / 8 * 8;
    msg_header(w, 0x0C, (int)(8 + npad + 16 + 8 + 8), 0);
    w.put(1, 1);
    w.put(0, 1);
    w.put(nlen, 2);
    w.put(12, 2);
    w.put(8, 2);
    w.bytes(attrName, nlen);
    w.zeros(npad - nlen);
    put_type_i32(w);
    w.zeros(4);
    w.put(1, 1);  // scalar dataspace (version 1, rank 0)
    w.zeros(7);
    w.put((uint32_t)attrValue, 4);
    w.zeros(4);
  }
  w.patch(hs, w.pos() - (hs + 8), 4);
  w.patch(addrAt, w.pos(), 8);
  w.bytes(data, bytes);
  w.align8();
  return h;
}

struct FieldIn {
  std::string name;
  int ftype;
  std::vector<uint64_t> shape;
  const double* values;
};

std::vector<uint8_t> write_file(int nodeDim, int nNodes, const double* coords, int nCells, int nodesPerCell,
                                const int* cells, const std::vector<FieldIn>& fields) {
  Writer w;
  // superblock v0 (root entry patched at the end)
  static const uint8_t S[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  w.bytes(S, 8);
  w.put(0, 1);  // superblock version
  w.put(0, 1);  // free-space version
  w.put(0, 1);  // root group symbol table entry version
  w.put(0, 1);
  w.put(0, 1);  // shared header message format version
  w.put(8, 1);  // size of offsets
  w.put(8, 1);  // size of lengths
  w.put(0, 1);
  w.put(K_LEAF, 2);
  w.put(K_INTERNAL, 2);
  w.put(0, 4);      // file consistency flags
  w.put(0, 8);      // base address
  w.put(UNDEF, 8);  // free-space info
  const uint64_t eofAt = w.pos();
  w.put(0, 8);
  w.put(UNDEF, 8);  // driver information block
  const uint64_t rootAt = w.pos();
  w.zeros(40);
  std::vector<Child> top;
  if (nNodes > 0 && nCells > 0) {
    std::vector<Child> mesh;
    mesh.push_back({"Nodes", write_dataset(w, {(uint64_t)nNodes, (uint64_t)nodeDim}, true, coords, nullptr, 0), false});
    mesh.push_back(
        {"Cells", write_dataset(w, {(uint64_t)nCells, (uint64_t)nodesPerCell}, false, cells, nullptr, 0), false});
    GroupAddr g = write_group(w, mesh);
    top.push_back({"Mesh", g.header, true, g.btree, g.heap});
  }
  if (!fields.empty()) {
    std::vector<Child> fd;
    for (const FieldIn& f : fields)
      fd.push_back({f.name, write_dataset(w, f.shape, true, f.values, "ftype", f.ftype), false});
    GroupAddr g = write_group(w, fd);
    top.push_back({"FieldData", g.header, true, g.btree, g.heap});
  }
  if (top.empty()) fail("nothing to write (no mesh and no field)");
  GroupAddr root = write_group(w, top);
  w.patch(rootAt, 0, 8);  // link name offset
  w.patch(rootAt + 8, root.header, 8);
  w.patch(rootAt + 16, 1, 4);  // cache type: group
  w.patch(rootAt + 24, root.btree, 8);
  w.patch(rootAt + 32, root.heap, 8);
  w.patch(eofAt, w.pos(), 8);
  return w.b;
}

int run(const std::function<void()>& f) {
  try {
    f();
  } catch (const H5Error& e) {
    set_io_error(e.msg);
    return HFX_ERR_ARG;
  } catch (const std::bad_alloc&) {
    set_io_error("hdf5: out of host memory");
    return HFX_ERR_ARG;
  }
  return HFX_OK;
}

}  // namespace
}  // namespace hfx

using namespace hfx;

extern "C" {

int hfx_h5_read_mesh(const char* path, int* nodeDim, int* nNodes, int* nCells, int* nodesPerCell, double* coords,
                     int* cells) {
  if (!path || !nodeDim || !nNodes || !nCells || !nodesPerCell) return HFX_ERR_ARG;
  return run([&] {
    Reader r;
    r.open(path);
    const uint64_t n = r.resolve("Mesh/Nodes"), c = r.resolve("Mesh/Cells");
    if (n == UNDEF || c == UNDEF) fail(std::string(path) + " has no /Mesh/Nodes and /Mesh/Cells");
    Reader::Dataset dn = r.dataset(n), dc = r.dataset(c);
    if (dn.dims.size() != 2 || dc.dims.size() != 2) fail("Nodes and Cells must be two-dimensional");
    if (dn.dims[0] > INT32_MAX || dc.dims[0] > INT32_MAX || dn.dims[1] > 3 || dc.dims[1] > 4096)
      fail("mesh sizes out of range");
    *nodeDim = (int)dn.dims[1];
    *nNodes = (int)dn.dims[0];
    *nCells = (int)dc.dims[0];
    *nodesPerCell = (int)dc.dims[1];
    if (coords) r.read<double>(dn, coords);
    if (cells) {
      r.read<int>(dc, cells);
      for (uint64_t i = 0; i < dc.dims[0] * dc.dims[1]; ++i)
        if (cells[i] < 0 || cells[i] >= *nNodes) fail("cell refers to a node outside Nodes");
    }
  });
}

int hfx_h5_field_names(const char* path, char* buf, int bufLen, int* nFields, int* needLen) {
  if (!path || !nFields) return HFX_ERR_ARG;
  return run([&] {
    Reader r;
    r.open(path);
    const uint64_t g = r.resolve("FieldData");
    std::string all;
    int n = 0;
    if (g != UNDEF)
      for (auto& kv : r.links(g)) {
        all += kv.first;
        all.push_back('\n');
        ++n;
      }
    *nFields = n;
    if (needLen) *needLen = (int)all.size() + 1;
    if (buf && bufLen > 0) {
      const size_t k = std::min(all.size(), (size_t)bufLen - 1);
      std::memcpy(buf, all.data(), k);
      buf[k] = 0;
    }
  });
}

int hfx_h5_read_field(const char* path, const char* name, int* ftype, int64_t* shape, double* values) {
  if (!path || !name || !ftype || !shape) return HFX_ERR_ARG;
  return run([&] {
    Reader r;
    r.open(path);
    const uint64_t f = r.resolve(std::string("FieldData/") + name);
    if (f == UNDEF) fail(std::string("field ") + name + " was not found in FieldData");
    Reader::Dataset ds = r.dataset(f);
    if (ds.dims.size() != 3) fail(std::string("field ") + name + " is not three-dimensional");
    int64_t ft = -1;
    if (!r.int_attribute(f, "ftype", &ft)) fail(std::string("attribute ftype could not be found for field: ") + name);
    *ftype = (int)ft;
    for (int i = 0; i < 3; ++i) shape[i] = (int64_t)ds.dims[i];
    if (values) r.read<double>(ds, values);
  });
}

int hfx_h5_write(const char* path, int nodeDim, int nNodes, const double* coords, int nCells, int nodesPerCell,
                 const int* cells, int nFields, const char* const* names, const int* ftypes, const int64_t* shapes,
                 const double* const* values) {
  if (!path || nFields < 0 || (nFields > 0 && (!names || !ftypes || !shapes || !values))) return HFX_ERR_ARG;
  if (nNodes > 0 && (!coords || !cells || nCells <= 0 || nodeDim < 1 || nodeDim > 3 || nodesPerCell < 1))
    return HFX_ERR_ARG;
  return run([&] {
    std::vector<FieldIn> fs;
    for (int i = 0; i < nFields; ++i) {
      if (!names[i] || !*names[i] || std::strchr(names[i], '/')) fail("bad field name");
      for (int k = 0; k < 3; ++k)
        if (shapes[3 * i + k] < 0) fail("negative field shape");
      fs.push_back({names[i], ftypes[i],
                    {(uint64_t)shapes[3 * i], (uint64_t)shapes[3 * i + 1], (uint64_t)shapes[3 * i + 2]}, values[i]});
    }
    std::vector<uint8_t> bytes = write_file(nodeDim, nNodes, coords, nCells, nodesPerCell, cells, fs);
    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    if (!out) fail(std::string("cannot create ") + path);
    out.write((const char*)bytes.data(), (std::streamsize)bytes.size());
    if (!out) fail(std::string("write failed: ") + path);
  });
}

}  // extern "C"
