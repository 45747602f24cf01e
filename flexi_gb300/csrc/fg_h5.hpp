// flexi_gb300 -- the subset of the HDF5 file format that FLEXI's mesh and state files use, without the
// HDF5 library (absent from this toolchain): superblock version 0/1 (after an optional user block, as
// FLEXI's state files carry one), version-1 object headers with continuation blocks, groups as symbol
// tables (version-1 B-tree of SNOD nodes + local heap), datasets with version-1/2 dataspaces and
// contiguous or compact layout, little-endian fixed-point (4/8 byte) and IEEE floating-point (8 byte)
// data, fixed-length strings, and attributes (message versions 1-3). Everything else (chunked or
// filtered storage, superblock 2/3, version-2 object headers, variable-length types) is rejected with a
// message naming it. The writer produces files of the same subset (superblock 0, root group of
// contiguous datasets and attributes).
//
// Layouts follow the published HDF5 File Format Specification (version 0 superblock, symbol table
// entry, local heap, v1 B-tree, symbol table node, object header v1, dataspace/datatype/fill value/
// data layout/attribute/continuation/symbol table messages).
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace fgh5 {

struct Type {
  int cls = -1;      // 0 fixed-point, 1 floating point, 3 string
  int size = 0;      // bytes per element
  bool sign = true;  // fixed-point: signed
};

struct Dataset {
  std::vector<uint64_t> dims;  // C order (the Fortran dimensions reversed)
  Type type;
  uint64_t addr = 0;           // contiguous data (relative to the superblock)
  std::vector<uint8_t> compact;
  bool isCompact = false;
  uint64_t count() const {
    uint64_t c = 1;
    for (uint64_t d : dims) c *= d;
    return c;
  }
};

class Reader {
 public:
  explicit Reader(const std::string& path) : path_(path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<uint8_t> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    size_t off = 0;
    // the superblock sits at 0, 512, 1024, 2048, ... (after a user block)
    while (off + 8 <= raw.size() && std::memcmp(raw.data() + off, sig, 8) != 0) off = off == 0 ? 512 : off * 2;
    if (off + 8 > raw.size()) throw std::runtime_error(path + ": not an HDF5 file");
    b_.assign(raw.begin() + (long)off, raw.end());
    const int ver = u8(8);
    if (ver != 0 && ver != 1) throw std::runtime_error(path + ": HDF5 superblock version " + std::to_string(ver) + " is not supported");
    if (u8(13) != 8 || u8(14) != 8) throw std::runtime_error(path + ": only 8-byte offsets and lengths are supported");
    size_t p = ver == 1 ? 28 : 24;
    p += 32;  // base, free-space, end-of-file and driver-block addresses
    root_ = u64(p + 8);  // root group symbol table entry: object header address
  }

  // datasets and groups of the root group: name -> object header address
  std::map<std::string, uint64_t> children() const {
    std::map<std::string, uint64_t> out;
    for (const Msg& m : messages(root_))
      if (m.type == 0x11) group_entries(u64(m.body), u64(m.body + 8), out);
    return out;
  }
  bool has(const std::string& name) const { return children().count(name) != 0; }

  Dataset dataset(const std::string& name) const {
    auto c = children();
    auto it = c.find(name);
    if (it == c.end()) throw std::runtime_error(path_ + ": no dataset '" + name + "'");
    Dataset d;
    bool haveLayout = false;
    for (const Msg& m : messages(it->second)) {
      if (m.type == 0x1) d.dims = dataspace(m.body);
      else if (m.type == 0x3) d.type = datatype(m.body);
      else if (m.type == 0xB) throw std::runtime_error(path_ + ": '" + name + "' uses filters (compression), not supported");
      else if (m.type == 0x8) { layout(m.body, d); haveLayout = true; }
    }
    if (!haveLayout || d.type.cls < 0) throw std::runtime_error(path_ + ": '" + name + "' is not a dataset");
    return d;
  }

  std::vector<long long> read_int(const std::string& name, std::vector<uint64_t>* dims = nullptr) const {
    const Dataset d = dataset(name);
    if (dims) *dims = d.dims;
    return ints(d.type, data(d), d.count(), name);
  }
  std::vector<double> read_real(const std::string& name, std::vector<uint64_t>* dims = nullptr) const {
    const Dataset d = dataset(name);
    if (dims) *dims = d.dims;
    return reals(d.type, data(d), d.count(), name);
  }
  std::vector<std::string> read_str(const std::string& name) const {
    const Dataset d = dataset(name);
    return strs(d.type, data(d), d.count(), name);
  }

  // attributes of the root group
  bool attr_int(const std::string& name, long long& v) const {
    Attr a;
    if (!attribute(name, a)) return false;
    v = ints(a.type, a.data, 1, name).at(0);
    return true;
  }
  bool attr_real(const std::string& name, double& v) const {
    Attr a;
    if (!attribute(name, a)) return false;
    v = reals(a.type, a.data, 1, name).at(0);
    return true;
  }
  bool attr_str(const std::string& name, std::vector<std::string>& v) const {
    Attr a;
    if (!attribute(name, a)) return false;
    uint64_t n = 1;
    for (uint64_t x : a.dims) n *= x;
    v = strs(a.type, a.data, n, name);
    return true;
  }

 private:
  struct Msg { uint16_t type; size_t body; size_t size; };
  struct Attr { Type type; std::vector<uint64_t> dims; const uint8_t* data = nullptr; };
  std::string path_;
  std::vector<uint8_t> b_;
  uint64_t root_ = 0;

  void need(size_t p, size_t n) const {
    if (p > b_.size() || n > b_.size() - p) throw std::runtime_error(path_ + ": truncated or corrupt HDF5 structure");
  }
  uint8_t u8(size_t p) const { need(p, 1); return b_[p]; }
  uint16_t u16(size_t p) const { need(p, 2); return (uint16_t)(b_[p] | (b_[p + 1] << 8)); }
  uint32_t u32(size_t p) const { need(p, 4); uint32_t v; std::memcpy(&v, &b_[p], 4); return v; }
  uint64_t u64(size_t p) const { need(p, 8); uint64_t v; std::memcpy(&v, &b_[p], 8); return v; }
  static bool undef(uint64_t a) { return a == ~0ull; }

  std::vector<Msg> messages(uint64_t addr) const {
    if (u8(addr) != 1) throw std::runtime_error(path_ + ": object header version " + std::to_string(u8(addr)) + " is not supported");
    const int nmsg = u16(addr + 2);
    std::vector<Msg> out;
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, u32(addr + 8)}};
    for (size_t bi = 0; bi < blocks.size() && (int)out.size() < nmsg; ++bi) {
      size_t p = blocks[bi].first;
      const size_t end = p + blocks[bi].second;
      need(p, blocks[bi].second);
      while (p + 8 <= end && (int)out.size() < nmsg) {
        Msg m{u16(p), p + 8, u16(p + 2)};
        need(m.body, m.size);
        out.push_back(m);
        if (m.type == 0x10) blocks.push_back({u64(m.body), u64(m.body + 8)});
        p = m.body + m.size;
      }
      if (blocks.size() > 4096) throw std::runtime_error(path_ + ": corrupt object header");
    }
    return out;
  }
  std::string heap_name(uint64_t heap, uint64_t off) const {
    need(heap, 32);
    if (std::memcmp(&b_[heap], "HEAP", 4) != 0) throw std::runtime_error(path_ + ": bad local heap");
    const uint64_t data = u64(heap + 24);
    size_t p = data + off;
    std::string s;
    while (u8(p) != 0) s += (char)b_[p++];
    return s;
  }
  void group_entries(uint64_t btree, uint64_t heap, std::map<std::string, uint64_t>& out, int depth = 0) const {
    if (depth > 64) throw std::runtime_error(path_ + ": corrupt group B-tree");
    need(btree, 24);
    if (std::memcmp(&b_[btree], "TREE", 4) != 0 || u8(btree + 4) != 0) throw std::runtime_error(path_ + ": bad group B-tree");
    const int level = u8(btree + 5), used = u16(btree + 6);
    size_t p = btree + 24 + 8;  // skip key 0
    for (int i = 0; i < used; ++i, p += 16) {
      const uint64_t child = u64(p);
      if (level > 0) { group_entries(child, heap, out, depth + 1); continue; }
      need(child, 8);
      if (std::memcmp(&b_[child], "SNOD", 4) != 0) throw std::runtime_error(path_ + ": bad symbol table node");
      const int nsym = u16(child + 6);
      for (int k = 0; k < nsym; ++k) {
        const size_t q = child + 8 + (size_t)k * 40;
        out[heap_name(heap, u64(q))] = u64(q + 8);
      }
    }
  }
  std::vector<uint64_t> dataspace(size_t p) const {
    const int ver = u8(p), nd = u8(p + 1);
    if (ver != 1 && ver != 2) throw std::runtime_error(path_ + ": dataspace version " + std::to_string(ver));
    if (ver == 2 && u8(p + 3) == 2) return {0};  // null dataspace
    std::vector<uint64_t> dims(nd);
    const size_t q = p + (ver == 1 ? 8 : 4);
    for (int i = 0; i < nd; ++i) dims[i] = u64(q + 8 * (size_t)i);
    return dims;  // rank 0: scalar
  }
  Type datatype(size_t p) const {
    Type t;
    t.cls = u8(p) & 15;
    t.size = (int)u32(p + 4);
    const int bits = u8(p + 1);
    if (t.cls == 0) {
      if (bits & 1) throw std::runtime_error(path_ + ": big-endian integers are not supported");
      t.sign = (bits & 8) != 0;
    } else if (t.cls == 1) {
      if ((bits & 1) || (bits & 0x40)) throw std::runtime_error(path_ + ": big-endian or VAX floats are not supported");
    } else if (t.cls != 3) {
      throw std::runtime_error(path_ + ": datatype class " + std::to_string(t.cls) + " is not supported");
    }
    return t;
  }
  void layout(size_t p, Dataset& d) const {
    const int ver = u8(p);
    if (ver == 3) {
      const int cls = u8(p + 1);
      if (cls == 0) {
        const int n = u16(p + 2);
        need(p + 4, n);
        d.isCompact = true;
        d.compact.assign(b_.begin() + (long)(p + 4), b_.begin() + (long)(p + 4 + n));
      } else if (cls == 1) {
        d.addr = u64(p + 2);
      } else {
        throw std::runtime_error(path_ + ": chunked datasets are not supported");
      }
    } else if (ver == 1 || ver == 2) {
      const int cls = u8(p + 2);
      if (cls != 1) throw std::runtime_error(path_ + ": only contiguous datasets are supported");
      d.addr = u64(p + 8);
    } else {
      throw std::runtime_error(path_ + ": data layout version " + std::to_string(ver));
    }
  }
  const uint8_t* data(const Dataset& d) const {
    const size_t n = (size_t)d.count() * (size_t)d.type.size;
    if (d.isCompact) {
      if (d.compact.size() < n) throw std::runtime_error(path_ + ": compact dataset too small");
      return d.compact.data();
    }
    if (n == 0) return b_.data();
    if (undef(d.addr)) throw std::runtime_error(path_ + ": dataset without storage");
    need(d.addr, n);
    return &b_[d.addr];
  }
  bool attribute(const std::string& name, Attr& a) const {
    for (const Msg& m : messages(root_)) {
      if (m.type != 0xC) continue;
      const size_t p = m.body;
      const int ver = u8(p);
      const int nsz = u16(p + 2), tsz = u16(p + 4), ssz = u16(p + 6);
      size_t q = p + (ver == 3 ? 9 : 8);
      auto pad = [&](int x) { return ver == 1 ? (size_t)((x + 7) / 8 * 8) : (size_t)x; };
      need(q, nsz);
      const std::string nm((const char*)&b_[q], strnlen((const char*)&b_[q], nsz));
      q += pad(nsz);
      if (nm != name) continue;
      a.type = datatype(q);
      q += pad(tsz);
      a.dims = dataspace(q);
      q += pad(ssz);
      a.data = &b_[q];
      uint64_t n = 1;
      for (uint64_t x : a.dims) n *= x;
      need(q, (size_t)n * (size_t)a.type.size);
      return true;
    }
    return false;
  }
  std::vector<long long> ints(const Type& t, const uint8_t* p, uint64_t n, const std::string& name) const {
    if (t.cls != 0 || (t.size != 4 && t.size != 8)) throw std::runtime_error(path_ + ": '" + name + "' is not a 4/8-byte integer");
    std::vector<long long> v(n);
    for (uint64_t i = 0; i < n; ++i) {
      if (t.size == 4) {
        int32_t x; uint32_t y;
        std::memcpy(&y, p + 4 * i, 4);
        std::memcpy(&x, &y, 4);
        v[i] = t.sign ? (long long)x : (long long)y;
      } else {
        int64_t x;
        std::memcpy(&x, p + 8 * i, 8);
        v[i] = x;
      }
    }
    return v;
  }
  std::vector<double> reals(const Type& t, const uint8_t* p, uint64_t n, const std::string& name) const {
    if (t.cls != 1 || (t.size != 8 && t.size != 4)) throw std::runtime_error(path_ + ": '" + name + "' is not an IEEE float");
    std::vector<double> v(n);
    for (uint64_t i = 0; i < n; ++i) {
      if (t.size == 8) std::memcpy(&v[i], p + 8 * i, 8);
      else { float f; std::memcpy(&f, p + 4 * i, 4); v[i] = f; }
    }
    return v;
  }
  std::vector<std::string> strs(const Type& t, const uint8_t* p, uint64_t n, const std::string& name) const {
    if (t.cls != 3) throw std::runtime_error(path_ + ": '" + name + "' is not a fixed-length string");
    std::vector<std::string> v(n);
    for (uint64_t i = 0; i < n; ++i) {
      std::string s((const char*)p + (size_t)t.size * i, (size_t)t.size);
      const size_t z = s.find('\0');
      if (z != std::string::npos) s.resize(z);
      while (!s.empty() && s.back() == ' ') s.pop_back();
      v[i] = s;
    }
    return v;
  }
};

// Writes a superblock-0 file whose root group holds contiguous datasets (up to eight, one symbol table
// node) and attributes, optionally after a user block of 512 * 2^k bytes.
class Writer {
 public:
  void attr_int(const std::string& name, const std::vector<long long>& v, bool scalar = false) {
    attrs_.push_back({name, t_int(), scalar ? std::vector<uint64_t>{} : std::vector<uint64_t>{v.size()}, bytes_int(v)});
  }
  void attr_real(const std::string& name, const std::vector<double>& v, bool scalar = false) {
    attrs_.push_back({name, t_real(), scalar ? std::vector<uint64_t>{} : std::vector<uint64_t>{v.size()}, bytes_real(v)});
  }
  void attr_str(const std::string& name, const std::vector<std::string>& v, bool scalar = false, int len = 255) {
    attrs_.push_back({name, t_str(len), scalar ? std::vector<uint64_t>{} : std::vector<uint64_t>{v.size()}, bytes_str(v, len)});
  }
  // dims in C order (the Fortran dimensions reversed)
  void dataset_real(const std::string& name, const std::vector<uint64_t>& dims, const double* v) {
    uint64_t n = 1;
    for (uint64_t d : dims) n *= d;
    std::vector<uint8_t> b((size_t)n * 8);
    if (n) std::memcpy(b.data(), v, b.size());
    sets_.push_back({name, t_real(), dims, std::move(b)});
  }
  void dataset_int(const std::string& name, const std::vector<uint64_t>& dims, const std::vector<long long>& v) {
    sets_.push_back({name, t_int(), dims, bytes_int(v)});
  }
  void dataset_str(const std::string& name, const std::vector<std::string>& v, int len = 255) {
    sets_.push_back({name, t_str(len), {v.size()}, bytes_str(v, len)});
  }

  void write(const std::string& path, const std::string& userblock = std::string()) {
    if (sets_.size() > 8) throw std::runtime_error("HDF5 writer: at most eight datasets");
    size_t ub = 0;
    if (!userblock.empty()) { ub = 512; while (ub < userblock.size()) ub *= 2; }
    std::vector<uint8_t> f;
    // superblock (96 bytes) and root symbol table entry
    const size_t superSize = 96;
    f.assign(superSize, 0);
    // local heap with the names (offset 0: the empty name of the root group)
    std::vector<uint8_t> heapData(8, 0);
    std::vector<size_t> nameOff;
    std::vector<size_t> order(sets_.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return sets_[a].name < sets_[b].name; });
    nameOff.resize(sets_.size());
    for (size_t k : order) {
      nameOff[k] = heapData.size();
      heapData.insert(heapData.end(), sets_[k].name.begin(), sets_[k].name.end());
      heapData.push_back(0);
      while (heapData.size() % 8) heapData.push_back(0);
    }
    const size_t heapHdr = f.size();
    f.resize(heapHdr + 32, 0);
    const size_t heapDataAddr = f.size();
    f.insert(f.end(), heapData.begin(), heapData.end());
    std::memcpy(&f[heapHdr], "HEAP", 4);
    put64(f, heapHdr + 8, heapData.size());
    put64(f, heapHdr + 16, ~0ull);  // no free block
    put64(f, heapHdr + 24, heapDataAddr);
    // datasets: object header, then data
    std::vector<size_t> hdrAddr(sets_.size());
    for (size_t i = 0; i < sets_.size(); ++i) {
      std::vector<uint8_t> msgs;
      add_msg(msgs, 0x1, space(sets_[i].dims));
      add_msg(msgs, 0x3, sets_[i].type);
      add_msg(msgs, 0x5, std::vector<uint8_t>{2, 2, 0, 0});  // fill value: version 2, late allocation, never written, undefined
      std::vector<uint8_t> lay(18, 0);
      lay[0] = 3; lay[1] = 1;  // version 3, contiguous
      add_msg(msgs, 0x8, lay);
      const size_t layPos = msgs.size() - 24;  // body of the layout message (18 bytes padded to 24)
      hdrAddr[i] = f.size();
      append_header(f, msgs, 4);
      const size_t dataAddr = f.size();
      f.insert(f.end(), sets_[i].data.begin(), sets_[i].data.end());
      while (f.size() % 8) f.push_back(0);
      put64(f, hdrAddr[i] + 16 + layPos + 2, dataAddr);
      put64(f, hdrAddr[i] + 16 + layPos + 10, sets_[i].data.size());
    }
    // symbol table node (room for 2 x leaf K = 8 entries) and B-tree (room for 2 x internal K = 32 children)
    const size_t snod = f.size();
    f.resize(snod + 8 + 8 * 40, 0);
    std::memcpy(&f[snod], "SNOD", 4);
    f[snod + 4] = 1;
    put16(f, snod + 6, sets_.size());
    for (size_t r = 0; r < order.size(); ++r) {
      const size_t q = snod + 8 + r * 40;
      put64(f, q, nameOff[order[r]]);
      put64(f, q + 8, hdrAddr[order[r]]);
    }
    const size_t btree = f.size();
    f.resize(btree + 24 + 33 * 8 + 32 * 8, 0);
    std::memcpy(&f[btree], "TREE", 4);
    f[btree + 4] = 0; f[btree + 5] = 0;
    put16(f, btree + 6, sets_.empty() ? 0 : 1);
    put64(f, btree + 8, ~0ull);
    put64(f, btree + 16, ~0ull);
    put64(f, btree + 24, 0);                                              // key 0: ""
    put64(f, btree + 32, snod);                                           // child 0
    put64(f, btree + 40, sets_.empty() ? 0 : nameOff[order.back()]);      // key 1: last name
    // root group object header: symbol table message and the attributes
    std::vector<uint8_t> msgs;
    std::vector<uint8_t> stab(16);
    std::memcpy(&stab[0], &btree, 8);
    std::memcpy(&stab[8], &heapHdr, 8);
    add_msg(msgs, 0x11, stab);
    for (const Item& a : attrs_) add_msg(msgs, 0xC, attribute(a));
    const size_t rootHdr = f.size();
    append_header(f, msgs, 1);
    // superblock
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    std::memcpy(&f[0], sig, 8);
    f[8] = 0; f[9] = 0; f[10] = 0; f[11] = 0; f[12] = 0; f[13] = 8; f[14] = 8; f[15] = 0;
    put16(f, 16, 4); put16(f, 18, 16);  // group leaf / internal node K
    put64(f, 24, ub);                   // base address: the superblock's absolute position
    put64(f, 32, ~0ull);                // no free-space info
    put64(f, 40, f.size());             // end of file (relative to the base)
    put64(f, 48, ~0ull);                // no driver block
    put64(f, 56, 0);                    // root entry: link name offset
    put64(f, 64, rootHdr);              //             object header
    put32(f, 72, 1);                    //             cache type 1: B-tree and heap in the scratch pad
    put64(f, 80, btree);
    put64(f, 88, heapHdr);
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("cannot write " + path);
    if (ub) {
      std::vector<char> u(ub, 0);
      std::memcpy(u.data(), userblock.data(), userblock.size());
      o.write(u.data(), (std::streamsize)u.size());
    }
    o.write((const char*)f.data(), (std::streamsize)f.size());
    if (!o) throw std::runtime_error("write failed: " + path);
  }

 private:
  struct Item { std::string name; std::vector<uint8_t> type; std::vector<uint64_t> dims; std::vector<uint8_t> data; };
  std::vector<Item> attrs_, sets_;

  static void put16(std::vector<uint8_t>& f, size_t p, uint64_t v) { uint16_t x = (uint16_t)v; std::memcpy(&f[p], &x, 2); }
  static void put32(std::vector<uint8_t>& f, size_t p, uint64_t v) { uint32_t x = (uint32_t)v; std::memcpy(&f[p], &x, 4); }
  static void put64(std::vector<uint8_t>& f, size_t p, uint64_t v) { std::memcpy(&f[p], &v, 8); }
  static std::vector<uint8_t> t_int() {  // signed 32-bit little endian
    std::vector<uint8_t> t(12, 0);
    t[0] = 0x10; t[1] = 0x08; t[4] = 4; t[10] = 32;
    return t;
  }
  static std::vector<uint8_t> t_real() {  // IEEE 754 double, little endian
    std::vector<uint8_t> t(20, 0);
    t[0] = 0x11; t[1] = 0x20; t[2] = 63; t[4] = 8;
    t[10] = 64;  // precision
    t[12] = 52; t[13] = 11; t[14] = 0; t[15] = 52;  // exponent location/size, mantissa location/size
    const uint32_t bias = 1023;
    std::memcpy(&t[16], &bias, 4);
    return t;
  }
  static std::vector<uint8_t> t_str(int len) {  // fixed length, space padded (as Fortran writes them)
    std::vector<uint8_t> t(8, 0);
    t[0] = 0x13; t[1] = 0x02;
    std::memcpy(&t[4], &len, 4);
    return t;
  }
  static std::vector<uint8_t> bytes_int(const std::vector<long long>& v) {
    std::vector<uint8_t> b(v.size() * 4);
    for (size_t i = 0; i < v.size(); ++i) { int32_t x = (int32_t)v[i]; std::memcpy(&b[4 * i], &x, 4); }
    return b;
  }
  static std::vector<uint8_t> bytes_real(const std::vector<double>& v) {
    std::vector<uint8_t> b(v.size() * 8);
    if (!v.empty()) std::memcpy(b.data(), v.data(), b.size());
    return b;
  }
  static std::vector<uint8_t> bytes_str(const std::vector<std::string>& v, int len) {
    std::vector<uint8_t> b(v.size() * (size_t)len, ' ');
    for (size_t i = 0; i < v.size(); ++i) std::memcpy(&b[i * (size_t)len], v[i].data(), std::min(v[i].size(), (size_t)len));
    return b;
  }
  static std::vector<uint8_t> space(const std::vector<uint64_t>& dims) {  // version 1, no maximum dimensions
    std::vector<uint8_t> s(8 + 8 * dims.size(), 0);
    s[0] = 1; s[1] = (uint8_t)dims.size();
    for (size_t i = 0; i < dims.size(); ++i) std::memcpy(&s[8 + 8 * i], &dims[i], 8);
    return s;
  }
  static void pad8(std::vector<uint8_t>& v) { while (v.size() % 8) v.push_back(0); }
  static void add_msg(std::vector<uint8_t>& msgs, uint16_t type, std::vector<uint8_t> body) {
    pad8(body);
    const size_t p = msgs.size();
    msgs.resize(p + 8, 0);
    std::memcpy(&msgs[p], &type, 2);
    const uint16_t sz = (uint16_t)body.size();
    std::memcpy(&msgs[p + 2], &sz, 2);
    msgs.insert(msgs.end(), body.begin(), body.end());
  }
  std::vector<uint8_t> attribute(const Item& a) const {  // version 1: name, type and space padded to 8
    std::vector<uint8_t> b(8, 0);
    b[0] = 1;
    const uint16_t nsz = (uint16_t)(a.name.size() + 1), tsz = (uint16_t)a.type.size();
    const std::vector<uint8_t> sp = space(a.dims);
    const uint16_t ssz = (uint16_t)sp.size();
    std::memcpy(&b[2], &nsz, 2); std::memcpy(&b[4], &tsz, 2); std::memcpy(&b[6], &ssz, 2);
    b.insert(b.end(), a.name.begin(), a.name.end());
    b.push_back(0);
    pad8(b);
    b.insert(b.end(), a.type.begin(), a.type.end());
    pad8(b);
    b.insert(b.end(), sp.begin(), sp.end());
    pad8(b);
    b.insert(b.end(), a.data.begin(), a.data.end());
    return b;
  }
  // version-1 object header (16-byte prefix, messages, a NIL message filling up to at least 256 bytes)
  static void append_header(std::vector<uint8_t>& f, std::vector<uint8_t> msgs, int nmsgWithoutNil) {
    (void)nmsgWithoutNil;
    int count = 0;
    for (size_t p = 0; p < msgs.size();) {
      uint16_t sz;
      std::memcpy(&sz, &msgs[p + 2], 2);
      p += 8 + sz;
      ++count;
    }
    if (msgs.size() < 256) {
      std::vector<uint8_t> nil(256 - msgs.size() - 8, 0);
      add_msg(msgs, 0x0, nil);
      ++count;
    }
    const size_t h = f.size();
    f.resize(h + 16, 0);
    f[h] = 1;
    put16(f, h + 2, count);
    put32(f, h + 4, 1);
    put32(f, h + 8, msgs.size());
    f.insert(f.end(), msgs.begin(), msgs.end());
  }
};

}  // namespace fgh5
