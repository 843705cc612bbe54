// Minimal HDF5 reader (see dg_hdf5.h for the supported subset).  Field layouts follow the
// published HDF5 file-format specification (superblock v0, object header v1, symbol table, local
// heap, v1 B-tree, dataspace / datatype / data-layout / attribute messages).
#include "dg_hdf5.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace gxh5 {

namespace {
const uint64_t kUndef = ~0ULL;
struct Range : std::runtime_error {
  Range() : std::runtime_error("HDF5: read past the end of the file") {}
};
}  // namespace

uint64_t File::u(uint64_t off, int n) const {
  if (off + (uint64_t)n > d_.size()) throw Range();
  uint64_t v = 0;
  for (int k = n - 1; k >= 0; --k) v = (v << 8) | d_[off + k];
  return v;
}

bool File::open(const std::string& path, std::string& err) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { err = "cannot open " + path; return false; }
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  d_.resize(sz > 0 ? (size_t)sz : 0);
  const size_t got = d_.empty() ? 0 : std::fread(d_.data(), 1, d_.size(), f);
  std::fclose(f);
  if (got != d_.size()) { err = "short read of " + path; return false; }
  try {
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    // the superblock sits at 0 or, after a user block (FLEXI stores its parameter file there), at
    // 512, 1024, 2048, ...; file addresses are relative to it (base address = its position)
    uint64_t base = 0;
    while (base + 96 <= d_.size() && std::memcmp(d_.data() + base, sig, 8) != 0) base = base ? 2 * base : 512;
    if (base + 96 > d_.size()) { err = path + " is not an HDF5 file"; return false; }
    if (base) {
      if (u(base + 24, 8) != base) { err = "HDF5 base address other than the superblock position is not supported"; return false; }
      d_.erase(d_.begin(), d_.begin() + (long)base);
    }
    if (d_[8] != 0) { err = "HDF5 superblock version " + std::to_string(d_[8]) + " is not supported (need 0)"; return false; }
    if (d_[13] != 8 || d_[14] != 8) { err = "HDF5 offsets/lengths other than 8 bytes are not supported"; return false; }
    // root group symbol table entry at 56: name offset, object header, cache type, reserved, scratch
    const uint64_t ent = 56;
    root_oh_ = u(ent + 8, 8);
    std::vector<Msg> ms;
    if (!messages(root_oh_, ms, err)) return false;
    for (const Msg& m : ms)
      if (m.type == 0x11) return read_group(u(m.off, 8), u(m.off + 8, 8), err);
    err = "HDF5 root group has no symbol table (new-style groups are not supported)";
    return false;
  } catch (const std::exception& x) {
    err = x.what();
    return false;
  }
}

bool File::messages(uint64_t oh, std::vector<Msg>& out, std::string& err) const {
  if (oh + 16 > d_.size()) throw Range();
  if (std::memcmp(&d_[oh], "OHDR", 4) == 0) { err = "HDF5 object header version 2 is not supported"; return false; }
  if (d_[oh] != 1) { err = "HDF5 object header version " + std::to_string(d_[oh]) + " is not supported"; return false; }
  const uint64_t nmsg = u(oh + 2, 2);
  std::vector<std::pair<uint64_t, uint64_t>> blocks{{oh + 16, u(oh + 8, 4)}};
  uint64_t seen = 0;
  for (size_t b = 0; b < blocks.size() && seen < nmsg; ++b) {
    uint64_t p = blocks[b].first;
    const uint64_t end = blocks[b].first + blocks[b].second;
    while (p + 8 <= end && seen < nmsg) {
      Msg m;
      m.type = (uint16_t)u(p, 2);
      m.size = (uint16_t)u(p + 2, 2);
      const uint8_t flags = (uint8_t)u(p + 4, 1);
      m.off = p + 8;
      if (m.off + m.size > d_.size()) throw Range();
      if (flags & 0x02) { err = "HDF5 shared header messages are not supported"; return false; }
      if (m.type == 0x10) blocks.push_back({u(m.off, 8), u(m.off + 8, 8)});
      out.push_back(m);
      ++seen;
      p = m.off + m.size;
    }
  }
  return true;
}

bool File::read_group(uint64_t btree, uint64_t heap, std::string& err) {
  if (heap + 32 > d_.size() || std::memcmp(&d_[heap], "HEAP", 4) != 0) { err = "HDF5 local heap not found"; return false; }
  const uint64_t hdata = u(heap + 24, 8);
  std::vector<uint64_t> todo{btree};
  while (!todo.empty()) {
    const uint64_t nd = todo.back();
    todo.pop_back();
    if (nd + 24 > d_.size() || std::memcmp(&d_[nd], "TREE", 4) != 0) { err = "HDF5 B-tree node not found"; return false; }
    if (d_[nd + 4] != 0) { err = "HDF5 B-tree is not a group tree"; return false; }
    const int level = d_[nd + 5];
    const uint64_t used = u(nd + 6, 2);
    uint64_t p = nd + 24;
    for (uint64_t k = 0; k < used; ++k) {
      const uint64_t child = u(p + 8, 8);  // after key k
      p += 16;
      if (level > 0) { todo.push_back(child); continue; }
      if (child + 8 > d_.size() || std::memcmp(&d_[child], "SNOD", 4) != 0) { err = "HDF5 symbol node not found"; return false; }
      const uint64_t nsym = u(child + 6, 2);
      for (uint64_t s = 0; s < nsym; ++s) {
        const uint64_t e = child + 8 + 40 * s;
        const uint64_t name_off = u(e, 8), ohdr = u(e + 8, 8);
        const uint64_t a = hdata + name_off;
        if (a >= d_.size()) throw Range();
        std::string name;
        for (uint64_t c = a; c < d_.size() && d_[c]; ++c) name.push_back((char)d_[c]);
        links_.push_back({name, ohdr});
      }
    }
  }
  return true;
}

bool File::decode_type(uint64_t off, Array& a, std::string& err) const {
  const uint8_t cv = (uint8_t)u(off, 1);
  a.cls = cv & 0x0f;
  const uint32_t bits = (uint32_t)u(off + 1, 3);
  a.size = (int)u(off + 4, 4);
  if (a.cls == 0) {
    if (bits & 1) { err = "HDF5 big-endian integers are not supported"; return false; }
    a.is_signed = (bits & 8) != 0;
  } else if (a.cls == 1) {
    if (bits & 1) { err = "HDF5 big-endian floats are not supported"; return false; }
    if (a.size != 4 && a.size != 8) { err = "HDF5 float size not supported"; return false; }
  } else if (a.cls != 3) {
    err = "HDF5 datatype class " + std::to_string(a.cls) + " is not supported";
    return false;
  }
  return true;
}

bool File::decode_space(uint64_t off, Array& a, std::string& err) const {
  const int ver = (int)u(off, 1), rank = (int)u(off + 1, 1);
  uint64_t p;
  if (ver == 1) p = off + 8;
  else if (ver == 2) p = off + 4;
  else {
    err = "HDF5 dataspace version " + std::to_string(ver) + " is not supported";
    return false;
  }
  a.dims.clear();
  for (int r = 0; r < rank; ++r) a.dims.push_back(u(p + 8 * r, 8));
  if (ver == 2 && u(off + 3, 1) == 2) a.dims.assign(1, 0);
  return true;
}

bool File::has_dataset(const std::string& name) const {
  for (const auto& l : links_)
    if (l.first == name) return true;
  return false;
}

bool File::dataset(const std::string& name, Array& out, std::string& err) const {
  try {
    uint64_t oh = kUndef;
    for (const auto& l : links_)
      if (l.first == name) oh = l.second;
    if (oh == kUndef) { err = "HDF5 dataset '" + name + "' not found"; return false; }
    std::vector<Msg> ms;
    if (!messages(oh, ms, err)) return false;
    bool have_space = false, have_type = false, have_layout = false;
    uint64_t addr = kUndef, bytes = 0, compact = 0;
    for (const Msg& m : ms) {
      if (m.type == 0x01) { if (!decode_space(m.off, out, err)) return false; have_space = true; }
      else if (m.type == 0x03) { if (!decode_type(m.off, out, err)) return false; have_type = true; }
      else if (m.type == 0x0B) { err = "HDF5 dataset '" + name + "' is filtered (compressed): not supported"; return false; }
      else if (m.type == 0x08) {
        const int ver = (int)u(m.off, 1);
        if (ver == 3) {
          const int cls = (int)u(m.off + 1, 1);
          if (cls == 0) { bytes = u(m.off + 2, 2); compact = m.off + 4; }
          else if (cls == 1) { addr = u(m.off + 2, 8); bytes = u(m.off + 10, 8); }
          else { err = "HDF5 dataset '" + name + "' is chunked: not supported"; return false; }
        } else if (ver == 1 || ver == 2) {
          const int rank = (int)u(m.off + 1, 1), cls = (int)u(m.off + 2, 1);
          if (cls != 1) { err = "HDF5 layout v1/v2 other than contiguous is not supported"; return false; }
          addr = u(m.off + 8, 8);
          bytes = 1;
          for (int r = 0; r < rank; ++r) bytes *= u(m.off + 16 + 4 * r, 4);
        } else {
          err = "HDF5 layout version " + std::to_string(ver) + " is not supported";
          return false;
        }
        have_layout = true;
      }
    }
    if (!have_space || !have_type || !have_layout) { err = "HDF5 dataset '" + name + "' lacks space/type/layout"; return false; }
    const uint64_t need = out.count() * (uint64_t)out.size;
    if (compact) {
      if (bytes < need) { err = "HDF5 compact dataset too short"; return false; }
      out.raw.assign(d_.begin() + compact, d_.begin() + compact + need);
    } else if (need == 0) {
      out.raw.clear();
    } else {
      if (addr == kUndef || addr + need > d_.size()) { err = "HDF5 dataset '" + name + "' has no (complete) storage"; return false; }
      out.raw.assign(d_.begin() + addr, d_.begin() + addr + need);
    }
    return true;
  } catch (const std::exception& x) {
    err = x.what();
    return false;
  }
}

bool File::attribute(const std::string& name, Array& out, std::string& err) const {
  try {
    std::vector<Msg> ms;
    if (!messages(root_oh_, ms, err)) return false;
    for (const Msg& m : ms) {
      if (m.type != 0x0C) continue;
      const int ver = (int)u(m.off, 1);
      const uint64_t nsz = u(m.off + 2, 2), tsz = u(m.off + 4, 2), ssz = u(m.off + 6, 2);
      uint64_t p = m.off + 8;
      if (ver == 3) p += 1;  // name character set
      else if (ver != 1 && ver != 2) continue;
      auto pad = [&](uint64_t x) { return ver == 1 ? (x + 7) / 8 * 8 : x; };
      std::string an;
      for (uint64_t c = 0; c + 1 < nsz; ++c) an.push_back((char)u(p + c, 1));
      while (!an.empty() && an.back() == '\0') an.pop_back();
      p += pad(nsz);
      if (an != name) continue;
      if (!decode_type(p, out, err)) return false;
      p += pad(tsz);
      if (!decode_space(p, out, err)) return false;
      p += pad(ssz);
      const uint64_t need = out.count() * (uint64_t)out.size;
      if (p + need > m.off + m.size) throw Range();
      out.raw.assign(d_.begin() + p, d_.begin() + p + need);
      return true;
    }
    err = "HDF5 attribute '" + name + "' not found";
    return false;
  } catch (const std::exception& x) {
    err = x.what();
    return false;
  }
}

std::vector<long long> Array::as_int() const {
  std::vector<long long> v(count());
  for (uint64_t k = 0; k < v.size(); ++k) {
    if (cls == 1) {
      double x;
      if (size == 8) std::memcpy(&x, &raw[8 * k], 8);
      else { float f; std::memcpy(&f, &raw[4 * k], 4); x = f; }
      v[k] = (long long)x;
      continue;
    }
    uint64_t w = 0;
    for (int b = size - 1; b >= 0; --b) w = (w << 8) | raw[size * k + b];
    if (is_signed && size < 8 && (w >> (8 * size - 1)) & 1) w |= ~0ULL << (8 * size);
    v[k] = (long long)w;
  }
  return v;
}

std::vector<double> Array::as_double() const {
  std::vector<double> v(count());
  if (cls != 1) {
    const std::vector<long long> iv = as_int();
    for (uint64_t k = 0; k < v.size(); ++k) v[k] = (double)iv[k];
    return v;
  }
  for (uint64_t k = 0; k < v.size(); ++k) {
    if (size == 8) std::memcpy(&v[k], &raw[8 * k], 8);
    else { float f; std::memcpy(&f, &raw[4 * k], 4); v[k] = f; }
  }
  return v;
}

std::vector<std::string> Array::as_strings() const {
  std::vector<std::string> v;
  if (cls != 3) return v;
  for (uint64_t k = 0; k < count(); ++k) {
    std::string s((const char*)&raw[size * k], (size_t)size);
    while (!s.empty() && (s.back() == '\0' || s.back() == ' ')) s.pop_back();
    v.push_back(s);
  }
  return v;
}

// ----------------------------------------------------------------------------------------------
// Writer
// ----------------------------------------------------------------------------------------------
namespace {
// datatype message bodies (class + version 1, bit field, size, properties)
std::vector<uint8_t> type_double() {
  return {0x11, 0x20, 0x3f, 0x00, 8, 0, 0, 0, 0, 0, 64, 0, 52, 11, 0, 52, 0xff, 0x03, 0, 0};
}
std::vector<uint8_t> type_int32() { return {0x10, 0x08, 0, 0, 4, 0, 0, 0, 0, 0, 32, 0}; }
std::vector<uint8_t> type_string(uint32_t len) {  // fixed length, space padded, ASCII
  return {0x13, 0x02, 0, 0, (uint8_t)(len & 0xff), (uint8_t)((len >> 8) & 0xff), (uint8_t)((len >> 16) & 0xff),
          (uint8_t)(len >> 24)};
}
// dataspace message v1 with maximum dimensions equal to the dimensions
std::vector<uint8_t> space(const std::vector<uint64_t>& dims) {
  std::vector<uint8_t> b = {1, (uint8_t)dims.size(), 1, 0, 0, 0, 0, 0};
  for (int rep = 0; rep < 2; ++rep)
    for (uint64_t d : dims)
      for (int k = 0; k < 8; ++k) b.push_back((uint8_t)(d >> (8 * k)));
  return b;
}
struct Buf {
  std::vector<uint8_t> b;
  void u(uint64_t v, int n) { for (int k = 0; k < n; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void bytes(const std::vector<uint8_t>& x) { b.insert(b.end(), x.begin(), x.end()); }
  void pad8() { while (b.size() % 8) b.push_back(0); }
  void at(size_t off, uint64_t v, int n) { for (int k = 0; k < n; ++k) b[off + k] = (uint8_t)(v >> (8 * k)); }
};
const uint64_t kUndefAddr = ~0ULL;
size_t pad8(size_t n) { return (n + 7) & ~(size_t)7; }
// one object-header message: type, size, flags, reserved, body padded to 8
void message(Buf& o, uint16_t type, uint8_t flags, const std::vector<uint8_t>& body) {
  const size_t sz = pad8(body.size());
  o.u(type, 2); o.u(sz, 2); o.u(flags, 1); o.u(0, 3);
  o.bytes(body);
  while (o.b.size() % 8) o.b.push_back(0);
}
// version-1 object header around the given messages (count, bytes)
std::vector<uint8_t> object_header(int nmsg, const std::vector<uint8_t>& msgs) {
  Buf h;
  h.u(1, 1); h.u(0, 1); h.u(nmsg, 2); h.u(1, 4); h.u(msgs.size(), 4); h.u(0, 4);
  h.bytes(msgs);
  return h.b;
}
}  // namespace

void Writer::attr_string(const std::string& name, const std::string& value) {
  std::string v = value;
  while (!v.empty() && v.back() == ' ') v.pop_back();
  const uint32_t len = v.empty() ? 1 : (uint32_t)v.size();
  Attr a{name, type_string(len), {1}, {}};
  a.data.assign(len, ' ');
  std::memcpy(a.data.data(), v.data(), v.size());
  attrs_.push_back(a);
}

void Writer::attr_strings(const std::string& name, const std::vector<std::string>& values, int len) {
  Attr a{name, type_string((uint32_t)len), {values.size()}, {}};
  a.data.assign(values.size() * (size_t)len, ' ');
  for (size_t i = 0; i < values.size(); ++i)
    std::memcpy(a.data.data() + i * len, values[i].data(), std::min((size_t)len, values[i].size()));
  attrs_.push_back(a);
}

void Writer::attr_int(const std::string& name, const std::vector<int32_t>& values) {
  Attr a{name, type_int32(), {values.size()}, {}};
  a.data.resize(values.size() * 4);
  std::memcpy(a.data.data(), values.data(), a.data.size());
  attrs_.push_back(a);
}

void Writer::attr_double(const std::string& name, const std::vector<double>& values) {
  Attr a{name, type_double(), {values.size()}, {}};
  a.data.resize(values.size() * 8);
  std::memcpy(a.data.data(), values.data(), a.data.size());
  attrs_.push_back(a);
}

void Writer::dataset_double(const std::string& name, const std::vector<uint64_t>& dims, const double* data) {
  uint64_t cnt = 1;
  for (uint64_t d : dims) cnt *= d;
  Dset d{name, dims, {}};
  d.data.resize(cnt * 8);
  if (cnt) std::memcpy(d.data.data(), data, d.data.size());
  dsets_.push_back(d);
}

bool Writer::write(const std::string& path, std::string& err) const {
  if (dsets_.size() > 8) { err = "HDF5 writer: at most 8 datasets"; return false; }
  const int leafK = 4, internK = 16;
  // local heap data segment: "" at 0, the dataset names in symbol-table (sorted) order, a free block
  std::vector<size_t> order(dsets_.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return dsets_[a].name < dsets_[b].name; });
  Buf heapseg;
  heapseg.u(0, 8);
  std::vector<size_t> name_off(dsets_.size());
  for (size_t i : order) {
    name_off[i] = heapseg.b.size();
    heapseg.bytes(std::vector<uint8_t>(dsets_[i].name.begin(), dsets_[i].name.end()));
    heapseg.u(0, 1);
    heapseg.pad8();
  }
  const size_t free_off = heapseg.b.size();
  heapseg.u(1, 8);   // next free block: none (H5HL_FREE_NULL)
  heapseg.u(16, 8);  // size of this free block
  // root object header: symbol table message + attribute messages
  const size_t sb_size = 96;
  Buf rootmsgs;
  message(rootmsgs, 0x11, 0, std::vector<uint8_t>(16, 0));  // patched below
  for (const Attr& a : attrs_) {
    Buf body;
    const std::vector<uint8_t> sp = space(a.dims);
    body.u(1, 1); body.u(0, 1); body.u(a.name.size() + 1, 2); body.u(a.type.size(), 2); body.u(sp.size(), 2);
    body.bytes(std::vector<uint8_t>(a.name.begin(), a.name.end())); body.u(0, 1); body.pad8();
    body.bytes(a.type); body.pad8();
    body.bytes(sp); body.pad8();
    body.bytes(a.data);
    if (body.b.size() > 65535 - 8) { err = "HDF5 writer: attribute " + a.name + " too large"; return false; }
    message(rootmsgs, 0x0c, 0, body.b);
  }
  const size_t root_addr = sb_size;
  const size_t root_size = 16 + rootmsgs.b.size();
  const size_t heap_addr = pad8(root_addr + root_size);
  const size_t heapseg_addr = heap_addr + 32;
  const size_t btree_addr = pad8(heapseg_addr + heapseg.b.size());
  const size_t btree_size = 24 + (2 * internK + 1) * 8 + 2 * internK * 8;
  const size_t snod_addr = btree_addr + btree_size;
  const size_t snod_size = 8 + 2 * leafK * 40;
  // dataset object headers, then the data
  size_t at = pad8(snod_addr + snod_size);
  std::vector<size_t> oh_addr(dsets_.size()), oh_size(dsets_.size());
  for (size_t i = 0; i < dsets_.size(); ++i) {
    // dataspace, datatype, fill value v2 (late allocation, fill written if set, default value),
    // layout v3 contiguous: 8-byte headers + padded bodies
    oh_size[i] = 16 + (8 + pad8(space(dsets_[i].dims).size())) + (8 + 24) + (8 + 8) + (8 + 24);
    oh_addr[i] = at;
    at = pad8(at + oh_size[i]);
  }
  std::vector<size_t> data_addr(dsets_.size());
  for (size_t i = 0; i < dsets_.size(); ++i) {
    data_addr[i] = at;
    at = pad8(at + dsets_[i].data.size());
  }
  const size_t eof = at;
  Buf f;
  f.b.reserve(eof);
  // superblock v0
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  f.bytes(std::vector<uint8_t>(sig, sig + 8));
  f.u(0, 1); f.u(0, 1); f.u(0, 1); f.u(0, 1); f.u(0, 1); f.u(8, 1); f.u(8, 1); f.u(0, 1);
  f.u(leafK, 2); f.u(internK, 2); f.u(0, 4);
  f.u(0, 8); f.u(kUndefAddr, 8); f.u(eof, 8); f.u(kUndefAddr, 8);
  // root symbol table entry: name offset, object header, cache type 1 (B-tree and heap cached)
  f.u(0, 8); f.u(root_addr, 8); f.u(1, 4); f.u(0, 4); f.u(btree_addr, 8); f.u(heap_addr, 8);
  // root object header (symbol table message body patched)
  Buf rm = rootmsgs;
  rm.at(8, btree_addr, 8); rm.at(16, heap_addr, 8);
  f.bytes(object_header(1 + (int)attrs_.size(), rm.b));
  while (f.b.size() < heap_addr) f.b.push_back(0);
  // local heap
  f.bytes({'H', 'E', 'A', 'P', 0, 0, 0, 0});
  f.u(heapseg.b.size(), 8); f.u(free_off, 8); f.u(heapseg_addr, 8);
  f.bytes(heapseg.b);
  while (f.b.size() < btree_addr) f.b.push_back(0);
  // B-tree leaf (group node, level 0) with one child, the symbol-table node
  f.bytes({'T', 'R', 'E', 'E', 0, 0});
  f.u(dsets_.empty() ? 0 : 1, 2); f.u(kUndefAddr, 8); f.u(kUndefAddr, 8);
  {
    Buf kc;
    if (!dsets_.empty()) {
      kc.u(0, 8); kc.u(snod_addr, 8); kc.u(name_off[order.back()], 8);
    }
    kc.b.resize(btree_size - 24, 0);
    f.bytes(kc.b);
  }
  // symbol-table node, entries sorted by name
  f.bytes({'S', 'N', 'O', 'D', 1, 0});
  f.u(dsets_.size(), 2);
  {
    Buf ent;
    for (size_t i : order) { ent.u(name_off[i], 8); ent.u(oh_addr[i], 8); ent.u(0, 4); ent.u(0, 4); ent.u(0, 16); }
    ent.b.resize(2 * leafK * 40, 0);
    f.bytes(ent.b);
  }
  // dataset object headers
  for (size_t i = 0; i < dsets_.size(); ++i) {
    while (f.b.size() < oh_addr[i]) f.b.push_back(0);
    Buf m;
    message(m, 0x01, 0, space(dsets_[i].dims));
    message(m, 0x03, 1, type_double());
    message(m, 0x05, 1, {2, 2, 2, 1, 0, 0, 0, 0});
    Buf lay;
    lay.u(3, 1); lay.u(1, 1); lay.u(data_addr[i], 8); lay.u(dsets_[i].data.size(), 8);
    message(m, 0x08, 1, lay.b);
    f.bytes(object_header(4, m.b));
  }
  for (size_t i = 0; i < dsets_.size(); ++i) {
    while (f.b.size() < data_addr[i]) f.b.push_back(0);
    f.bytes(dsets_[i].data);
  }
  while (f.b.size() < eof) f.b.push_back(0);
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) { err = "cannot create " + path; return false; }
  const size_t w = std::fwrite(f.b.data(), 1, f.b.size(), fp);
  const bool ok = std::fclose(fp) == 0 && w == f.b.size();
  if (!ok) { err = "short write of " + path; return false; }
  return true;
}

}  // namespace gxh5
