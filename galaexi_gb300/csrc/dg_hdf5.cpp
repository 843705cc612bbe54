// Minimal HDF5 reader (see dg_hdf5.h for the supported subset).  Field layouts follow the
// published HDF5 file-format specification (superblock v0, object header v1, symbol table, local
// heap, v1 B-tree, dataspace / datatype / data-layout / attribute messages).
#include "dg_hdf5.h"

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

}  // namespace gxh5
