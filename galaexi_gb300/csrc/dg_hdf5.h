// Minimal HDF5 reader for the datasets and attributes of HOPR mesh files and FLEXI state files.
//
// Covers the file-format subset these files use: an optional user block, superblock version 0 (8-byte offsets and
// lengths), object headers version 1 with continuation blocks, old-style groups (symbol-table
// message, v1 B-tree of group nodes, local heap), dataspace messages v1/v2, fixed-point,
// floating-point and fixed-length string datatypes, contiguous and compact data layouts (layout
// message v3), attribute messages v1-v3.  Anything else (chunked or filtered datasets, new-style
// groups, variable-length types) is reported as unsupported rather than guessed.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gxh5 {

struct Array {
  std::vector<uint64_t> dims;   // HDF5 (C) order: slowest first
  int cls = -1;                 // 0 fixed-point, 1 floating-point, 3 string
  int size = 0;                 // bytes per element
  bool is_signed = true;
  std::vector<uint8_t> raw;     // little-endian raw bytes
  uint64_t count() const {
    uint64_t c = 1;
    for (uint64_t d : dims) c *= d;
    return c;
  }
  std::vector<long long> as_int() const;
  std::vector<double> as_double() const;
  std::vector<std::string> as_strings() const;
};

class File {
 public:
  // false (and err set) if the file cannot be read or is not a supported HDF5 file
  bool open(const std::string& path, std::string& err);
  // datasets and attributes of the root group; false (and err set) if absent or unsupported
  bool dataset(const std::string& name, Array& out, std::string& err) const;
  bool attribute(const std::string& name, Array& out, std::string& err) const;
  bool has_dataset(const std::string& name) const;

 private:
  struct Msg {
    uint16_t type;
    uint64_t off;   // file offset of the message data
    uint16_t size;
  };
  std::vector<uint8_t> d_;
  uint64_t root_oh_ = 0;
  std::vector<std::pair<std::string, uint64_t>> links_;  // root-group members: name -> object header
  bool messages(uint64_t oh, std::vector<Msg>& out, std::string& err) const;
  bool read_group(uint64_t btree, uint64_t heap, std::string& err);
  bool decode_type(uint64_t off, Array& a, std::string& err) const;
  bool decode_space(uint64_t off, Array& a, std::string& err) const;
  uint64_t u(uint64_t off, int n) const;
};

// Writer for the same subset: superblock version 0 at offset 0, a root group with a symbol table
// (one v1 B-tree leaf, one symbol-table node, one local heap), version-1 object headers, attribute
// messages v1 on the root group, contiguous datasets (layout message v3).  The structures mirror the
// state files FLEXI writes through the HDF5 library (fixed-length space-padded strings, rank-1
// attributes, maximum dimensions equal to the dimensions).  At most 8 datasets.
class Writer {
 public:
  void attr_string(const std::string& name, const std::string& value);  // length = trimmed length
  void attr_strings(const std::string& name, const std::vector<std::string>& values, int len);
  void attr_int(const std::string& name, const std::vector<int32_t>& values);
  void attr_double(const std::string& name, const std::vector<double>& values);
  // dims slowest first (HDF5/C order); data copied
  void dataset_double(const std::string& name, const std::vector<uint64_t>& dims, const double* data);
  bool write(const std::string& path, std::string& err) const;

 private:
  struct Attr { std::string name; std::vector<uint8_t> type; std::vector<uint64_t> dims; std::vector<uint8_t> data; };
  struct Dset { std::string name; std::vector<uint64_t> dims; std::vector<uint8_t> data; };
  std::vector<Attr> attrs_;
  std::vector<Dset> dsets_;
};

}  // namespace gxh5
