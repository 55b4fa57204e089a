// Minimal HDF5 reader and writer for the reference's data files, written from
// the public HDF5 file-format specification (no libhdf5 is available on the
// build or GPU machines).
//
// Reader: superblock versions 0 and 1, groups stored as symbol tables
// (version-1 B-trees of SNOD nodes with a local heap), version-1 object
// headers with continuation blocks, simple dataspaces, IEEE float /
// integer / compound datatypes, contiguous and compact layouts.  That covers
// the force-constant file (dataset of shape (N,N,3,3), read at
// Phonon_Calculations/SRC/force_read.F90:89-164) and the band files
// (write_output.F90:91-484).
//
// Writer: superblock 0, symbol-table groups, version-1 object headers,
// contiguous datasets; groups and datasets are appended as they come and the
// root group and superblock are written on close, so that per-q groups with
// eigenvectors need not be held in memory.
#pragma once
#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace h5min {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// Datatype of a dataset: 'f' IEEE float, 'i' signed / 'u' unsigned
// integer, 'c' compound of float64 members.
struct Type {
  char cls = 0;
  uint32_t size = 0;
  bool big_endian = false;
  std::vector<std::string> member_names;
  std::vector<uint32_t> member_offsets;
};

class Reader {
 public:
  explicit Reader(const std::string &path);
  ~Reader();
  Reader(const Reader &) = delete;
  Reader &operator=(const Reader &) = delete;

  // member names of a group ("/" for the root), sorted
  std::vector<std::string> keys(const std::string &group = "/") const;
  // shape and type of a dataset
  std::vector<uint64_t> shape(const std::string &path, Type *type = nullptr) const;
  // the dataset converted to double (float / integer types; compound types
  // give their members interleaved, i.e. (r, i) pairs for the evec type)
  std::vector<double> read_f64(const std::string &path, std::vector<uint64_t> *shape = nullptr) const;

 private:
  struct Msg {
    uint16_t type;
    uint64_t body;
    uint16_t size;
  };
  struct Dset {
    std::vector<uint64_t> shape;
    Type type;
    uint64_t addr = ~0ull, bytes = 0;
    std::vector<uint8_t> compact;
    bool is_compact = false;
  };
  FILE *f_ = nullptr;
  uint64_t root_ = 0;
  void at(uint64_t off, void *dst, size_t n) const;
  uint8_t u8(uint64_t off) const;
  uint16_t u16(uint64_t off) const;
  uint32_t u32(uint64_t off) const;
  uint64_t u64(uint64_t off) const;
  std::vector<Msg> messages(uint64_t header) const;
  std::map<std::string, uint64_t> links(uint64_t header) const;
  void walk_btree(uint64_t addr, uint64_t heap_data, std::map<std::string, uint64_t> &out) const;
  std::string heap_name(uint64_t heap_data, uint64_t off) const;
  uint64_t resolve(const std::string &path) const;
  Dset dataset(uint64_t header) const;
  Type datatype(uint64_t p, uint64_t *props_len = nullptr) const;
};

class Writer {
 public:
  explicit Writer(const std::string &path);
  ~Writer();
  Writer(const Writer &) = delete;
  Writer &operator=(const Writer &) = delete;

  // One dataset of a group: float64 data of the given shape, or complex
  // (interleaved re, im) data stored with the reference's compound type
  // {r: f64, i: f64}.
  struct Item {
    std::string name;
    std::vector<uint64_t> shape;
    const double *data;
    bool complex_rec;
  };
  // Write a group of datasets now; it becomes a member of the root group.
  void add_group(const std::string &name, const std::vector<Item> &items);
  // A float64 dataset in the root group.
  void add_dataset(const Item &item);
  void close();

 private:
  struct Entry {
    std::string name;
    uint64_t header;
    bool is_group;
    uint64_t btree, heap;
  };
  FILE *f_ = nullptr;
  uint64_t pos_ = 0;
  std::vector<Entry> root_;
  uint64_t alloc(const void *data, size_t n);
  uint64_t object_header(const std::vector<std::vector<uint8_t>> &msgs);
  uint64_t write_item(const Item &it);
  void group(std::vector<Entry> entries, uint64_t *header, uint64_t *btree, uint64_t *heap);
};

}  // namespace h5min
