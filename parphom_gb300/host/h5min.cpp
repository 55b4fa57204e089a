#include "h5min.hpp"

#include <algorithm>
#include <cstring>

namespace h5min {

namespace {
const uint8_t SIG[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr uint64_t UNDEF = ~0ull;
constexpr int LEAF_K = 64;      // a symbol-table node holds up to 2K entries
constexpr int INTERNAL_K = 64;  // a group B-tree node holds up to 2K children

void put(std::vector<uint8_t> &b, const void *p, size_t n) {
  const uint8_t *c = (const uint8_t *)p;
  b.insert(b.end(), c, c + n);
}
template <class T>
void put_le(std::vector<uint8_t> &b, T v) {
  for (size_t i = 0; i < sizeof(T); ++i) b.push_back((uint8_t)((uint64_t)v >> (8 * i)));
}
void pad8(std::vector<uint8_t> &b) {
  while (b.size() % 8) b.push_back(0);
}
std::vector<uint8_t> msg(uint16_t type, std::vector<uint8_t> body, uint8_t flags = 0) {
  pad8(body);
  std::vector<uint8_t> m;
  put_le<uint16_t>(m, type);
  put_le<uint16_t>(m, (uint16_t)body.size());
  m.push_back(flags);
  m.insert(m.end(), 3, 0);
  m.insert(m.end(), body.begin(), body.end());
  return m;
}
// class 1 (floating point), version 1: little endian, IEEE double layout
std::vector<uint8_t> dt_f64() {
  std::vector<uint8_t> b = {0x11, 0x20, 0x3F, 0x00};
  put_le<uint32_t>(b, 8);
  put_le<uint16_t>(b, 0);
  put_le<uint16_t>(b, 64);
  b.push_back(52);
  b.push_back(11);
  b.push_back(0);
  b.push_back(52);
  put_le<uint32_t>(b, 1023);
  return b;
}
// version-1 compound of float64 members r (offset 0) and i (offset 8)
std::vector<uint8_t> dt_complex() {
  std::vector<uint8_t> b = {0x16};
  put_le<uint16_t>(b, 2);
  b.push_back(0);
  put_le<uint32_t>(b, 16);
  const char *names[2] = {"r", "i"};
  for (int k = 0; k < 2; ++k) {
    std::vector<uint8_t> nm(names[k], names[k] + strlen(names[k]) + 1);
    pad8(nm);
    put(b, nm.data(), nm.size());
    put_le<uint32_t>(b, 8u * k);  // byte offset
    b.push_back(0);               // dimensionality
    b.insert(b.end(), 3, 0);
    put_le<uint32_t>(b, 0);       // permutation
    put_le<uint32_t>(b, 0);
    for (int d = 0; d < 4; ++d) put_le<uint32_t>(b, 0);
    auto f = dt_f64();
    put(b, f.data(), f.size());
  }
  return b;
}
}  // namespace

// ============================================================================
// Reader
Reader::Reader(const std::string &path) {
  f_ = fopen(path.c_str(), "rb");
  if (!f_) throw Error("cannot open " + path);
  uint8_t sb[16];
  at(0, sb, 16);
  if (memcmp(sb, SIG, 8) != 0) throw Error(path + ": not an HDF5 file (no superblock signature at offset 0)");
  const int ver = sb[8];
  if (ver != 0 && ver != 1) throw Error("superblock version " + std::to_string(ver) + " not supported");
  if (sb[13] != 8 || sb[14] != 8) throw Error("only 8-byte offsets and lengths are supported");
  uint64_t p = 16 + 4 + 4 + (ver == 1 ? 4 : 0);
  p += 32;               // base, free space, end of file, driver info
  root_ = u64(p + 8);    // root symbol table entry: object header address
}
Reader::~Reader() {
  if (f_) fclose(f_);
}
void Reader::at(uint64_t off, void *dst, size_t n) const {
  if (fseeko(f_, (off_t)off, SEEK_SET) != 0 || fread(dst, 1, n, f_) != n) throw Error("read beyond end of file");
}
uint8_t Reader::u8(uint64_t off) const {
  uint8_t v;
  at(off, &v, 1);
  return v;
}
uint16_t Reader::u16(uint64_t off) const {
  uint8_t b[2];
  at(off, b, 2);
  return (uint16_t)(b[0] | (b[1] << 8));
}
uint32_t Reader::u32(uint64_t off) const {
  uint8_t b[4];
  at(off, b, 4);
  return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
}
uint64_t Reader::u64(uint64_t off) const {
  uint8_t b[8];
  at(off, b, 8);
  uint64_t v = 0;
  for (int i = 7; i >= 0; --i) v = (v << 8) | b[i];
  return v;
}

std::vector<Reader::Msg> Reader::messages(uint64_t addr) const {
  if (u8(addr) != 1) throw Error("object header version " + std::to_string(u8(addr)) + " not supported");
  const uint16_t nmsg = u16(addr + 2);
  const uint32_t size = u32(addr + 8);
  std::vector<std::pair<uint64_t, uint64_t>> blocks = {{addr + 16, size}};
  std::vector<Msg> out;
  for (size_t bi = 0; bi < blocks.size() && out.size() < nmsg; ++bi) {
    const uint64_t start = blocks[bi].first, len = blocks[bi].second;
    uint64_t p = start;
    while (p + 8 <= start + len && out.size() < nmsg) {
      const uint16_t type = u16(p), msize = u16(p + 2);
      const uint64_t body = p + 8;
      if (type == 0x10) blocks.push_back({u64(body), u64(body + 8)});  // continuation
      out.push_back({type, body, msize});
      p = body + msize;
    }
  }
  return out;
}

std::string Reader::heap_name(uint64_t heap_data, uint64_t off) const {
  std::string s;
  for (uint64_t p = heap_data + off;; ++p) {
    const char c = (char)u8(p);
    if (!c) break;
    s.push_back(c);
  }
  return s;
}

void Reader::walk_btree(uint64_t addr, uint64_t heap_data, std::map<std::string, uint64_t> &out) const {
  char sig[4];
  at(addr, sig, 4);
  if (memcmp(sig, "TREE", 4) != 0) throw Error("bad B-tree node");
  if (u8(addr + 4) != 0) throw Error("not a group B-tree");
  const int level = u8(addr + 5);
  const int used = u16(addr + 6);
  uint64_t p = addr + 24 + 8;  // after the header and key 0
  for (int k = 0; k < used; ++k) {
    const uint64_t child = u64(p);
    p += 16;
    if (level > 0) {
      walk_btree(child, heap_data, out);
    } else {
      at(child, sig, 4);
      if (memcmp(sig, "SNOD", 4) != 0) throw Error("bad symbol table node");
      const int nsym = u16(child + 6);
      for (int e = 0; e < nsym; ++e) {
        const uint64_t ent = child + 8 + 40ull * e;
        out[heap_name(heap_data, u64(ent))] = u64(ent + 8);
      }
    }
  }
}

std::map<std::string, uint64_t> Reader::links(uint64_t header) const {
  for (const Msg &m : messages(header)) {
    if (m.type == 0x11) {
      const uint64_t btree = u64(m.body), heap = u64(m.body + 8);
      char sig[4];
      at(heap, sig, 4);
      if (memcmp(sig, "HEAP", 4) != 0) throw Error("bad local heap");
      std::map<std::string, uint64_t> out;
      walk_btree(btree, u64(heap + 24), out);
      return out;
    }
  }
  throw Error("object is not a symbol-table group");
}

uint64_t Reader::resolve(const std::string &path) const {
  uint64_t addr = root_;
  size_t s = 0;
  while (s < path.size()) {
    size_t e = path.find('/', s);
    if (e == std::string::npos) e = path.size();
    const std::string part = path.substr(s, e - s);
    s = e + 1;
    if (part.empty()) continue;
    const auto l = links(addr);
    const auto it = l.find(part);
    if (it == l.end()) throw Error("no member '" + part + "' in path " + path);
    addr = it->second;
  }
  return addr;
}

std::vector<std::string> Reader::keys(const std::string &group) const {
  std::vector<std::string> out;
  for (auto &kv : links(resolve(group))) out.push_back(kv.first);
  return out;
}

Type Reader::datatype(uint64_t p, uint64_t *props_len) const {
  const uint8_t cv = u8(p);
  const int cls = cv & 0x0F, ver = cv >> 4;
  const uint8_t bits0 = u8(p + 1);
  Type t;
  t.size = u32(p + 4);
  t.big_endian = bits0 & 1;
  if (cls == 1) {
    t.cls = 'f';
    if (props_len) *props_len = 12;
  } else if (cls == 0) {
    t.cls = ((bits0 >> 3) & 1) ? 'i' : 'u';
    if (props_len) *props_len = 4;
  } else if (cls == 6) {
    t.cls = 'c';
    const int nmemb = u16(p + 1);
    uint64_t q = p + 8;
    for (int k = 0; k < nmemb; ++k) {
      std::string name;
      for (;;) {
        const char c = (char)u8(q + name.size());
        if (!c) break;
        name.push_back(c);
      }
      const uint64_t nlen = name.size() + 1;
      uint32_t moff;
      if (ver < 3) {
        q += (nlen + 7) / 8 * 8;
        moff = u32(q);
        q += 4 + 1 + 3 + 4 + 4 + 16;
      } else {
        q += nlen;
        const int nb = t.size < 256 ? 1 : t.size < 65536 ? 2 : 4;
        moff = 0;
        for (int i = 0; i < nb; ++i) moff |= (uint32_t)u8(q + i) << (8 * i);
        q += nb;
      }
      uint64_t ml = 0;
      const Type mt = datatype(q, &ml);
      if (mt.cls != 'f' || mt.size != 8) throw Error("compound members other than float64 are not supported");
      q += 8 + ml;
      t.member_names.push_back(name);
      t.member_offsets.push_back(moff);
    }
    if (props_len) *props_len = q - (p + 8);
  } else {
    throw Error("datatype class " + std::to_string(cls) + " not supported");
  }
  return t;
}

Reader::Dset Reader::dataset(uint64_t header) const {
  Dset d;
  bool have_space = false, have_type = false;
  for (const Msg &m : messages(header)) {
    if (m.type == 0x01) {
      const int ver = u8(m.body), ndim = u8(m.body + 1);
      const uint64_t off = m.body + (ver == 1 ? 8 : 4);
      for (int k = 0; k < ndim; ++k) d.shape.push_back(u64(off + 8ull * k));
      have_space = true;
    } else if (m.type == 0x03) {
      d.type = datatype(m.body);
      have_type = true;
    } else if (m.type == 0x08) {
      const int ver = u8(m.body);
      if (ver == 3) {
        const int cls = u8(m.body + 1);
        if (cls == 1) {
          d.addr = u64(m.body + 2);
          d.bytes = u64(m.body + 10);
        } else if (cls == 0) {
          const uint16_t sz = u16(m.body + 2);
          d.compact.resize(sz);
          if (sz) at(m.body + 4, d.compact.data(), sz);
          d.is_compact = true;
        } else {
          throw Error("chunked layout not supported");
        }
      } else if (ver == 1 || ver == 2) {
        if (u8(m.body + 2) != 1) throw Error("only contiguous layout supported for layout v1/v2");
        d.addr = u64(m.body + 8);
      } else {
        throw Error("layout version " + std::to_string(ver) + " not supported");
      }
    }
  }
  if (!have_space || !have_type) throw Error("dataset without dataspace or datatype");
  return d;
}

std::vector<uint64_t> Reader::shape(const std::string &path, Type *type) const {
  Dset d = dataset(resolve(path));
  if (type) *type = d.type;
  return d.shape;
}

std::vector<double> Reader::read_f64(const std::string &path, std::vector<uint64_t> *shape) const {
  const Dset d = dataset(resolve(path));
  uint64_t count = 1;
  for (uint64_t s : d.shape) count *= s;
  const uint64_t nbytes = count * d.type.size;
  std::vector<uint8_t> raw(nbytes);
  if (d.is_compact) {
    if (d.compact.size() < nbytes) throw Error("truncated compact dataset");
    memcpy(raw.data(), d.compact.data(), nbytes);
  } else if (d.addr != UNDEF && nbytes) {
    at(d.addr, raw.data(), nbytes);
  }
  const uint32_t sz = d.type.size;
  auto word = [&](uint64_t byte_off, uint32_t n) {
    uint64_t v = 0;
    for (uint32_t i = 0; i < n; ++i) {
      const uint8_t b = raw[byte_off + (d.type.big_endian ? i : n - 1 - i)];
      v = (v << 8) | b;
    }
    return v;
  };
  std::vector<double> out;
  if (d.type.cls == 'c') {
    const size_t nm = d.type.member_offsets.size();
    out.resize(count * nm);
    for (uint64_t e = 0; e < count; ++e)
      for (size_t k = 0; k < nm; ++k) {
        const uint64_t bits = word(e * sz + d.type.member_offsets[k], 8);
        double v;
        memcpy(&v, &bits, 8);
        out[e * nm + k] = v;
      }
  } else {
    out.resize(count);
    for (uint64_t e = 0; e < count; ++e) {
      const uint64_t bits = word(e * sz, sz);
      double v;
      if (d.type.cls == 'f') {
        if (sz == 8) {
          memcpy(&v, &bits, 8);
        } else if (sz == 4) {
          const uint32_t b32 = (uint32_t)bits;
          float fv;
          memcpy(&fv, &b32, 4);
          v = fv;
        } else {
          throw Error("float size " + std::to_string(sz) + " not supported");
        }
      } else if (d.type.cls == 'i') {
        const int sh = 64 - 8 * (int)sz;
        v = (double)((int64_t)(bits << sh) >> sh);
      } else {
        v = (double)bits;
      }
      out[e] = v;
    }
  }
  if (shape) *shape = d.shape;
  return out;
}

// ============================================================================
// Writer
Writer::Writer(const std::string &path) {
  f_ = fopen(path.c_str(), "wb");
  if (!f_) throw Error("cannot create " + path);
  std::vector<uint8_t> zero(96, 0);
  if (fwrite(zero.data(), 1, 96, f_) != 96) throw Error("write failed");
  pos_ = 96;
}
Writer::~Writer() {
  try {
    close();
  } catch (...) {
  }
}

uint64_t Writer::alloc(const void *data, size_t n) {
  static const uint8_t zeros[8] = {0};
  const size_t pad = (8 - pos_ % 8) % 8;
  if (pad) {
    if (fwrite(zeros, 1, pad, f_) != pad) throw Error("write failed");
    pos_ += pad;
  }
  const uint64_t addr = pos_;
  if (n && fwrite(data, 1, n, f_) != n) throw Error("write failed");
  pos_ += n;
  return addr;
}

uint64_t Writer::object_header(const std::vector<std::vector<uint8_t>> &msgs) {
  std::vector<uint8_t> body;
  for (auto &m : msgs) body.insert(body.end(), m.begin(), m.end());
  std::vector<uint8_t> h = {1, 0};
  put_le<uint16_t>(h, (uint16_t)msgs.size());
  put_le<uint32_t>(h, 1);
  put_le<uint32_t>(h, (uint32_t)body.size());
  h.insert(h.end(), 4, 0);
  h.insert(h.end(), body.begin(), body.end());
  return alloc(h.data(), h.size());
}

uint64_t Writer::write_item(const Item &it) {
  uint64_t count = 1;
  for (uint64_t s : it.shape) count *= s;
  const uint64_t nbytes = count * (it.complex_rec ? 16 : 8);
  const uint64_t data = nbytes ? alloc(it.data, nbytes) : UNDEF;
  std::vector<uint8_t> space = {1, (uint8_t)it.shape.size(), 0, 0, 0, 0, 0, 0};
  for (uint64_t s : it.shape) put_le<uint64_t>(space, s);
  std::vector<uint8_t> layout = {3, 1};
  put_le<uint64_t>(layout, data);
  put_le<uint64_t>(layout, nbytes);
  return object_header({msg(0x0001, space), msg(0x0003, it.complex_rec ? dt_complex() : dt_f64(), 1),
                        msg(0x0008, layout)});
}

void Writer::group(std::vector<Entry> entries, uint64_t *header, uint64_t *btree, uint64_t *heap) {
  std::sort(entries.begin(), entries.end(), [](const Entry &a, const Entry &b) { return a.name < b.name; });
  std::vector<uint8_t> heapdata(8, 0);  // offset 0: the empty name
  std::vector<uint64_t> offs;
  for (auto &e : entries) {
    offs.push_back(heapdata.size());
    heapdata.insert(heapdata.end(), e.name.begin(), e.name.end());
    heapdata.push_back(0);
    pad8(heapdata);
  }
  const uint64_t data_addr = alloc(heapdata.data(), heapdata.size());
  std::vector<uint8_t> hp = {'H', 'E', 'A', 'P', 0, 0, 0, 0};
  put_le<uint64_t>(hp, heapdata.size());
  put_le<uint64_t>(hp, UNDEF);
  put_le<uint64_t>(hp, data_addr);
  *heap = alloc(hp.data(), hp.size());
  // symbol-table nodes of at most 2 LEAF_K entries each
  const size_t cap = 2 * LEAF_K;
  std::vector<std::pair<size_t, size_t>> chunks;
  for (size_t i = 0; i < std::max<size_t>(entries.size(), 1); i += cap)
    chunks.push_back({i, std::min(i + cap, entries.size())});
  if (chunks.size() > 2 * INTERNAL_K) throw Error("too many group members for a one-level group B-tree");
  std::vector<uint64_t> snods;
  for (auto &ch : chunks) {
    std::vector<uint8_t> node = {'S', 'N', 'O', 'D', 1, 0};
    put_le<uint16_t>(node, (uint16_t)(ch.second - ch.first));
    for (size_t k = ch.first; k < ch.second; ++k) {
      const Entry &e = entries[k];
      put_le<uint64_t>(node, offs[k]);
      put_le<uint64_t>(node, e.header);
      put_le<uint32_t>(node, e.is_group ? 1 : 0);
      put_le<uint32_t>(node, 0);
      if (e.is_group) {
        put_le<uint64_t>(node, e.btree);
        put_le<uint64_t>(node, e.heap);
      } else {
        node.insert(node.end(), 16, 0);
      }
    }
    node.insert(node.end(), 40 * (cap - (ch.second - ch.first)), 0);
    snods.push_back(alloc(node.data(), node.size()));
  }
  std::vector<uint8_t> tree = {'T', 'R', 'E', 'E', 0, 0};
  put_le<uint16_t>(tree, (uint16_t)snods.size());
  put_le<uint64_t>(tree, UNDEF);
  put_le<uint64_t>(tree, UNDEF);
  put_le<uint64_t>(tree, 0);  // key 0
  for (size_t i = 0; i < snods.size(); ++i) {
    const auto &ch = chunks[i];
    put_le<uint64_t>(tree, snods[i]);
    put_le<uint64_t>(tree, ch.second > ch.first ? offs[ch.second - 1] : 0);
  }
  tree.insert(tree.end(), 16 * (2 * INTERNAL_K - snods.size()), 0);
  *btree = alloc(tree.data(), tree.size());
  std::vector<uint8_t> stmsg;
  put_le<uint64_t>(stmsg, *btree);
  put_le<uint64_t>(stmsg, *heap);
  *header = object_header({msg(0x0011, stmsg)});
}

void Writer::add_group(const std::string &name, const std::vector<Item> &items) {
  std::vector<Entry> ents;
  for (const Item &it : items) ents.push_back({it.name, write_item(it), false, 0, 0});
  Entry g{name, 0, true, 0, 0};
  group(ents, &g.header, &g.btree, &g.heap);
  root_.push_back(g);
}

void Writer::add_dataset(const Item &item) { root_.push_back({item.name, write_item(item), false, 0, 0}); }

void Writer::close() {
  if (!f_) return;
  uint64_t hdr, btree, heap;
  group(root_, &hdr, &btree, &heap);
  std::vector<uint8_t> sb(SIG, SIG + 8);
  const uint8_t v[8] = {0, 0, 0, 0, 0, 8, 8, 0};
  put(sb, v, 8);
  put_le<uint16_t>(sb, LEAF_K);
  put_le<uint16_t>(sb, INTERNAL_K);
  put_le<uint32_t>(sb, 0);
  put_le<uint64_t>(sb, 0);      // base address
  put_le<uint64_t>(sb, UNDEF);  // free-space info
  put_le<uint64_t>(sb, pos_);   // end of file
  put_le<uint64_t>(sb, UNDEF);  // driver info
  put_le<uint64_t>(sb, 0);      // root entry: link name offset
  put_le<uint64_t>(sb, hdr);
  put_le<uint32_t>(sb, 1);
  put_le<uint32_t>(sb, 0);
  put_le<uint64_t>(sb, btree);
  put_le<uint64_t>(sb, heap);
  FILE *f = f_;
  f_ = nullptr;
  if (sb.size() != 96 || fseeko(f, 0, SEEK_SET) != 0 || fwrite(sb.data(), 1, 96, f) != 96) {
    fclose(f);
    throw Error("cannot write the superblock");
  }
  if (fclose(f) != 0) throw Error("close failed");
}

}  // namespace h5min
