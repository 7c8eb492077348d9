// MATLAB MAT-file (level 5) reading and writing for the facade's file forms:
// KData(app, "x.mat"), XData(app, "x.mat"), KData::matlabSave and
// XData::matlabSave.  The reference does this through matio
// (src/Data.cpp:1392-1485, MatVarInfo.cpp, NDArray.cpp:74-130), which is not
// part of this library; this header implements the published level-5 format
// itself, including the zlib-compressed elements matio writes (DEFLATE,
// RFC 1951, inside a zlib stream, RFC 1950), so it needs no other library.
//
// Scope: numeric arrays (double, single, int8..uint64; real or complex) as
// top-level variables, plain or compressed, little-endian files.  Cell,
// struct, sparse, character and object variables are skipped; big-endian and
// HDF5-based (-v7.3) files are refused with std::invalid_argument.  Writing
// produces uncompressed numeric variables, which MATLAB, matio and
// scipy.io read as they read compressed ones.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace OpenCLIPER {
namespace matfile {

// array classes (mxClassID)
enum ClassType : int {
  kDouble = 6,
  kSingle = 7,
  kInt8 = 8,
  kUInt8 = 9,
  kInt16 = 10,
  kUInt16 = 11,
  kInt32 = 12,
  kUInt32 = 13,
  kInt64 = 14,
  kUInt64 = 15
};

// data element types (miTYPE)
enum DataType : uint32_t {
  miINT8 = 1,
  miUINT8 = 2,
  miINT16 = 3,
  miUINT16 = 4,
  miINT32 = 5,
  miUINT32 = 6,
  miSINGLE = 7,
  miDOUBLE = 9,
  miINT64 = 12,
  miUINT64 = 13,
  miMATRIX = 14,
  miCOMPRESSED = 15,
  miUTF8 = 16
};

inline size_t class_bytes(int cls) {
  switch (cls) {
    case kDouble: case kInt64: case kUInt64: return 8;
    case kSingle: case kInt32: case kUInt32: return 4;
    case kInt16: case kUInt16: return 2;
    case kInt8: case kUInt8: return 1;
    default: return 0;
  }
}

/// One numeric variable.  dims are MATLAB's (column-major: dims[0] varies
/// fastest); re / im hold the elements in the class's own type.
struct Var {
  std::string name;
  int cls = 0;
  bool complex = false;
  std::vector<uint64_t> dims;
  std::vector<uint8_t> re, im;
  size_t numel() const {
    size_t n = 1;
    for (uint64_t d : dims) n *= size_t(d);
    return dims.empty() ? 0 : n;
  }
  template <typename T>
  const T* real() const { return reinterpret_cast<const T*>(re.data()); }
  template <typename T>
  const T* imag() const { return reinterpret_cast<const T*>(im.data()); }
};

namespace detail {

[[noreturn]] inline void fail(const std::string& what) { throw std::invalid_argument("MAT file: " + what); }

// ---------------------------------------------------------------------------
// DEFLATE decoder (RFC 1951) for the zlib streams (RFC 1950) of miCOMPRESSED
// elements.  Huffman codes are canonical: decoded with a 9-bit lookup table
// and, for longer codes, by walking the code lengths in order.
// ---------------------------------------------------------------------------
class Inflater {
 public:
  Inflater(const uint8_t* p, size_t n) : p_(p), n_(n) {}

  std::vector<uint8_t> run() {
    if (n_ < 6) fail("truncated zlib stream");
    const unsigned cmf = p_[0], flg = p_[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0) fail("bad zlib header");
    if (flg & 0x20) fail("zlib preset dictionary not supported");
    pos_ = 2;
    bool last = false;
    while (!last) {
      last = bits(1) != 0;
      const unsigned type = bits(2);
      if (type == 0) stored();
      else if (type == 1) fixed();
      else if (type == 2) dynamic();
      else fail("invalid DEFLATE block type");
    }
    // the Adler-32 of the output follows, byte-aligned, most significant byte first
    align();
    if (pos_ + 4 > n_) fail("truncated zlib checksum");
    const uint32_t want = (uint32_t(p_[pos_]) << 24) | (uint32_t(p_[pos_ + 1]) << 16) | (uint32_t(p_[pos_ + 2]) << 8) |
                          uint32_t(p_[pos_ + 3]);
    if (adler32(out_) != want) fail("zlib checksum mismatch");
    return std::move(out_);
  }

  static uint32_t adler32(const std::vector<uint8_t>& v) {
    uint32_t a = 1, b = 0;
    size_t i = 0;
    while (i < v.size()) {
      const size_t end = std::min(v.size(), i + 5552);  // keeps b below 2^32 between reductions
      for (; i < end; ++i) {
        a += v[i];
        b += a;
      }
      a %= 65521u;
      b %= 65521u;
    }
    return (b << 16) | a;
  }

 private:
  struct Huffman {
    std::array<uint16_t, 16> count{};   // codes of each length
    std::vector<uint16_t> symbol;       // symbols ordered by (length, value)
    std::array<uint16_t, 512> fast{};   // 9-bit lookup: (length << 12) | symbol, 0 = not a short code
  };

  unsigned bits(unsigned need) {
    uint32_t v = bitbuf_;
    while (bitcnt_ < need) {
      if (pos_ >= n_) fail("truncated DEFLATE data");
      v |= uint32_t(p_[pos_++]) << bitcnt_;
      bitcnt_ += 8;
    }
    bitbuf_ = v >> need;
    bitcnt_ -= need;
    return v & ((1u << need) - 1u);
  }

  // to the next byte boundary: whole bytes read ahead into the bit buffer go back
  void align() {
    pos_ -= bitcnt_ / 8;
    bitbuf_ = 0;
    bitcnt_ = 0;
  }

  void stored() {
    align();
    if (pos_ + 4 > n_) fail("truncated stored block");
    const unsigned len = p_[pos_] | (unsigned(p_[pos_ + 1]) << 8);
    const unsigned nlen = p_[pos_ + 2] | (unsigned(p_[pos_ + 3]) << 8);
    pos_ += 4;
    if ((len ^ 0xFFFFu) != nlen) fail("stored block length check failed");
    if (pos_ + len > n_) fail("truncated stored block");
    out_.insert(out_.end(), p_ + pos_, p_ + pos_ + len);
    pos_ += len;
  }

  static void build(Huffman& h, const uint8_t* lengths, int n) {
    h.count.fill(0);
    for (int s = 0; s < n; ++s) h.count[lengths[s]]++;
    h.count[0] = 0;
    // first[len] = index of the first symbol of length len in `symbol`
    std::array<uint16_t, 16> first{};
    int total = 0;
    for (int len = 1; len < 16; ++len) {
      first[len] = uint16_t(total);
      total += h.count[len];
    }
    h.symbol.assign(size_t(total), 0);
    std::array<uint16_t, 16> next = first;
    for (int s = 0; s < n; ++s)
      if (lengths[s]) h.symbol[next[lengths[s]]++] = uint16_t(s);
    // canonical codes: consecutive values within a length, shifted left between lengths
    h.fast.fill(0);
    unsigned code = 0, idx = 0;
    for (int len = 1; len <= 9; ++len) {
      for (unsigned k = 0; k < h.count[len]; ++k, ++code, ++idx) {
        // DEFLATE sends Huffman codes most significant bit first into an LSB-first stream
        unsigned rev = 0;
        for (int b = 0; b < len; ++b) rev |= ((code >> b) & 1u) << (len - 1 - b);
        for (unsigned fill = rev; fill < 512; fill += (1u << len))
          h.fast[fill] = uint16_t((len << 12) | h.symbol[idx]);
      }
      code <<= 1;
    }
  }

  int decode(const Huffman& h) {
    // fast path: a code of at most 9 bits, when 9 bits are available
    while (bitcnt_ < 9 && pos_ < n_) {
      bitbuf_ |= uint32_t(p_[pos_++]) << bitcnt_;
      bitcnt_ += 8;
    }
    if (bitcnt_ >= 9) {
      const uint16_t e = h.fast[bitbuf_ & 511u];
      if (e) {
        const unsigned len = e >> 12;
        bitbuf_ >>= len;
        bitcnt_ -= len;
        return e & 0xFFF;
      }
    }
    // slow path: one bit at a time through the canonical code ranges
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= int(bits(1));
      const int count = h.count[len];
      if (code - first < count) return h.symbol[size_t(index + code - first)];
      index += count;
      first = (first + count) << 1;
      code <<= 1;
    }
    fail("invalid Huffman code");
  }

  void codes(const Huffman& lit, const Huffman& dist) {
    // RFC 1951 section 3.2.5: base lengths / distances and their extra bits
    static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                       31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
      int sym = decode(lit);
      if (sym < 256) {
        out_.push_back(uint8_t(sym));
      } else if (sym == 256) {
        return;
      } else {
        sym -= 257;
        if (sym >= 29) fail("invalid length symbol");
        const size_t len = lbase[sym] + bits(lext[sym]);
        const int ds = decode(dist);
        if (ds >= 30) fail("invalid distance symbol");
        const size_t d = dbase[ds] + bits(dext[ds]);
        if (d > out_.size()) fail("distance before the start of the data");
        const size_t from = out_.size() - d;
        for (size_t k = 0; k < len; ++k) out_.push_back(out_[from + k]);  // may overlap its own output
      }
    }
  }

  void fixed() {
    if (!fixed_ready_) {
      uint8_t l[288];
      for (int s = 0; s < 144; ++s) l[s] = 8;
      for (int s = 144; s < 256; ++s) l[s] = 9;
      for (int s = 256; s < 280; ++s) l[s] = 7;
      for (int s = 280; s < 288; ++s) l[s] = 8;
      build(fixed_lit_, l, 288);
      uint8_t d[30];
      for (int s = 0; s < 30; ++s) d[s] = 5;
      build(fixed_dist_, d, 30);
      fixed_ready_ = true;
    }
    codes(fixed_lit_, fixed_dist_);
  }

  void dynamic() {
    static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    const unsigned nlen = bits(5) + 257, ndist = bits(5) + 1, ncode = bits(4) + 4;
    if (nlen > 286 || ndist > 30) fail("bad dynamic block counts");
    uint8_t lengths[320] = {0};
    for (unsigned i = 0; i < ncode; ++i) lengths[order[i]] = uint8_t(bits(3));
    Huffman lencode;
    build(lencode, lengths, 19);
    unsigned idx = 0;
    std::memset(lengths, 0, sizeof(lengths));
    while (idx < nlen + ndist) {
      const int sym = decode(lencode);
      if (sym < 16) {
        lengths[idx++] = uint8_t(sym);
      } else {
        uint8_t val = 0;
        unsigned rep;
        if (sym == 16) {
          if (idx == 0) fail("repeat with no previous length");
          val = lengths[idx - 1];
          rep = 3 + bits(2);
        } else if (sym == 17) {
          rep = 3 + bits(3);
        } else {
          rep = 11 + bits(7);
        }
        if (idx + rep > nlen + ndist) fail("too many code lengths");
        while (rep--) lengths[idx++] = val;
      }
    }
    if (lengths[256] == 0) fail("no end-of-block code");
    Huffman lit, dist;
    build(lit, lengths, int(nlen));
    build(dist, lengths + nlen, int(ndist));
    codes(lit, dist);
  }

  const uint8_t* p_;
  size_t n_, pos_ = 0;
  uint32_t bitbuf_ = 0;
  unsigned bitcnt_ = 0;
  std::vector<uint8_t> out_;
  Huffman fixed_lit_, fixed_dist_;
  bool fixed_ready_ = false;
};

inline uint32_t rd32(const uint8_t* p) {
  return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}

// one data element: type, payload and the offset just past it (8-byte padded
// inside a matrix; compressed top-level elements are not padded)
struct Element {
  uint32_t type;
  const uint8_t* data;
  size_t bytes;
  size_t next;
};

inline Element element(const uint8_t* p, size_t n, size_t off, bool pad) {
  if (off + 8 > n) fail("truncated data element tag");
  const uint32_t w0 = rd32(p + off);
  if (w0 >> 16) {  // small data element: 2-byte size, 2-byte type, 4 bytes of data
    const uint32_t bytes = w0 >> 16;
    if (bytes > 4) fail("bad small data element");
    return Element{w0 & 0xFFFFu, p + off + 4, bytes, off + 8};
  }
  const size_t bytes = rd32(p + off + 4);
  if (off + 8 + bytes > n) fail("truncated data element");
  size_t next = off + 8 + bytes;
  if (pad) next = (next + 7) & ~size_t(7);
  return Element{w0, p + off + 8, bytes, next};
}

inline size_t mi_bytes(uint32_t t) {
  switch (t) {
    case miINT8: case miUINT8: return 1;
    case miINT16: case miUINT16: return 2;
    case miINT32: case miUINT32: case miSINGLE: return 4;
    case miDOUBLE: case miINT64: case miUINT64: return 8;
    default: return 0;
  }
}

template <typename D>
void convert_from(const Element& e, size_t count, D* out) {
  const size_t sz = mi_bytes(e.type);
  if (!sz || e.bytes < count * sz) fail("numeric data shorter than the array");
  for (size_t i = 0; i < count; ++i) {
    const uint8_t* q = e.data + i * sz;
    switch (e.type) {
      case miINT8: { int8_t v; std::memcpy(&v, q, 1); out[i] = D(v); break; }
      case miUINT8: { out[i] = D(*q); break; }
      case miINT16: { int16_t v; std::memcpy(&v, q, 2); out[i] = D(v); break; }
      case miUINT16: { uint16_t v; std::memcpy(&v, q, 2); out[i] = D(v); break; }
      case miINT32: { int32_t v; std::memcpy(&v, q, 4); out[i] = D(v); break; }
      case miUINT32: { uint32_t v; std::memcpy(&v, q, 4); out[i] = D(v); break; }
      case miSINGLE: { float v; std::memcpy(&v, q, 4); out[i] = D(v); break; }
      case miDOUBLE: { double v; std::memcpy(&v, q, 8); out[i] = D(v); break; }
      case miINT64: { int64_t v; std::memcpy(&v, q, 8); out[i] = D(v); break; }
      case miUINT64: { uint64_t v; std::memcpy(&v, q, 8); out[i] = D(v); break; }
      default: fail("unsupported numeric data type");
    }
  }
}

// the element's values converted to the array class (MATLAB may store an
// array in a smaller type than its class)
inline std::vector<uint8_t> numeric(const Element& e, int cls, size_t count) {
  std::vector<uint8_t> v(count * class_bytes(cls));
  switch (cls) {
    case kDouble: convert_from(e, count, reinterpret_cast<double*>(v.data())); break;
    case kSingle: convert_from(e, count, reinterpret_cast<float*>(v.data())); break;
    case kInt8: convert_from(e, count, reinterpret_cast<int8_t*>(v.data())); break;
    case kUInt8: convert_from(e, count, reinterpret_cast<uint8_t*>(v.data())); break;
    case kInt16: convert_from(e, count, reinterpret_cast<int16_t*>(v.data())); break;
    case kUInt16: convert_from(e, count, reinterpret_cast<uint16_t*>(v.data())); break;
    case kInt32: convert_from(e, count, reinterpret_cast<int32_t*>(v.data())); break;
    case kUInt32: convert_from(e, count, reinterpret_cast<uint32_t*>(v.data())); break;
    case kInt64: convert_from(e, count, reinterpret_cast<int64_t*>(v.data())); break;
    case kUInt64: convert_from(e, count, reinterpret_cast<uint64_t*>(v.data())); break;
    default: fail("unsupported array class");
  }
  return v;
}

// parses the payload of an miMATRIX element; false for classes this reader skips
inline bool matrix(const uint8_t* p, size_t n, Var& v) {
  if (n == 0) return false;  // an empty matrix element
  const Element flags = element(p, n, 0, true);
  if (flags.type != miUINT32 || flags.bytes < 8) fail("bad array flags");
  const uint32_t f = rd32(flags.data);
  v.cls = int(f & 0xFF);
  v.complex = (f & 0x0800u) != 0;
  const Element dims = element(p, n, flags.next, true);
  if (dims.type != miINT32 || dims.bytes < 8 || dims.bytes % 4) fail("bad dimensions");
  v.dims.clear();
  for (size_t i = 0; i < dims.bytes / 4; ++i) {
    int32_t d;
    std::memcpy(&d, dims.data + 4 * i, 4);
    if (d < 0) fail("negative dimension");
    v.dims.push_back(uint64_t(d));
  }
  const Element name = element(p, n, dims.next, true);
  if (name.type != miINT8 && name.type != miUINT8) fail("bad array name");
  v.name.assign(reinterpret_cast<const char*>(name.data), name.bytes);
  if (!class_bytes(v.cls)) return false;  // cell, struct, char, sparse, object: skipped
  const size_t count = v.numel();
  const Element re = element(p, n, name.next, true);
  v.re = numeric(re, v.cls, count);
  v.im.clear();
  if (v.complex) {
    const Element im = element(p, n, re.next, true);
    v.im = numeric(im, v.cls, count);
  }
  return true;
}

inline std::vector<uint8_t> slurp(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::invalid_argument("Error opening MAT file '" + path + "'!");
  return std::vector<uint8_t>((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

inline void put32(std::vector<uint8_t>& o, uint32_t v) {
  for (int i = 0; i < 4; ++i) o.push_back(uint8_t(v >> (8 * i)));
}
inline void pad8(std::vector<uint8_t>& o) {
  while (o.size() % 8) o.push_back(0);
}
inline void put_element(std::vector<uint8_t>& o, uint32_t type, const void* data, size_t bytes) {
  put32(o, type);
  put32(o, uint32_t(bytes));
  const uint8_t* b = static_cast<const uint8_t*>(data);
  o.insert(o.end(), b, b + bytes);
  pad8(o);
}
inline uint32_t mi_of_class(int cls) {
  switch (cls) {
    case kDouble: return miDOUBLE;
    case kSingle: return miSINGLE;
    case kInt8: return miINT8;
    case kUInt8: return miUINT8;
    case kInt16: return miINT16;
    case kUInt16: return miUINT16;
    case kInt32: return miINT32;
    case kUInt32: return miUINT32;
    case kInt64: return miINT64;
    case kUInt64: return miUINT64;
    default: fail("unsupported array class");
  }
}

}  // namespace detail

/// zlib stream -> bytes (exposed for tests).
inline std::vector<uint8_t> zlib_inflate(const uint8_t* p, size_t n) { return detail::Inflater(p, n).run(); }

/// True when the file starts like a level-5 MAT-file.
inline bool is_mat(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  char h[128];
  if (!in.read(h, 128)) return false;
  return std::memcmp(h, "MATLAB", 6) == 0 && (std::memcmp(h + 126, "IM", 2) == 0 || std::memcmp(h + 126, "MI", 2) == 0);
}

/// All numeric top-level variables of a level-5 MAT-file, by name.
inline std::map<std::string, Var> read(const std::string& path) {
  const std::vector<uint8_t> f = detail::slurp(path);
  if (f.size() < 128 || std::memcmp(f.data(), "MATLAB", 6) != 0)
    throw std::invalid_argument("Error opening MAT file '" + path + "'!");
  if (std::memcmp(f.data() + 126, "MI", 2) == 0) detail::fail("big-endian files are not supported");
  if (std::memcmp(f.data() + 126, "IM", 2) != 0) detail::fail(path + " is not a level-5 MAT-file (e.g. -v7.3)");
  std::map<std::string, Var> vars;
  size_t off = 128;
  while (off + 8 <= f.size()) {
    const detail::Element e = detail::element(f.data(), f.size(), off, false);
    off = e.next;
    std::vector<uint8_t> inflated;
    const uint8_t* mp = nullptr;
    size_t mn = 0;
    if (e.type == miCOMPRESSED) {
      inflated = zlib_inflate(e.data, e.bytes);
      const detail::Element inner = detail::element(inflated.data(), inflated.size(), 0, false);
      if (inner.type != miMATRIX) continue;
      mp = inner.data;
      mn = inner.bytes;
    } else if (e.type == miMATRIX) {
      mp = e.data;
      mn = e.bytes;
      off = (off + 7) & ~size_t(7);
    } else {
      off = (off + 7) & ~size_t(7);
      continue;
    }
    Var v;
    if (detail::matrix(mp, mn, v)) {
      if (v.dims.size() < 2) detail::fail("invalid rank in variable " + v.name);
      vars[v.name] = std::move(v);
    }
  }
  return vars;
}

/// Writes the variables (uncompressed) to a new level-5 MAT-file.
inline void write(const std::string& path, const std::vector<Var>& vars) {
  std::vector<uint8_t> o;
  std::string text = "MATLAB 5.0 MAT-file, Platform: OpenCLIPER GB300 facade, Created by: gbn_matfile.hpp";
  text.resize(116, ' ');
  o.insert(o.end(), text.begin(), text.end());
  for (int i = 0; i < 8; ++i) o.push_back(0);  // no subsystem data
  o.push_back(0x00);
  o.push_back(0x01);  // version 0x0100
  o.push_back('I');
  o.push_back('M');
  for (const Var& v : vars) {
    const size_t esz = class_bytes(v.cls);
    if (!esz) detail::fail("cannot write class " + std::to_string(v.cls));
    if (v.dims.size() < 2) detail::fail("variable " + v.name + " needs at least two dimensions");
    const size_t count = v.numel();
    if (v.re.size() != count * esz || (v.complex && v.im.size() != count * esz))
      detail::fail("variable " + v.name + ": data size does not match its dimensions");
    std::vector<uint8_t> m;
    const uint32_t flags[2] = {uint32_t(v.cls) | (v.complex ? 0x0800u : 0u), 0u};
    detail::put_element(m, miUINT32, flags, 8);
    std::vector<int32_t> d;
    for (uint64_t x : v.dims) {
      if (x > 0x7FFFFFFFull) detail::fail("dimension too large");
      d.push_back(int32_t(x));
    }
    detail::put_element(m, miINT32, d.data(), d.size() * 4);
    detail::put_element(m, miINT8, v.name.data(), v.name.size());
    const uint32_t mt = detail::mi_of_class(v.cls);
    detail::put_element(m, mt, v.re.data(), v.re.size());
    if (v.complex) detail::put_element(m, mt, v.im.data(), v.im.size());
    detail::put32(o, miMATRIX);
    detail::put32(o, uint32_t(m.size()));
    o.insert(o.end(), m.begin(), m.end());
  }
  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) throw std::invalid_argument("Error creating MAT file " + path);
  out.write(reinterpret_cast<const char*>(o.data()), std::streamsize(o.size()));
  if (!out) throw std::invalid_argument("Error writing MAT file " + path);
}

// ---- layout helpers: MATLAB's column-major slices <-> row-major [rows][cols] ----

/// Builds a variable from row-major [slices][rows][cols] data of type T
/// (MATLAB dims = rows, cols, then `outer`), transposing each slice.
template <typename T>
Var from_row_major(const std::string& name, int cls, const T* re, const T* im, size_t rows, size_t cols,
                   const std::vector<uint64_t>& outer) {
  Var v;
  v.name = name;
  v.cls = cls;
  v.complex = im != nullptr;
  v.dims = {rows, cols};
  size_t slices = 1;
  for (uint64_t d : outer) {
    v.dims.push_back(d);
    slices *= size_t(d);
  }
  const size_t plane = rows * cols;
  v.re.resize(plane * slices * sizeof(T));
  if (im) v.im.resize(plane * slices * sizeof(T));
  T* ore = reinterpret_cast<T*>(v.re.data());
  T* oim = im ? reinterpret_cast<T*>(v.im.data()) : nullptr;
  for (size_t s = 0; s < slices; ++s)
    for (size_t r = 0; r < rows; ++r)
      for (size_t c = 0; c < cols; ++c) {
        ore[s * plane + c * rows + r] = re[s * plane + r * cols + c];
        if (im) oim[s * plane + c * rows + r] = im[s * plane + r * cols + c];
      }
  return v;
}

/// Row-major [slices][rows][cols] copy of a variable whose MATLAB dims start
/// with (rows, cols); `out_im` may be null.
template <typename T>
void to_row_major(const Var& v, std::vector<T>& out_re, std::vector<T>* out_im) {
  const size_t rows = size_t(v.dims[0]), cols = size_t(v.dims[1]);
  const size_t plane = rows * cols, slices = plane ? v.numel() / plane : 0;
  out_re.resize(plane * slices);
  if (out_im) out_im->assign(plane * slices, T(0));
  const T* re = v.real<T>();
  const T* im = v.complex ? v.imag<T>() : nullptr;
  for (size_t s = 0; s < slices; ++s)
    for (size_t r = 0; r < rows; ++r)
      for (size_t c = 0; c < cols; ++c) {
        out_re[s * plane + r * cols + c] = re[s * plane + c * rows + r];
        if (out_im && im) (*out_im)[s * plane + r * cols + c] = im[s * plane + c * rows + r];
      }
}

}  // namespace matfile
}  // namespace OpenCLIPER
