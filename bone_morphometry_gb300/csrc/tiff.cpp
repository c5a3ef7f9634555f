// Multi-page 8-bit grayscale TIFF decoding into caller buffers (tiff_io.rs:33-149).
//
// The reference reads the bone and ROI stacks with the `tiff` crate (0.11.3):
// every page must be Gray(8) with the first page's dimensions, the decoded
// samples are validated (any value, strictly 0/255, or 0/1/255 for ROI masks)
// and stored as u8 (sample > threshold).  This reader covers the encodings
// that crate decodes for such pages -- classic and BigTIFF, either byte order,
// strips or tiles, no compression, PackBits, LZW (MSB-first, early code-width
// change) and Deflate (zlib), with or without horizontal differencing -- and
// writes straight into the caller's buffer (pinned host memory for the GPU
// path).  Pages are decoded in parallel; errors carry the reference's texts
// and report the first failing page, as its sequential loop would.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "bm.h"

namespace bm {

void set_thread_error(const char* msg);  // api.cu

namespace {

struct TiffError {
  int status;
  std::string msg;
};

std::string fmt(const char* f, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, f);
  std::vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}

// ---- file and IFD access --------------------------------------------------

struct Mapped {
  const uint8_t* p = nullptr;
  size_t n = 0;
  int fd = -1;
  ~Mapped() {
    if (p && n) munmap(const_cast<uint8_t*>(p), n);
    if (fd >= 0) close(fd);
  }
};

struct Entry {
  uint16_t tag = 0, type = 0;
  uint64_t count = 0;
  uint64_t value_or_offset = 0;  // raw field (inline value bytes or offset)
  size_t field_pos = 0;          // file position of the value field
};

struct Page {
  uint64_t width = 0, height = 0;
  uint32_t bits = 1, spp = 1, photometric = 1, compression = 1, predictor = 1, planar = 1, sample_format = 1;
  bool has_photometric = false;
  bool tiled = false;
  uint64_t rows_per_strip = 0, tile_w = 0, tile_h = 0;
  std::vector<uint64_t> offsets, counts;
};

class File {
 public:
  File(const uint8_t* p, size_t n, const std::string& path) : p_(p), n_(n), path_(path) {}

  void header(uint64_t* first_ifd) {
    if (n_ < 8) throw TiffError{BM_ERR_INVALID, fmt("initializing TIFF decoder for %s: file too short", path_.c_str())};
    if (p_[0] == 'I' && p_[1] == 'I') le_ = true;
    else if (p_[0] == 'M' && p_[1] == 'M') le_ = false;
    else throw TiffError{BM_ERR_INVALID, fmt("initializing TIFF decoder for %s: not a TIFF file", path_.c_str())};
    const uint16_t magic = u16(2);
    if (magic == 42) {
      big_ = false;
      *first_ifd = u32(4);
    } else if (magic == 43) {
      big_ = true;
      if (n_ < 16 || u16(4) != 8)
        throw TiffError{BM_ERR_INVALID, fmt("initializing TIFF decoder for %s: bad BigTIFF header", path_.c_str())};
      *first_ifd = u64(8);
    } else {
      throw TiffError{BM_ERR_INVALID, fmt("initializing TIFF decoder for %s: not a TIFF file", path_.c_str())};
    }
  }

  // Parses the IFD at off into entries; returns the next IFD offset.
  uint64_t ifd(uint64_t off, std::vector<Entry>& out) {
    out.clear();
    const size_t esz = big_ ? 20 : 12;
    const size_t csz = big_ ? 8 : 2;
    need(off, csz);
    const uint64_t cnt = big_ ? u64(off) : u16(off);
    need(off + csz, cnt * esz + (big_ ? 8 : 4));
    for (uint64_t i = 0; i < cnt; ++i) {
      const size_t e = off + csz + i * esz;
      Entry en;
      en.tag = u16(e);
      en.type = u16(e + 2);
      en.count = big_ ? u64(e + 4) : u32(e + 4);
      en.field_pos = e + (big_ ? 12 : 8);
      out.push_back(en);
    }
    const size_t nx = off + csz + cnt * esz;
    return big_ ? u64(nx) : u32(nx);
  }

  static size_t type_size(uint16_t t) {
    switch (t) {
      case 1: case 2: case 6: case 7: return 1;
      case 3: case 8: return 2;
      case 4: case 9: case 11: case 13: return 4;
      case 5: case 10: case 12: case 16: case 17: case 18: return 8;
      default: return 0;
    }
  }

  // Unsigned integer values of an entry (BYTE, SHORT, LONG, LONG8 and IFD types).
  std::vector<uint64_t> uints(const Entry& en) {
    const size_t ts = type_size(en.type);
    if (en.count == 0 || en.count > n_)
      throw TiffError{BM_ERR_INVALID, fmt("tag %u of %s has an invalid value count", en.tag, path_.c_str())};
    if (ts == 0 || en.type == 2 || en.type == 5 || en.type == 10 || en.type == 11 || en.type == 12)
      throw TiffError{BM_ERR_INVALID, fmt("tag %u of %s has a non-integer type", en.tag, path_.c_str())};
    const uint64_t bytes = ts * en.count;
    const size_t inl = big_ ? 8 : 4;
    size_t pos = en.field_pos;
    if (bytes > inl) pos = big_ ? u64(en.field_pos) : u32(en.field_pos);
    need(pos, bytes);
    std::vector<uint64_t> v(en.count);
    for (uint64_t i = 0; i < en.count; ++i) {
      const size_t q = pos + i * ts;
      switch (ts) {
        case 1: v[i] = p_[q]; break;
        case 2: v[i] = u16(q); break;
        case 4: v[i] = u32(q); break;
        default: v[i] = u64(q); break;
      }
    }
    return v;
  }

  void need(uint64_t off, uint64_t len) const {
    if (off > n_ || len > n_ - off)
      throw TiffError{BM_ERR_INVALID, fmt("%s: TIFF structure points past the end of the file", path_.c_str())};
  }

  const uint8_t* at(uint64_t off, uint64_t len) const {
    need(off, len);
    return p_ + off;
  }

  uint16_t u16(size_t o) const {
    need(o, 2);
    return le_ ? (uint16_t)(p_[o] | (p_[o + 1] << 8)) : (uint16_t)((p_[o] << 8) | p_[o + 1]);
  }
  uint32_t u32(size_t o) const {
    need(o, 4);
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)p_[o + (le_ ? i : 3 - i)] << (8 * i);
    return v;
  }
  uint64_t u64(size_t o) const {
    need(o, 8);
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p_[o + (le_ ? i : 7 - i)] << (8 * i);
    return v;
  }

 private:
  const uint8_t* p_;
  size_t n_;
  std::string path_;
  bool le_ = true, big_ = false;
};

Page parse_page(File& f, const std::vector<Entry>& ents) {
  Page pg;
  bool have_w = false, have_h = false;
  for (const Entry& en : ents) {
    switch (en.tag) {
      case 256: pg.width = f.uints(en)[0]; have_w = true; break;
      case 257: pg.height = f.uints(en)[0]; have_h = true; break;
      case 258: {
        const auto v = f.uints(en);
        pg.bits = (uint32_t)v[0];
        for (uint64_t b : v)
          if (b != v[0]) pg.bits = 0;  // mixed sample sizes: unsupported
        break;
      }
      case 259: pg.compression = (uint32_t)f.uints(en)[0]; break;
      case 262: pg.photometric = (uint32_t)f.uints(en)[0]; pg.has_photometric = true; break;
      case 273: pg.offsets = f.uints(en); break;
      case 277: pg.spp = (uint32_t)f.uints(en)[0]; break;
      case 278: pg.rows_per_strip = f.uints(en)[0]; break;
      case 279: pg.counts = f.uints(en); break;
      case 284: pg.planar = (uint32_t)f.uints(en)[0]; break;
      case 317: pg.predictor = (uint32_t)f.uints(en)[0]; break;
      case 322: pg.tile_w = f.uints(en)[0]; pg.tiled = true; break;
      case 323: pg.tile_h = f.uints(en)[0]; pg.tiled = true; break;
      case 324: pg.offsets = f.uints(en); pg.tiled = true; break;
      case 325: pg.counts = f.uints(en); pg.tiled = true; break;
      case 339: pg.sample_format = (uint32_t)f.uints(en)[0]; break;
      default: break;
    }
  }
  if (!have_w || !have_h) throw TiffError{BM_ERR_INVALID, "required ImageWidth/ImageLength tag missing"};
  return pg;
}

// The tiff crate's colour-type name of a page (as its Debug text), or "" for Gray(8).
std::string color_type(const Page& pg) {
  const unsigned b = pg.bits;
  switch (pg.photometric) {
    case 0:
    case 1:
      if (pg.spp == 1) return b == 8 ? std::string() : fmt("Gray(%u)", b);
      if (pg.spp == 2) return fmt("GrayA(%u)", b);
      break;
    case 2:
      if (pg.spp == 3) return fmt("RGB(%u)", b);
      if (pg.spp == 4) return fmt("RGBA(%u)", b);
      break;
    case 3: return fmt("Palette(%u)", b);
    case 5: return fmt("CMYK(%u)", b);
    case 6: return fmt("YCbCr(%u)", b);
    default: break;
  }
  return fmt("Unsupported(photometric %u, %u samples of %u bits)", pg.photometric, pg.spp, b);
}

// ---- decompressors ----------------------------------------------------------

void unpackbits(const uint8_t* in, size_t n, uint8_t* out, size_t cap) {
  size_t i = 0, o = 0;
  while (i < n && o < cap) {
    const int c = (int8_t)in[i++];
    if (c >= 0) {
      const size_t k = (size_t)c + 1;
      if (i + k > n) throw TiffError{BM_ERR_INVALID, "PackBits literal run past the end of the data"};
      const size_t m = std::min(k, cap - o);
      std::memcpy(out + o, in + i, m);
      i += k;
      o += m;
    } else if (c != -128) {
      if (i >= n) throw TiffError{BM_ERR_INVALID, "PackBits repeat past the end of the data"};
      const size_t k = (size_t)(1 - c);
      const size_t m = std::min(k, cap - o);
      std::memset(out + o, in[i++], m);
      o += m;
    }
  }
  if (o < cap) throw TiffError{BM_ERR_INVALID, "PackBits data too short for the strip"};
}

// TIFF LZW: codes of 9..12 bits, most significant bit first, ClearCode 256,
// EndOfInformation 257, code width growing one code early (TIFF 6.0).
void unlzw(const uint8_t* in, size_t n, uint8_t* out, size_t cap) {
  std::vector<uint16_t> prefix(4096);
  std::vector<uint8_t> suffix(4096), first(4096);
  std::vector<uint16_t> len(4096);
  for (int i = 0; i < 256; ++i) {
    suffix[i] = first[i] = (uint8_t)i;
    len[i] = 1;
  }
  size_t o = 0;
  uint64_t bitbuf = 0;
  int bits = 0;
  size_t pos = 0;
  int width = 9, next = 258, prev = -1;
  std::vector<uint8_t> stack(4096);
  while (o < cap) {
    while (bits < width) {
      if (pos >= n) goto done;  // data ended without EndOfInformation
      bitbuf = (bitbuf << 8) | in[pos++];
      bits += 8;
    }
    {
      const int code = (int)((bitbuf >> (bits - width)) & ((1u << width) - 1));
      bits -= width;
      if (code == 256) {
        width = 9;
        next = 258;
        prev = -1;
        continue;
      }
      if (code == 257) break;
      int cur;
      if (code < next && (code < 256 || code >= 258)) {
        cur = code;
      } else if (code == next && prev >= 0) {
        cur = -1;  // KwKwK: prev's string plus its own first byte
      } else {
        throw TiffError{BM_ERR_INVALID, "invalid LZW code"};
      }
      const int src = cur >= 0 ? cur : prev;
      int k = len[src];
      int c = src;
      for (int j = k - 1; j >= 0; --j) {
        stack[j] = suffix[c];
        c = prefix[c];
      }
      if (cur < 0) stack[k++] = first[prev];
      const size_t m = std::min((size_t)k, cap - o);
      std::memcpy(out + o, stack.data(), m);
      o += m;
      if (prev >= 0 && next < 4096) {
        prefix[next] = (uint16_t)prev;
        suffix[next] = stack[0];
        first[next] = first[prev];
        len[next] = (uint16_t)(len[prev] + 1);
        ++next;
      }
      prev = cur >= 0 ? cur : next - 1;
      if (next + 1 >= (1 << width) && width < 12) ++width;
    }
  }
done:
  if (o < cap) throw TiffError{BM_ERR_INVALID, "LZW data too short for the strip"};
}

// Deflate decoding (RFC 1950 zlib framing around RFC 1951 data).
//
// Design: each prefix code is expanded into a two-level lookup table.  The
// root level is indexed by the next `root` input bits (9 for literals and
// lengths, 6 for distances, 7 for the code-length code); codes no longer than
// that fill every root slot they prefix, and each longer code's first `root`
// bits select a root slot that links to a second-level table sized for the
// longest code sharing that prefix.  A symbol therefore costs one or two table
// reads and one bit-buffer shift, and building a dynamic block's tables
// writes a few hundred slots.  Deflate sends Huffman codes most significant
// bit first inside an LSB-first bit stream, so a code is stored reversed.
// The length and distance symbols' base values are derived from their
// extra-bit counts (RFC 1951 3.2.5: each base is the previous base plus the
// span of the previous symbol's extra bits).
class DeflateStream {
 public:
  DeflateStream(const uint8_t* src, size_t src_len, uint8_t* dst, size_t dst_len)
      : src_(src), src_len_(src_len), dst_(dst), dst_len_(dst_len) {}

  // Decodes until the destination is full; fails on malformed data or when
  // the stream ends first.
  void decode_all() {
    if (src_len_ < 2) bad("zlib stream too short");
    const unsigned cmf = src_[0], flg = src_[1];
    // method 8 (deflate), header checksum, and no preset dictionary
    if ((cmf & 15u) != 8u || ((cmf << 8) | flg) % 31u != 0u || (flg & 32u)) bad("bad zlib header");
    next_byte_ = 2;
    bool final_block = false;
    while (!final_block && produced_ < dst_len_) {
      final_block = take(1) != 0;
      switch (take(2)) {
        case 0: raw_block(); break;
        case 1: fixed_tables(); inflate_block(); break;
        case 2: dynamic_tables(); inflate_block(); break;
        default: bad("invalid deflate block type");
      }
    }
    if (produced_ < dst_len_) bad("deflate data too short for the strip");
  }

 private:
  static constexpr int kMaxBits = 15;

  // Slot encoding: bit 31 set = link {second-level offset in bits 8..30,
  // its index width in bits 0..7}; otherwise a leaf {symbol in bits 8..30,
  // code bits consumed at this level in bits 0..7}; 0 = no code.
  struct Table {
    int root = 0;
    std::vector<uint32_t> slot;

    void assign(const uint8_t* len, int nsym, int root_bits) {
      root = root_bits;
      int per_len[kMaxBits + 1] = {0};
      for (int i = 0; i < nsym; ++i) per_len[len[i]]++;
      per_len[0] = 0;
      // canonical code assignment (RFC 1951 3.2.2): shorter codes first, then by symbol
      unsigned next_code[kMaxBits + 1] = {0};
      unsigned c = 0;
      long space = 1;  // Kraft check in units of 2^-l
      for (int l = 1; l <= kMaxBits; ++l) {
        c = (c + (unsigned)per_len[l - 1]) << 1;
        next_code[l] = c;
        space = (space << 1) - per_len[l];
        if (space < 0) throw TiffError{BM_ERR_INVALID, "over-subscribed deflate code"};
      }
      std::vector<uint32_t> rev(nsym, 0);
      for (int sym = 0; sym < nsym; ++sym) {
        const int l = len[sym];
        if (!l) continue;
        const unsigned code = next_code[l]++;
        unsigned r = 0;
        for (int b = 0; b < l; ++b) r |= ((code >> b) & 1u) << (l - 1 - b);
        rev[sym] = r;
      }
      const uint32_t rmask = (1u << root) - 1u;
      slot.assign((size_t)1 << root, 0u);
      // second-level widths per root prefix, then their offsets
      std::vector<uint8_t> width((size_t)1 << root, 0);
      for (int sym = 0; sym < nsym; ++sym)
        if (len[sym] > root) {
          const uint32_t p = rev[sym] & rmask;
          width[p] = (uint8_t)std::max<int>(width[p], len[sym] - root);
        }
      for (uint32_t p = 0; p <= rmask; ++p)
        if (width[p]) {
          slot[p] = 0x80000000u | ((uint32_t)slot.size() << 8) | width[p];
          slot.resize(slot.size() + ((size_t)1 << width[p]), 0u);
        }
      for (int sym = 0; sym < nsym; ++sym) {
        const int l = len[sym];
        if (!l) continue;
        if (l <= root) {
          for (uint32_t k = rev[sym]; k <= rmask; k += 1u << l) slot[k] = ((uint32_t)sym << 8) | (uint32_t)l;
        } else {
          const uint32_t link = slot[rev[sym] & rmask];
          const uint32_t base = (link & 0x7fffffffu) >> 8, w = link & 0xffu;
          const uint32_t sub = l - root;
          for (uint32_t k = rev[sym] >> root; k < (1u << w); k += 1u << sub)
            slot[base + k] = ((uint32_t)sym << 8) | sub;
        }
      }
    }
  };

  // Base value and extra-bit count of the 29 length and 30 distance symbols.
  struct Bases {
    uint16_t len_base[29], dist_base[30];
    uint8_t len_extra[29], dist_extra[30];
    Bases() {
      int b = 3;
      for (int i = 0; i < 28; ++i) {  // 8 symbols without extra bits, then 4 per extra bit count 1..5
        len_extra[i] = (uint8_t)(i < 8 ? 0 : i / 4 - 1);
        len_base[i] = (uint16_t)b;
        b += 1 << len_extra[i];
      }
      len_base[28] = 258;  // symbol 285
      len_extra[28] = 0;
      int d = 1;
      for (int i = 0; i < 30; ++i) {  // 4 symbols without extra bits, then 2 per extra bit count 1..13
        dist_extra[i] = (uint8_t)(i < 4 ? 0 : i / 2 - 1);
        dist_base[i] = (uint16_t)d;
        d += 1 << dist_extra[i];
      }
    }
  };
  static const Bases& bases() {
    static const Bases b;
    return b;
  }

  [[noreturn]] void bad(const char* what) { throw TiffError{BM_ERR_INVALID, what}; }

  // Keeps at least `n` (<= 32) bits in the buffer; past the end of the input
  // the buffer is padded with zero bits, and consuming a padded bit fails.
  void fill(int n) {
    while (have_ < n) {
      const uint64_t byte = next_byte_ < src_len_ ? src_[next_byte_] : 0u;
      ++next_byte_;
      acc_ |= byte << have_;
      have_ += 8;
    }
  }
  void drop(int n) {
    acc_ >>= n;
    have_ -= n;
    if (next_byte_ > src_len_ && (next_byte_ - src_len_) * 8 > (size_t)have_) bad("deflate data ended early");
  }
  unsigned take(int n) {
    if (n == 0) return 0;
    fill(n);
    const unsigned v = (unsigned)(acc_ & ((1ull << n) - 1));
    drop(n);
    return v;
  }
  int symbol(const Table& t) {
    fill(kMaxBits);
    uint32_t e = t.slot[acc_ & ((1u << t.root) - 1u)];
    if (e & 0x80000000u) {
      drop(t.root);
      e = t.slot[((e & 0x7fffffffu) >> 8) + (acc_ & ((1u << (e & 0xffu)) - 1u))];
    }
    if (!e) bad("invalid Huffman code");
    drop((int)(e & 0xffu));
    return (int)(e >> 8);
  }

  void emit(uint8_t b) { dst_[produced_++] = b; }

  void raw_block() {
    drop(have_ & 7);  // to the byte boundary
    const unsigned len = take(16), inv = take(16);
    if ((len ^ 0xffffu) != inv) bad("deflate stored block length mismatch");
    for (unsigned i = 0; i < len && produced_ < dst_len_; ++i) emit((uint8_t)take(8));
  }

  void fixed_tables() {
    uint8_t len[288];
    for (int i = 0; i < 288; ++i) len[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
    lit_.assign(len, 288, 9);
    uint8_t dl[30];
    std::memset(dl, 5, sizeof dl);
    dist_.assign(dl, 30, 6);
  }

  void dynamic_tables() {
    const int nlit = (int)take(5) + 257, ndist = (int)take(5) + 1, nclen = (int)take(4) + 4;
    if (nlit > 286 || ndist > 30) bad("bad deflate code counts");
    // code-length alphabet, its lengths sent in this order (RFC 1951 3.2.7)
    static const uint8_t kClenOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
    uint8_t clen[19] = {0};
    for (int i = 0; i < nclen; ++i) clen[kClenOrder[i]] = (uint8_t)take(3);
    Table meta;
    meta.assign(clen, 19, 7);
    uint8_t len[286 + 30] = {0};
    const int total = nlit + ndist;
    int k = 0;
    while (k < total) {
      const int c = symbol(meta);
      int run = 1;
      uint8_t v = (uint8_t)c;
      if (c == 16) {
        if (k == 0) bad("deflate repeat with no previous length");
        v = len[k - 1];
        run = 3 + (int)take(2);
      } else if (c == 17) {
        v = 0;
        run = 3 + (int)take(3);
      } else if (c == 18) {
        v = 0;
        run = 11 + (int)take(7);
      }
      if (k + run > total) bad("deflate code lengths overflow");
      std::memset(len + k, v, (size_t)run);
      k += run;
    }
    if (len[256] == 0) bad("deflate block without an end-of-block code");
    lit_.assign(len, nlit, 9);
    dist_.assign(len + nlit, ndist, 6);
  }

  void inflate_block() {
    const Bases& B = bases();
    for (;;) {
      const int c = symbol(lit_);
      if (c < 256) {
        if (produced_ == dst_len_) return;
        emit((uint8_t)c);
        continue;
      }
      if (c == 256) return;
      const int li = c - 257;
      if (li >= 29) bad("invalid deflate length symbol");
      const int length = B.len_base[li] + (int)take(B.len_extra[li]);
      const int di = symbol(dist_);
      if (di >= 30) bad("invalid deflate distance symbol");
      const size_t distance = B.dist_base[di] + take(B.dist_extra[di]);
      if (distance > produced_) bad("deflate distance before the start of the data");
      for (int i = 0; i < length && produced_ < dst_len_; ++i) emit(dst_[produced_ - distance]);
      if (produced_ == dst_len_) return;
    }
  }

  const uint8_t* src_;
  size_t src_len_, next_byte_ = 0;
  uint8_t* dst_;
  size_t dst_len_, produced_ = 0;
  uint64_t acc_ = 0;
  int have_ = 0;
  Table lit_, dist_;
};

// Decodes one strip or tile into out (rows x row_len bytes).
void decode_chunk(const Page& pg, const uint8_t* in, size_t n, uint8_t* out, size_t rows, size_t row_len) {
  const size_t cap = rows * row_len;
  switch (pg.compression) {
    case 1:
      if (n < cap) throw TiffError{BM_ERR_INVALID, "uncompressed strip shorter than its rows"};
      std::memcpy(out, in, cap);
      break;
    case 32773: unpackbits(in, n, out, cap); break;
    case 5: unlzw(in, n, out, cap); break;
    case 8:
    case 32946: DeflateStream(in, n, out, cap).decode_all(); break;
    default: throw TiffError{BM_ERR_INVALID, fmt("unsupported compression method %u", pg.compression)};
  }
  if (pg.predictor == 2) {
    for (size_t r = 0; r < rows; ++r) {
      uint8_t* row = out + r * row_len;
      for (size_t i = 1; i < row_len; ++i) row[i] = (uint8_t)(row[i] + row[i - 1]);
    }
  } else if (pg.predictor != 1) {
    throw TiffError{BM_ERR_INVALID, fmt("unsupported predictor %u", pg.predictor)};
  }
}

void decode_page(const File& f, const Page& pg, uint8_t* dst) {
  const size_t w = (size_t)pg.width, h = (size_t)pg.height;
  if (pg.tiled) {
    if (pg.tile_w == 0 || pg.tile_h == 0) throw TiffError{BM_ERR_INVALID, "tile size missing"};
    const size_t tw = (size_t)pg.tile_w, th = (size_t)pg.tile_h;
    const size_t across = (w + tw - 1) / tw, down = (h + th - 1) / th;
    if (pg.offsets.size() < across * down || pg.counts.size() < across * down)
      throw TiffError{BM_ERR_INVALID, "fewer tile offsets than tiles"};
    std::vector<uint8_t> tile(tw * th);
    for (size_t ty = 0; ty < down; ++ty)
      for (size_t tx = 0; tx < across; ++tx) {
        const size_t k = ty * across + tx;
        decode_chunk(pg, f.at(pg.offsets[k], pg.counts[k]), (size_t)pg.counts[k], tile.data(), th, tw);
        const size_t x0 = tx * tw, y0 = ty * th;
        const size_t cw = std::min(tw, w - x0), ch = std::min(th, h - y0);
        for (size_t r = 0; r < ch; ++r) std::memcpy(dst + (y0 + r) * w + x0, tile.data() + r * tw, cw);
      }
  } else {
    const size_t rps = pg.rows_per_strip ? (size_t)std::min<uint64_t>(pg.rows_per_strip, h) : h;
    const size_t strips = (h + rps - 1) / rps;
    if (pg.offsets.size() < strips || pg.counts.size() < strips)
      throw TiffError{BM_ERR_INVALID, "fewer strip offsets than strips"};
    for (size_t k = 0; k < strips; ++k) {
      const size_t rows = std::min(rps, h - k * rps);
      decode_chunk(pg, f.at(pg.offsets[k], pg.counts[k]), (size_t)pg.counts[k], dst + k * rps * w, rows, w);
    }
  }
}

struct Stack {
  size_t width = 0, height = 0;
  std::vector<Page> pages;  // pages that passed the structural checks
  // the first page whose structural check failed (pages.size() of them passed)
  bool failed = false;
  TiffError error{BM_OK, ""};
};

// The reference's per-page checks before decoding (tiff_io.rs:47-90):
// dimensions, colour type, consistency, then the next page.  They stop at
// the first failure, which is reported only if no earlier page fails to
// decode or validate.
Stack read_stack(File& f, const std::string& path) {
  uint64_t off = 0;
  f.header(&off);
  Stack st;
  std::vector<Entry> ents;
  std::vector<uint64_t> seen;
  try {
    while (off) {
      if (std::find(seen.begin(), seen.end(), off) != seen.end())
        throw TiffError{BM_ERR_INVALID, fmt("advancing to the next page of %s: IFD loop", path.c_str())};
      seen.push_back(off);
      uint64_t next = 0;
      Page pg;
      try {
        next = f.ifd(off, ents);
        pg = parse_page(f, ents);
      } catch (const TiffError& e) {
        throw TiffError{e.status, fmt("reading dimensions from %s: %s", path.c_str(), e.msg.c_str())};
      }
      const std::string ct = color_type(pg);
      if (!ct.empty())
        throw TiffError{BM_ERR_INVALID,
                        fmt("%s must contain 8-bit grayscale pages; found %s", path.c_str(), ct.c_str())};
      if (st.pages.empty()) {
        st.width = (size_t)pg.width;
        st.height = (size_t)pg.height;
      } else if (pg.width != st.width || pg.height != st.height) {
        throw TiffError{BM_ERR_INVALID,
                        fmt("TIFF pages in %s do not have consistent dimensions: expected %zux%zu, got %llux%llu",
                            path.c_str(), st.width, st.height, (unsigned long long)pg.width,
                            (unsigned long long)pg.height)};
      }
      st.pages.push_back(pg);
      off = next;
    }
  } catch (const TiffError& e) {
    st.failed = true;
    st.error = e;
  }
  return st;
}

}  // namespace

}  // namespace bm

using namespace bm;

extern "C" {

int bm_tiff_read(const char* path, unsigned threshold, int accepted, uint8_t* out, size_t capacity, size_t* width,
                 size_t* height, size_t* depth) {
  if (!path || accepted < 0 || accepted > 2 || threshold > 255) {
    set_thread_error("invalid argument");
    return BM_ERR_INVALID;
  }
  const std::string spath(path);
  try {
    Mapped m;
    m.fd = open(path, O_RDONLY);
    if (m.fd < 0) throw TiffError{BM_ERR_INVALID, fmt("opening %s: %s", path, std::strerror(errno))};
    struct stat sb;
    if (fstat(m.fd, &sb) != 0) throw TiffError{BM_ERR_INVALID, fmt("opening %s: %s", path, std::strerror(errno))};
    m.n = (size_t)sb.st_size;
    if (m.n) {
      void* p = mmap(nullptr, m.n, PROT_READ, MAP_PRIVATE, m.fd, 0);
      if (p == MAP_FAILED) throw TiffError{BM_ERR_INVALID, fmt("opening %s: %s", path, std::strerror(errno))};
      m.p = static_cast<const uint8_t*>(p);
    }
    File f(m.p, m.n, spath);
    Stack st = read_stack(f, spath);
    if (st.failed && st.pages.empty()) throw st.error;
    const size_t w = st.width, h = st.height, d = st.pages.size();
    const size_t page_len = w * h;
    if (h && page_len / h != w) throw TiffError{BM_ERR_INVALID, "TIFF page dimensions overflow usize"};
    if (!out) {  // dimensions only: of the pages before any structural failure, which the
                 // decoding call reports after checking those pages' samples (reference order)
      if (width) *width = w;
      if (height) *height = h;
      if (depth) *depth = d;
      return BM_OK;
    }
    if (capacity < page_len * d) throw TiffError{BM_ERR_INVALID, "output buffer smaller than the volume"};
    // decode the pages that passed the structural checks, in parallel; each
    // records its first failure, and the earliest failing page is reported
    std::vector<std::string> errs(d);
    std::vector<int> err_status(d, BM_OK);
    std::atomic<size_t> next_page{0};
    std::atomic<size_t> first_bad{d};
    auto worker = [&]() {
      for (;;) {
        const size_t k = next_page.fetch_add(1);
        if (k >= d || k > first_bad.load()) return;
        uint8_t* dst = out + k * page_len;
        try {
          try {
            decode_page(f, st.pages[k], dst);
          } catch (const TiffError& e) {
            throw TiffError{e.status, fmt("decoding page %zu of %s: %s", k + 1, path, e.msg.c_str())};
          }
          if (st.pages[k].sample_format != 1)
            throw TiffError{BM_ERR_INVALID,
                            fmt("%s decoded to an unsupported pixel type; expected unsigned 8-bit samples", path)};
          // validation (tiff_io.rs:106-133) then threshold (:135)
          for (size_t i = 0; i < page_len; ++i) {
            const uint8_t v = dst[i];
            const bool bad =
                accepted == 1 ? (v != 0 && v != 255) : accepted == 2 ? (v != 0 && v != 1 && v != 255) : false;
            if (bad)
              throw TiffError{BM_ERR_INVALID,
                              fmt("%s is not a valid binary image: page %zu, sample %zu has value %u (expected %s)",
                                  path, k + 1, i, (unsigned)v, accepted == 1 ? "0 or 255" : "0/1 or 0/255")};
            dst[i] = v > threshold ? 1u : 0u;
          }
        } catch (const TiffError& e) {
          errs[k] = e.msg;
          err_status[k] = e.status;
          size_t cur = first_bad.load();
          while (k < cur && !first_bad.compare_exchange_weak(cur, k)) {
          }
        }
      }
    };
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 4;
    nt = (unsigned)std::min<size_t>(nt, std::max<size_t>(d, 1));
    std::vector<std::thread> th;
    for (unsigned i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto& t : th) t.join();
    const size_t fb = first_bad.load();
    if (fb < d) throw TiffError{err_status[fb], errs[fb]};
    if (st.failed) throw st.error;
    if (width) *width = w;
    if (height) *height = h;
    if (depth) *depth = d;
    // the reference builds a BinaryVolume: every dimension at least 2 (volume.rs:27-34)
    if (w < 2 || h < 2 || d < 2)
      throw TiffError{BM_ERR_DIMS, fmt("all dimensions must be at least 2 for 3-D morphometry; got %zux%zux%zu", w,
                                       h, d)};
    return BM_OK;
  } catch (const TiffError& e) {
    set_thread_error(e.msg.c_str());
    return e.status;
  } catch (const std::bad_alloc&) {
    set_thread_error("out of host memory while decoding a TIFF");
    return BM_ERR_OOM;
  } catch (const std::exception& e) {
    set_thread_error(fmt("reading %s: %s", path, e.what()).c_str());
    return BM_ERR_INVALID;
  }
}

}  // extern "C"
