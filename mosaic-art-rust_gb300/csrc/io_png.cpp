// io_png.cpp -- the two ends of the path for PNG files: a file held in memory
// to an RGB8 buffer, and an RGB8 buffer to a file.
//
// Reference: main.rs:492 and :548 open the target and each chosen material with
// image::open (image 0.25.6, PNG through png 0.17.16) and every consumer works
// on DynamicImage::to_rgb8 of it (lib.rs:94-119, main.rs:687-738); main.rs:672
// writes the output with DynamicImage::save.  mg_png_decode is image::open +
// to_rgb8 for PNG data; mg_png_encode is save for a .png path.
//
// Decoding writes straight into the caller's buffer, which can be pinned
// memory from mg_host_alloc that mg_generate then reads in place over the
// CPU-GPU link: a decoded target goes to the kernels without a staging copy.
// Many files (a material folder) decode on several host threads at once.
//
// Decoder: RFC 1950 (zlib) / RFC 1951 (deflate) inflate with a 10-bit lookup
// table per Huffman code and canonical decoding for longer codes, then the PNG
// 1.2 unfiltering (None, Sub, Up, Average, Paeth), Adam7 de-interlacing and the
// conversion to RGB8 that to_rgb8 applies to what the png crate returns: grey
// replicated to three channels, alpha dropped, palette indices looked up,
// 1/2/4-bit grey scaled to 8 bits (x255, x85, x17), 16-bit samples rounded to 8
// bits ((v + 128) / 257).  Chunk CRCs and the zlib Adler-32 are checked; the
// image data must inflate to exactly the size IHDR implies.
//
// Encoder: 8-bit RGB, one filter per row (the one with the smallest sum of
// absolute residuals as signed bytes), then deflate blocks of up to 65535
// filtered bytes.  Level 0 writes stored blocks; level 1 writes literal-only
// blocks with their own dynamic Huffman code, or a stored block where that is
// smaller.  Every block ends on a byte boundary (an empty stored block follows
// a Huffman block), so the blocks are encoded on several threads and simply
// concatenated; the Adler-32 of the parts is combined arithmetically.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "mosaic_gpu.h"

namespace mg {
void set_error(const std::string& msg);
}

namespace {

struct Status {
  int code = MG_OK;
  std::string msg;
  bool bad(int c, const char* m) {
    code = c;
    msg = m;
    return false;
  }
};

// ---- checksums ----------------------------------------------------------------------
// CRC-32 (ISO 3309, reflected polynomial 0xEDB88320), eight bytes a step
// ("slicing-by-8", Kounavis and Berry 2005): t[k][b] is the CRC of byte b
// followed by k zero bytes, so the eight table entries of one 8-byte word
// combine by XOR; bytes are read one by one (no alignment or byte-order
// assumption).
struct CrcTable {
  uint32_t t[8][256];
  CrcTable() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      t[0][n] = c;
    }
    for (int k = 1; k < 8; ++k)
      for (uint32_t n = 0; n < 256; ++n) t[k][n] = (t[k - 1][n] >> 8) ^ t[0][t[k - 1][n] & 0xFFu];
  }
};
const CrcTable& crc_table() {
  static const CrcTable tab;
  return tab;
}
uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
  const auto& t = crc_table().t;
  uint32_t c = crc ^ 0xFFFFFFFFu;
  for (; n >= 8; p += 8, n -= 8) {
    const uint32_t lo = c ^ ((uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24);
    const uint32_t hi = (uint32_t)p[4] | (uint32_t)p[5] << 8 | (uint32_t)p[6] << 16 | (uint32_t)p[7] << 24;
    c = t[7][lo & 0xFFu] ^ t[6][(lo >> 8) & 0xFFu] ^ t[5][(lo >> 16) & 0xFFu] ^ t[4][lo >> 24] ^ t[3][hi & 0xFFu] ^
        t[2][(hi >> 8) & 0xFFu] ^ t[1][(hi >> 16) & 0xFFu] ^ t[0][hi >> 24];
  }
  for (; n; ++p, --n) c = t[0][(c ^ *p) & 0xFFu] ^ (c >> 8);
  return c ^ 0xFFFFFFFFu;
}

constexpr uint32_t kAdlerMod = 65521;
uint32_t adler32(uint32_t adler, const uint8_t* p, size_t n) {
  uint32_t a = adler & 0xFFFFu, b = adler >> 16;
  while (n) {
    const size_t m = std::min<size_t>(n, 5552);  // no 32-bit overflow before the reduction
    for (size_t i = 0; i < m; ++i) {
      a += p[i];
      b += a;
    }
    a %= kAdlerMod;
    b %= kAdlerMod;
    p += m;
    n -= m;
  }
  return (b << 16) | a;
}
// Adler-32 of the concatenation from the parts' values: the second part's A
// values all rise by (A1 - 1), which adds len2 * (A1 - 1) to its B.
uint32_t adler32_combine(uint32_t a1, uint32_t a2, size_t len2) {
  const uint64_t A1 = a1 & 0xFFFFu, B1 = a1 >> 16, A2 = a2 & 0xFFFFu, B2 = a2 >> 16;
  const uint64_t A = (A1 + A2 + kAdlerMod - 1) % kAdlerMod;
  const uint64_t B = (B1 + B2 + (uint64_t)(len2 % kAdlerMod) * ((A1 + kAdlerMod - 1) % kAdlerMod)) % kAdlerMod;
  return (uint32_t)((B << 16) | A);
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
void put_be32(uint8_t* p, uint32_t v) {
  p[0] = (uint8_t)(v >> 24);
  p[1] = (uint8_t)(v >> 16);
  p[2] = (uint8_t)(v >> 8);
  p[3] = (uint8_t)v;
}

// ---- deflate tables (RFC 1951 3.2.5) --------------------------------------------------
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
const uint8_t kClenOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

uint32_t reverse_bits(uint32_t v, int n) {
  uint32_t r = 0;
  for (int i = 0; i < n; ++i) r |= ((v >> i) & 1u) << (n - 1 - i);
  return r;
}

// ---- inflate ----------------------------------------------------------------------------
struct Huff {
  static constexpr int kFast = 10;
  uint16_t fast[1 << kFast];  // (length << 9) | symbol; 0 = not in the table
  uint16_t count[16];
  uint16_t sym[320];
  int max_len = 0;
  // Canonical code of n symbols with the given lengths.  Over-subscribed sets
  // are rejected; an incomplete set only as one code of length 1 (RFC 1951
  // 3.2.7) or no code at all (decoding it is then an error).
  bool build(const uint8_t* lens, int n, bool allow_incomplete) {
    std::memset(count, 0, sizeof(count));
    for (int i = 0; i < n; ++i) count[lens[i]]++;
    count[0] = 0;
    int left = 1;
    max_len = 0;
    for (int len = 1; len <= 15; ++len) {
      left <<= 1;
      left -= count[len];
      if (left < 0) return false;
      if (count[len]) max_len = len;
    }
    if (left > 0 && max_len > 0 && !(allow_incomplete && max_len == 1)) return false;
    uint16_t offs[16];
    offs[1] = 0;
    for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
    for (int i = 0; i < n; ++i)
      if (lens[i]) sym[offs[lens[i]]++] = (uint16_t)i;
    std::memset(fast, 0, sizeof(fast));
    uint32_t code = 0;
    int idx = 0;
    for (int len = 1; len <= 15; ++len) {
      for (int j = 0; j < count[len]; ++j, ++idx, ++code) {
        if (len > kFast) continue;
        const uint32_t r = reverse_bits(code, len);
        const uint16_t e = (uint16_t)(len << 9 | sym[idx]);
        for (uint32_t f = r; f < (1u << kFast); f += 1u << len) fast[f] = e;
      }
      code <<= 1;
    }
    return true;
  }
};

// Literal/length lookups of kBits bits: an entry decodes one symbol, or two
// literals whose codes together fit in kBits (two output bytes per lookup on
// literal-heavy data).  Entry: bits 0-8 the (first) symbol, 9-16 the second
// literal, 24-28 the bits consumed, 30-31 the symbol count (0: a code longer
// than kBits, decoded by Huff).
struct PairTable {
  static constexpr int kBits = 11;
  uint32_t e[1u << kBits];
  void build(const Huff& h) {
    std::memset(e, 0, sizeof(e));
    uint32_t code = 0;
    int idx = 0;
    for (int len = 1; len <= 15; ++len) {
      for (int j = 0; j < h.count[len]; ++j, ++idx, ++code) {
        if (len > kBits) continue;
        const uint32_t v = 1u << 30 | (uint32_t)len << 24 | h.sym[idx];
        for (uint32_t f = reverse_bits(code, len); f < (1u << kBits); f += 1u << len) e[f] = v;
      }
      code <<= 1;
    }
    // Descending, so e[i >> l1] (<= i) still holds its single entry; the
    // second code is known when its l2 bits lie within the kBits - l1 known ones.
    for (uint32_t i = (1u << kBits); i-- > 0;) {
      const uint32_t a = e[i];
      const uint32_t s1 = a & 0x1FFu, l1 = (a >> 24) & 31u;
      if ((a >> 30) != 1 || s1 >= 256 || l1 >= (uint32_t)kBits) continue;
      const uint32_t b = e[i >> l1];
      const uint32_t s2 = b & 0x1FFu, l2 = (b >> 24) & 31u;
      if ((b >> 30) != 1 || s2 >= 256 || l1 + l2 > (uint32_t)kBits) continue;
      e[i] = 2u << 30 | (l1 + l2) << 24 | s2 << 9 | s1;
    }
  }
};

// Whether two literal codes (lengths lens[0..255]) can fit in one PairTable lookup.
bool pairs_possible(const uint8_t* lens) {
  int shortest = 16;
  for (int i = 0; i < 256; ++i)
    if (lens[i]) shortest = std::min(shortest, (int)lens[i]);
  return 2 * shortest <= PairTable::kBits;
}

struct FixedCodes {  // literal codes of 8 and 9 bits: no pairs
  Huff lit, dist;
  FixedCodes() {
    uint8_t l[288];
    for (int i = 0; i < 144; ++i) l[i] = 8;
    for (int i = 144; i < 256; ++i) l[i] = 9;
    for (int i = 256; i < 280; ++i) l[i] = 7;
    for (int i = 280; i < 288; ++i) l[i] = 8;
    lit.build(l, 288, false);
    uint8_t d[32];  // codes 30 and 31 are part of the code but never valid
    for (int i = 0; i < 32; ++i) d[i] = 5;
    dist.build(d, 32, false);
  }
};
const FixedCodes& fixed_codes() {
  static const FixedCodes fc;
  return fc;
}

// Inflates the zlib stream [src, src+n) into exactly `want` bytes at out,
// which has kInflateSlack writable bytes past `want`.  With `progress`, the
// count of finished output bytes is published (release) at least every
// kPublish bytes, for a reader of the rows on another thread; inflate only
// reads back what it wrote itself, so that reader must not modify it.
// The bit reader lives in locals of this function (stores to the output
// cannot alias them): a 64-bit buffer refilled to >= 56 bits before each
// symbol, enough for a literal/length code, its extra bits, a distance code
// and its extra bits (15 + 5 + 15 + 13).
constexpr size_t kInflateSlack = 8;
constexpr size_t kPublish = 1u << 16;
// part: src is one independent piece of the deflate data (no zlib header, no
// reference before its own output), inflated without the Adler-32 check into
// out[0, want) while other threads write the neighbouring parts, so nothing
// is written past `want`.  The piece must decode to exactly `want` bytes and
// end exactly at src + n on a byte boundary; only the final piece carries
// BFINAL.  Anything else fails, and the caller falls back to the serial
// inflate of the whole stream.
enum PartKind { kWhole = 0, kInnerPart = 1, kFinalPart = 2 };
bool inflate_zlib(const uint8_t* src, size_t n, uint8_t* out, size_t want, Status& st,
                  std::atomic<size_t>* progress = nullptr, PartKind part = kWhole) {
  if (!part) {
    if (n < 6) return st.bad(MG_ERR_ARG, "PNG image data: zlib stream too short");
    const unsigned cmf = src[0], flg = src[1];
    if ((cmf & 0x0F) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0)
      return st.bad(MG_ERR_ARG, "PNG image data: bad zlib header");
    if (flg & 0x20) return st.bad(MG_ERR_ARG, "PNG image data: preset dictionary");
  }
  const uint8_t* ip = part ? src : src + 2;
  const uint8_t* const iend = src + n;
  uint64_t bitbuf = 0;
  int bitcnt = 0;
  size_t phantom = 0;  // zero bytes fed past the end of the input
  // Whole bytes up to 56..63 buffered bits.  The fast form loads 8 bytes and
  // advances past the whole ones only; the bits above bitcnt then repeat the
  // next byte's low bits, which the next load ORs in again unchanged.
  auto refill = [&]() {
    if (iend - ip >= 8) {
      uint64_t v = 0;
      for (int i = 0; i < 8; ++i) v |= (uint64_t)ip[i] << (8 * i);
      bitbuf |= v << bitcnt;
      ip += (63 - bitcnt) >> 3;
      bitcnt |= 56;
      return;
    }
    while (bitcnt <= 56) {
      uint64_t v = 0;
      if (ip < iend)
        v = *ip++;
      else
        ++phantom;
      bitbuf |= v << bitcnt;
      bitcnt += 8;
    }
  };
  auto take = [&](int k) -> uint32_t {  // k <= 32, after a refill that covers it
    const uint32_t v = (uint32_t)(bitbuf & ((1ull << k) - 1));
    bitbuf >>= k;
    bitcnt -= k;
    return v;
  };
  auto bits = [&](int k) -> uint32_t {
    if (bitcnt < k) refill();
    return take(k);
  };
  // more bits consumed than the input held
  auto overrun = [&]() { return (size_t)(bitcnt / 8) < phantom; };
  // all of [src, src + n) consumed, on a byte boundary
  auto at_end = [&]() { return 8 * ((size_t)(ip - src) + phantom) - (size_t)bitcnt == 8 * n; };
  // next symbol of h (>= 15 buffered bits), -1 on a code outside the set
  auto decode = [&](const Huff& h) -> int {
    const uint16_t e = h.fast[bitbuf & ((1u << Huff::kFast) - 1)];
    if (e) {
      const int len = e >> 9;
      bitbuf >>= len;
      bitcnt -= len;
      return e & 0x1FF;
    }
    int code = 0, first = 0, index = 0;
    for (int len = 1; len <= 15; ++len) {
      code |= (int)((bitbuf >> (len - 1)) & 1u);
      const int c = h.count[len];
      if (code - c < first) {
        bitbuf >>= len;
        bitcnt -= len;
        return h.sym[index + (code - first)];
      }
      index += c;
      first += c;
      first <<= 1;
      code <<= 1;
    }
    return -1;
  };
  size_t pos = 0;
  Huff dyn[2];
  PairTable dyn_pairs;
  bool last = false;
  while (!last && !(part && pos == want && at_end())) {
    last = bits(1) != 0;
    const uint32_t type = bits(2);
    if (type == 0) {
      const int drop = bitcnt & 7;  // to the byte boundary
      bitbuf >>= drop;
      bitcnt -= drop;
      const uint32_t len = bits(16), nlen = bits(16);
      if ((len ^ 0xFFFFu) != nlen) return st.bad(MG_ERR_ARG, "PNG image data: stored block length check");
      if (len > want - pos) return st.bad(MG_ERR_ARG, "PNG image data: more data than the image holds");
      uint32_t k = 0;
      for (; k < len && bitcnt >= 8; ++k) out[pos++] = (uint8_t)take(8);  // bytes already in the bit buffer
      if (overrun()) return st.bad(MG_ERR_ARG, "PNG image data: truncated");
      if (bitcnt == 0) bitbuf = 0;  // drop the look-ahead bits of the byte the copy below moves past
      const size_t rest = len - k;
      if ((size_t)(iend - ip) < rest) return st.bad(MG_ERR_ARG, "PNG image data: truncated");
      std::memcpy(out + pos, ip, rest);
      ip += rest;
      pos += rest;
      if (progress) progress->store(pos, std::memory_order_release);
      continue;
    }
    const Huff* lit;
    const Huff* dist;
    const PairTable* pairs;
    if (type == 1) {
      lit = &fixed_codes().lit;
      dist = &fixed_codes().dist;
      pairs = nullptr;
    } else if (type == 2) {
      const int hlit = (int)bits(5) + 257, hdist = (int)bits(5) + 1, hclen = (int)bits(4) + 4;
      if (hlit > 286 || hdist > 30) return st.bad(MG_ERR_ARG, "PNG image data: bad code counts");
      uint8_t cl[19] = {};
      for (int i = 0; i < hclen; ++i) cl[kClenOrder[i]] = (uint8_t)bits(3);
      Huff clh;
      if (!clh.build(cl, 19, false)) return st.bad(MG_ERR_ARG, "PNG image data: bad code-length code");
      uint8_t lens[320];
      int i = 0;
      while (i < hlit + hdist) {
        if (bitcnt < 15 + 7) refill();
        const int s = decode(clh);
        if (s < 0) return st.bad(MG_ERR_ARG, "PNG image data: bad code length");
        if (s < 16) {
          lens[i++] = (uint8_t)s;
          continue;
        }
        int rep;
        uint8_t v = 0;
        if (s == 16) {
          if (i == 0) return st.bad(MG_ERR_ARG, "PNG image data: repeat with no previous length");
          v = lens[i - 1];
          rep = 3 + (int)take(2);
        } else if (s == 17) {
          rep = 3 + (int)take(3);
        } else {
          rep = 11 + (int)take(7);
        }
        if (i + rep > hlit + hdist) return st.bad(MG_ERR_ARG, "PNG image data: code lengths overflow");
        for (int r = 0; r < rep; ++r) lens[i++] = v;
      }
      if (lens[256] == 0) return st.bad(MG_ERR_ARG, "PNG image data: no end-of-block code");
      if (!dyn[0].build(lens, hlit, true) || !dyn[1].build(lens + hlit, hdist, true))
        return st.bad(MG_ERR_ARG, "PNG image data: bad Huffman code");
      lit = &dyn[0];
      dist = &dyn[1];
      pairs = nullptr;
      if (pairs_possible(lens)) {
        dyn_pairs.build(dyn[0]);
        pairs = &dyn_pairs;
      }
    } else {
      return st.bad(MG_ERR_ARG, "PNG image data: bad block type");
    }
    size_t next_pub = progress ? pos + kPublish : SIZE_MAX;
    for (;;) {
      if (pos >= next_pub) {
        progress->store(pos, std::memory_order_release);
        next_pub = pos + kPublish;
      }
      if (bitcnt < 48) refill();
      const uint32_t pe = pairs ? pairs->e[bitbuf & ((1u << PairTable::kBits) - 1)] : 0u;
      int s;
      if ((pe >> 30) == 2 && want - pos >= 2) {
        out[pos] = (uint8_t)pe;
        out[pos + 1] = (uint8_t)(pe >> 9);
        pos += 2;
        const int len = (int)((pe >> 24) & 31u);
        bitbuf >>= len;
        bitcnt -= len;
        continue;
      }
      if ((pe >> 30) == 1) {
        s = (int)(pe & 0x1FFu);
        const int len = (int)((pe >> 24) & 31u);
        bitbuf >>= len;
        bitcnt -= len;
      } else {
        s = decode(*lit);  // a code longer than the table, or a pair where one byte is left
      }
      if (s < 256) {
        if (s < 0) return st.bad(MG_ERR_ARG, "PNG image data: bad literal/length code");
        if (pos >= want) return st.bad(MG_ERR_ARG, "PNG image data: more data than the image holds");
        out[pos++] = (uint8_t)s;
        continue;
      }
      if (s == 256) break;
      if (s > 285) return st.bad(MG_ERR_ARG, "PNG image data: bad length symbol");
      const size_t len = kLenBase[s - 257] + take(kLenExtra[s - 257]);
      const int ds = decode(*dist);
      if (ds < 0 || ds > 29) return st.bad(MG_ERR_ARG, "PNG image data: bad distance code");
      const size_t d = kDistBase[ds] + take(kDistExtra[ds]);
      if (d > pos) return st.bad(MG_ERR_ARG, "PNG image data: distance before the start");
      if (len > want - pos) return st.bad(MG_ERR_ARG, "PNG image data: more data than the image holds");
      uint8_t* o = out + pos;
      const uint8_t* from = o - d;
      if (d >= 8 && (!part || want - pos >= ((len + 7) & ~(size_t)7))) {
        // 8-byte steps, each reading bytes at least 8 behind what it writes;
        // the last step may write up to 7 bytes past the match (a whole
        // stream's buffer has kInflateSlack spare bytes, overwritten by what
        // follows; a part copies exactly near its end instead, as the bytes
        // after it belong to the next part's thread)
        for (size_t k = 0; k < len; k += 8) std::memcpy(o + k, from + k, 8);
      } else if (d == 1) {
        std::memset(o, *from, len);
      } else {
        for (size_t k = 0; k < len; ++k) o[k] = from[k];  // overlapping: repeats the last d bytes
      }
      pos += len;
    }
    if (overrun()) return st.bad(MG_ERR_ARG, "PNG image data: truncated");
    if (progress) progress->store(pos, std::memory_order_release);
  }
  if (pos != want) return st.bad(MG_ERR_ARG, "PNG image data: less data than the image holds");
  if (part) {
    if (last != (part == kFinalPart)) return st.bad(MG_ERR_ARG, "PNG image data: part ends on the wrong block");
    const int drop = bitcnt & 7;
    bitbuf >>= drop;
    bitcnt -= drop;
    if (overrun() || !at_end()) return st.bad(MG_ERR_ARG, "PNG image data: part does not end where indexed");
    return true;
  }
  {
    const int drop = bitcnt & 7;
    bitbuf >>= drop;
    bitcnt -= drop;
  }
  const uint32_t a = bits(8) << 24 | bits(8) << 16 | bits(8) << 8 | bits(8);
  if (overrun()) return st.bad(MG_ERR_ARG, "PNG image data: truncated");
  if (a != adler32(1, out, want)) return st.bad(MG_ERR_ARG, "PNG image data: Adler-32 mismatch");
  return true;
}

// fn(0..n-1) on up to `threads` threads (<= 0: one per hardware thread).
template <typename F>
void parallel_for(size_t n, int threads, F&& fn) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  const int t = (int)std::max<size_t>(1, std::min<size_t>(n, (size_t)threads));
  if (t <= 1) {
    for (size_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<size_t> next{0};
  auto work = [&]() {
    for (size_t i; (i = next.fetch_add(1)) < n;) fn(i);
  };
  // Threads that cannot be created (a thread or process limit) leave their
  // share to the ones running: work() takes items until none are left, so the
  // calling thread alone still finishes everything.
  std::vector<std::thread> pool;
  pool.reserve((size_t)t - 1);
  for (int k = 1; k < t; ++k) {
    try {
      pool.emplace_back(work);
    } catch (const std::exception&) {
      break;
    }
  }
  work();
  for (auto& th : pool) th.join();
}

// ---- PNG decode -------------------------------------------------------------------------
struct Header {
  uint32_t w = 0, h = 0;
  int depth = 0, color = 0, interlace = 0;
  int channels() const { return color == 0 ? 1 : color == 2 ? 3 : color == 3 ? 1 : color == 4 ? 2 : 4; }
  int bits_pp() const { return channels() * depth; }
  size_t row_bytes(uint32_t width) const { return ((size_t)width * bits_pp() + 7) / 8; }
  int filter_bpp() const { return std::max(1, bits_pp() / 8); }
};

const uint8_t kSignature[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
const int kAdam7[7][4] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                          {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};  // x0, y0, dx, dy

bool parse_header(const uint8_t* d, size_t n, Header& H, Status& st) {
  if (!d || n < 8 + 25) return st.bad(MG_ERR_ARG, "not a PNG file (too short)");
  if (std::memcmp(d, kSignature, 8) != 0) return st.bad(MG_ERR_ARG, "not a PNG file (signature)");
  if (be32(d + 8) != 13 || std::memcmp(d + 12, "IHDR", 4) != 0) return st.bad(MG_ERR_ARG, "PNG: IHDR is not first");
  if (crc32_update(0, d + 12, 17) != be32(d + 29)) return st.bad(MG_ERR_ARG, "PNG: IHDR CRC mismatch");
  const uint8_t* p = d + 16;
  H.w = be32(p);
  H.h = be32(p + 4);
  H.depth = p[8];
  H.color = p[9];
  H.interlace = p[12];
  if (H.w == 0 || H.h == 0 || H.w > 0x7FFFFFFFu || H.h > 0x7FFFFFFFu) return st.bad(MG_ERR_ARG, "PNG: bad dimensions");
  if (p[10] != 0 || p[11] != 0 || H.interlace > 1) return st.bad(MG_ERR_ARG, "PNG: unknown compression, filter or interlace method");
  bool ok;
  switch (H.color) {
    case 0: ok = H.depth == 1 || H.depth == 2 || H.depth == 4 || H.depth == 8 || H.depth == 16; break;
    case 3: ok = H.depth == 1 || H.depth == 2 || H.depth == 4 || H.depth == 8; break;
    case 2: case 4: case 6: ok = H.depth == 8 || H.depth == 16; break;
    default: ok = false;
  }
  if (!ok) return st.bad(MG_ERR_ARG, "PNG: bad colour type / bit depth");
  return true;
}

typedef int16_t V4s __attribute__((vector_size(8)));
typedef uint8_t V4u __attribute__((vector_size(4)));
inline V4s load4(const uint8_t* p) {
  V4u u;
  std::memcpy(&u, p, 4);
  return __builtin_convertvector(u, V4s);
}
inline V4s vabs(V4s v) {
  const V4s m = v >> 15;
  return (v ^ m) - m;
}

// One row: in = its filtered bytes, x = the unfiltered row out (4 writable
// bytes past rb), prev = the
// unfiltered row above (zeros for the first row of a pass).  BPP: bytes per
// complete pixel.
template <int BPP>
void unfilter_row(int f, const uint8_t* in, uint8_t* x, const uint8_t* prev, size_t rb) {
  const size_t head = std::min<size_t>(BPP, rb);
  switch (f) {
    case 0:
      std::memcpy(x, in, rb);
      break;
    case 1:
      for (size_t i = 0; i < head; ++i) x[i] = in[i];
      for (size_t i = BPP; i < rb; ++i) x[i] = (uint8_t)(in[i] + x[i - BPP]);
      break;
    case 2:
      for (size_t i = 0; i < rb; ++i) x[i] = (uint8_t)(in[i] + prev[i]);
      break;
    case 3:
      for (size_t i = 0; i < head; ++i) x[i] = (uint8_t)(in[i] + (prev[i] >> 1));
      for (size_t i = BPP; i < rb; ++i) x[i] = (uint8_t)(in[i] + ((x[i - BPP] + prev[i]) >> 1));
      break;
    default: {
      size_t i = 0;
      if constexpr (BPP == 3 || BPP == 4) {
        // a pixel's channels side by side in one small vector (portable GCC
        // vector extensions); the left pixel `a` stays in a register.  With
        // three-byte pixels the fourth lane reads the next pixel's first byte,
        // computes nothing used and is overwritten by the next store, so the
        // loop stops where that byte would lie outside the row.
        V4s a = {0, 0, 0, 0}, c = {0, 0, 0, 0};
        for (; i + 4 <= rb; i += BPP) {
          const V4s b = load4(prev + i), d = load4(in + i);
          const V4s pa = vabs(b - c), pb = vabs(a - c), pc = vabs(a + b - c - c);
          const V4s ma = (pa <= pb) & (pa <= pc);
          const V4s mb = ~ma & (pb <= pc);
          const V4s r = (d + ((a & ma) | (b & mb) | (c & ~(ma | mb)))) & 0xFF;
          const V4u o = __builtin_convertvector(r, V4u);
          std::memcpy(x + i, &o, 4);
          a = r;
          c = b;
        }
      }
      for (; i < rb; ++i) {
        const int a = i >= BPP ? x[i - BPP] : 0, b = prev[i], c = i >= BPP ? prev[i - BPP] : 0;
        const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
        const int ma = -(int)((pa <= pb) & (pa <= pc));
        const int mb = ~ma & -(int)(pb <= pc);
        x[i] = (uint8_t)(in[i] + ((a & ma) | (b & mb) | (c & ~(ma | mb))));
      }
      break;
    }
  }
}

void unfilter_any(int bpp, int f, const uint8_t* in, uint8_t* x, const uint8_t* prev, size_t rb) {
  switch (bpp) {
    case 1: unfilter_row<1>(f, in, x, prev, rb); break;
    case 2: unfilter_row<2>(f, in, x, prev, rb); break;
    case 3: unfilter_row<3>(f, in, x, prev, rb); break;
    case 4: unfilter_row<4>(f, in, x, prev, rb); break;
    case 6: unfilter_row<6>(f, in, x, prev, rb); break;
    default: unfilter_row<8>(f, in, x, prev, rb); break;
  }
}

// Sample `i` of an unfiltered row, as 8 bits the way to_rgb8 sees it.
inline uint8_t sample8(const uint8_t* x, size_t i, int depth, bool scale_low) {
  switch (depth) {
    case 8: return x[i];
    case 16: {
      const uint32_t v = (uint32_t)x[2 * i] << 8 | x[2 * i + 1];
      return (uint8_t)((v + 128) / 257);
    }
    default: {
      const size_t bit = i * depth;
      const uint32_t v = (x[bit >> 3] >> (8 - depth - (bit & 7))) & ((1u << depth) - 1);
      return scale_low ? (uint8_t)(v * (255u / ((1u << depth) - 1))) : (uint8_t)v;
    }
  }
}

// One unfiltered row of `width` pixels to RGB8 at out (pixel step `step` pixels).
void row_to_rgb(const Header& H, const uint8_t* x, uint32_t width, const uint8_t* plte, int plte_n, uint8_t* out,
                size_t step) {
  if (H.depth == 8 && step == 1) {  // the common files, without the per-sample switch
    if (H.color == 2) {
      std::memcpy(out, x, 3 * (size_t)width);
      return;
    }
    if (H.color == 6) {
      for (uint32_t px = 0; px < width; ++px) {
        out[3 * px] = x[4 * px];
        out[3 * px + 1] = x[4 * px + 1];
        out[3 * px + 2] = x[4 * px + 2];
      }
      return;
    }
  }
  const int ch = H.channels();
  for (uint32_t px = 0; px < width; ++px, out += 3 * step) {
    const size_t s = (size_t)px * ch;
    if (H.color == 3) {
      const uint8_t idx = sample8(x, s, H.depth, false);
      if (idx < plte_n) {
        out[0] = plte[3 * idx];
        out[1] = plte[3 * idx + 1];
        out[2] = plte[3 * idx + 2];
      } else {
        out[0] = out[1] = out[2] = 0;
      }
    } else if (H.color == 0 || H.color == 4) {
      const uint8_t g = sample8(x, s, H.depth, true);
      out[0] = out[1] = out[2] = g;
    } else {
      out[0] = sample8(x, s, H.depth, false);
      out[1] = sample8(x, s + 1, H.depth, false);
      out[2] = sample8(x, s + 2, H.depth, false);
    }
  }
}

constexpr size_t kPipelineMin = 1u << 20;  // inflated bytes below which one thread does everything

// Files this library writes carry a private chunk "mgIX" (ancillary, unsafe to
// copy, so an editor that rewrites the image data drops it): the count of
// independent deflate parts, then per part its offset in the zlib stream and
// in the inflated data (big-endian u32, then u64 pairs).  Parts share no
// back-references, so they inflate on all threads; any inconsistency, or a
// part that fails, leaves the serial inflate to decide.
bool inflate_indexed(const std::vector<uint8_t>& z, const uint8_t* idx, size_t idx_len, uint8_t* raw, size_t total) {
  if (idx_len < 4 || z.size() < 6) return false;
  const size_t count = be32(idx);
  if (count == 0 || count > (idx_len - 4) / 16 || idx_len != 4 + 16 * count) return false;
  std::vector<size_t> zo(count + 1), ro(count + 1);
  for (size_t i = 0; i < count; ++i) {
    const uint8_t* q = idx + 4 + 16 * i;
    zo[i] = (size_t)((uint64_t)be32(q) << 32 | be32(q + 4));
    ro[i] = (size_t)((uint64_t)be32(q + 8) << 32 | be32(q + 12));
  }
  zo[count] = z.size() - 4;  // the Adler-32 follows the last part
  ro[count] = total;
  if (zo[0] != 2 || ro[0] != 0) return false;
  for (size_t i = 0; i < count; ++i)
    if (zo[i + 1] <= zo[i] || ro[i + 1] <= ro[i] || zo[i + 1] > z.size() - 4 || ro[i + 1] > total) return false;
  std::vector<uint32_t> adl(count);
  std::atomic<bool> ok{true};
  parallel_for(count, 0, [&](size_t i) {
    Status st;
    if (!ok.load(std::memory_order_relaxed)) return;
    if (!inflate_zlib(z.data() + zo[i], zo[i + 1] - zo[i], raw + ro[i], ro[i + 1] - ro[i], st, nullptr,
                      i + 1 == count ? kFinalPart : kInnerPart)) {
      ok.store(false);
      return;
    }
    adl[i] = adler32(1, raw + ro[i], ro[i + 1] - ro[i]);
  });
  if (!ok.load()) return false;
  uint32_t a = adl[0];
  for (size_t i = 1; i < count; ++i) a = adler32_combine(a, adl[i], ro[i + 1] - ro[i]);
  return a == be32(z.data() + z.size() - 4);
}

int decode_png(const uint8_t* d, size_t n, uint8_t* out, int64_t stride, Status& st, bool pipelined) {
  Header H;
  if (!parse_header(d, n, H, st)) return st.code;
  if (!out) return st.bad(MG_ERR_ARG, "null output buffer"), st.code;
  if (stride < 3ll * (int64_t)H.w) return st.bad(MG_ERR_ARG, "output stride below 3 * width"), st.code;
  std::vector<uint8_t> z;
  uint8_t plte[768];
  int plte_n = 0;
  bool seen_idat = false;
  const uint8_t* index = nullptr;
  size_t index_len = 0;
  size_t pos = 8;
  try {
    while (pos + 12 <= n) {
      const uint32_t len = be32(d + pos);
      const uint8_t* type = d + pos + 4;
      if (len > 0x7FFFFFFFu || len > n - pos - 12) return st.bad(MG_ERR_ARG, "PNG: chunk runs past the end of the file"), st.code;
      const uint8_t* data = d + pos + 8;
      if (crc32_update(0, type, 4 + (size_t)len) != be32(data + len)) return st.bad(MG_ERR_ARG, "PNG: chunk CRC mismatch"), st.code;
      if (!std::memcmp(type, "IDAT", 4)) {
        z.insert(z.end(), data, data + len);
        seen_idat = true;
      } else if (!std::memcmp(type, "PLTE", 4)) {
        if (len % 3 != 0 || len > 768 || len == 0) return st.bad(MG_ERR_ARG, "PNG: bad PLTE length"), st.code;
        std::memcpy(plte, data, len);
        plte_n = (int)(len / 3);
      } else if (!std::memcmp(type, "mgIX", 4)) {
        index = data;
        index_len = len;
      } else if (!std::memcmp(type, "IEND", 4)) {
        break;
      } else if (!(type[0] & 0x20) && std::memcmp(type, "IHDR", 4) != 0) {
        return st.bad(MG_ERR_ARG, "PNG: unknown critical chunk"), st.code;
      }
      pos += 12 + (size_t)len;
    }
    if (!seen_idat) return st.bad(MG_ERR_ARG, "PNG: no image data"), st.code;
    if (H.color == 3 && plte_n == 0) return st.bad(MG_ERR_ARG, "PNG: palette image without PLTE"), st.code;
    // inflated size and pass geometry
    struct Pass {
      uint32_t w, h;
      size_t off, rb;
    } pass[7];
    int npass = H.interlace ? 7 : 1;
    size_t total = 0;
    for (int i = 0; i < npass; ++i) {
      uint32_t pw = H.w, ph = H.h;
      if (H.interlace) {
        const int* a = kAdam7[i];
        pw = H.w > (uint32_t)a[0] ? (H.w - a[0] + a[2] - 1) / a[2] : 0;
        ph = H.h > (uint32_t)a[1] ? (H.h - a[1] + a[3] - 1) / a[3] : 0;
      }
      pass[i] = Pass{pw, ph, total, H.row_bytes(pw)};
      if (pw && ph) {
        const size_t bytes = (size_t)ph * (pass[i].rb + 1);
        if (bytes / ph != pass[i].rb + 1 || total + bytes < total) return st.bad(MG_ERR_ARG, "PNG: image too large"), st.code;
        total += bytes;
      }
    }
    // not value-initialised: a header that claims a huge image costs no page
    // until inflate writes it, and inflate stops at the data the file has
    std::unique_ptr<uint8_t[]> raw(new uint8_t[total + kInflateSlack]);
    // Rows are unfiltered out of place (inflate reads back its own output)
    // into two row buffers and converted while they are hot.  A large image
    // inflates on a second thread while this one follows it row by row.
    std::atomic<size_t> progress{0};
    std::atomic<bool> inflate_failed{false};
    Status ist;
    std::thread worker;
    auto run_inflate = [&]() {
      if (!inflate_zlib(z.data(), z.size(), raw.get(), total, ist, &progress)) inflate_failed.store(true);
    };
    if (pipelined && total >= kPipelineMin && index && inflate_indexed(z, index, index_len, raw.get(), total)) {
      progress.store(total);
    } else if (pipelined && total >= kPipelineMin) {
      try {
        worker = std::thread(run_inflate);
      } catch (const std::exception&) {
        run_inflate();
      }
    } else {
      run_inflate();
    }
    struct Join {
      std::thread& t;
      ~Join() {
        if (t.joinable()) t.join();
      }
    } join{worker};
    size_t max_rb = 0;
    for (int i = 0; i < npass; ++i) max_rb = std::max(max_rb, pass[i].rb);
    std::vector<uint8_t> rowbuf(3 * (max_rb + 8), 0);  // zeros, prev, cur
    const uint8_t* zero = rowbuf.data();
    uint8_t* ra = rowbuf.data() + (max_rb + 8);
    uint8_t* rb2 = rowbuf.data() + 2 * (max_rb + 8);
    const int bpp = H.filter_bpp();
    bool ok = true;
    for (int i = 0; i < npass && ok; ++i) {
      const Pass& P = pass[i];
      if (!P.w || !P.h) continue;
      const int* a = kAdam7[H.interlace ? i : 0];
      const int x0 = H.interlace ? a[0] : 0, y0 = H.interlace ? a[1] : 0, dx = H.interlace ? a[2] : 1,
                dy = H.interlace ? a[3] : 1;
      const uint8_t* prev = zero;
      uint8_t* cur = ra;
      for (uint32_t r = 0; r < P.h; ++r) {
        const size_t row_end = P.off + (size_t)(r + 1) * (P.rb + 1);
        while (progress.load(std::memory_order_acquire) < row_end) {
          if (inflate_failed.load()) break;
          std::this_thread::yield();
        }
        if (progress.load(std::memory_order_acquire) < row_end) {
          ok = false;
          break;
        }
        const uint8_t* in = raw.get() + row_end - P.rb - 1;
        if (in[0] > 4) {
          st.bad(MG_ERR_ARG, "PNG: bad filter type");
          ok = false;
          break;
        }
        unfilter_any(bpp, in[0], in + 1, cur, prev, P.rb);
        uint8_t* o = out + (size_t)(y0 + (size_t)r * dy) * (size_t)stride + (size_t)x0 * 3;
        row_to_rgb(H, cur, P.w, plte, plte_n, o, (size_t)dx);
        prev = cur;
        cur = cur == ra ? rb2 : ra;
      }
    }
    if (worker.joinable()) worker.join();
    if (inflate_failed.load()) {
      st = ist;  // the inflate defect comes first (a filter byte read from it may be garbage)
      return st.code;
    }
    if (!ok) return st.code;
  } catch (const std::bad_alloc&) {
    return st.bad(MG_ERR_OOM, "out of host memory"), st.code;
  } catch (const std::exception& e) {
    return st.bad(MG_ERR_ARG, e.what()), st.code;
  }
  return MG_OK;
}

// ---- PNG encode -------------------------------------------------------------------------
struct BitOut {
  std::vector<uint8_t> bytes;
  uint64_t buf = 0;
  int cnt = 0;
  void put(uint32_t v, int n) {  // n <= 32, LSB first
    buf |= (uint64_t)v << cnt;
    cnt += n;
    while (cnt >= 8) {
      bytes.push_back((uint8_t)buf);
      buf >>= 8;
      cnt -= 8;
    }
  }
  void align() {
    if (cnt) put(0, 8 - cnt);
  }
};

// Huffman code lengths (<= max_len) for `n` symbols with frequencies `freq`;
// at least two symbols get a code.  Lengths beyond max_len are cured by
// flattening the frequencies and rebuilding.
void huff_lengths(const uint32_t* freq_in, int n, int max_len, uint8_t* lens) {
  std::vector<uint32_t> freq(freq_in, freq_in + n);
  int used = 0;
  for (int i = 0; i < n; ++i) used += freq[i] != 0;
  for (int i = 0; used < 2 && i < n; ++i)
    if (!freq[i]) freq[i] = 1, ++used;
  for (;;) {
    struct Node {
      uint64_t f;
      int a, b;  // children (-1: leaf)
      int sym;
    };
    std::vector<Node> nodes;
    std::vector<int> order;
    for (int i = 0; i < n; ++i)
      if (freq[i]) {
        nodes.push_back(Node{freq[i], -1, -1, i});
        order.push_back((int)nodes.size() - 1);
      }
    std::sort(order.begin(), order.end(), [&](int x, int y) {
      return nodes[x].f != nodes[y].f ? nodes[x].f < nodes[y].f : nodes[x].sym < nodes[y].sym;
    });
    // two-queue construction: sorted leaves, internal nodes in creation order
    std::vector<int> inner;
    size_t li = 0, ii = 0;
    auto take = [&]() {
      if (li < order.size() && (ii >= inner.size() || nodes[order[li]].f <= nodes[inner[ii]].f)) return order[li++];
      return inner[ii++];
    };
    while ((order.size() - li) + (inner.size() - ii) > 1) {
      const int x = take(), y = take();
      nodes.push_back(Node{nodes[x].f + nodes[y].f, x, y, -1});
      inner.push_back((int)nodes.size() - 1);
    }
    std::memset(lens, 0, n);
    std::vector<std::pair<int, int>> stack{{(int)nodes.size() - 1, 0}};
    int deepest = 0;
    while (!stack.empty()) {
      const auto [id, depth] = stack.back();
      stack.pop_back();
      if (nodes[id].a < 0) {
        lens[nodes[id].sym] = (uint8_t)depth;
        deepest = std::max(deepest, depth);
      } else {
        stack.push_back({nodes[id].a, depth + 1});
        stack.push_back({nodes[id].b, depth + 1});
      }
    }
    if (deepest <= max_len) return;
    for (auto& f : freq)
      if (f) f = (f >> 1) | 1u;
  }
}

// Canonical codes (bit-reversed for LSB-first output) from lengths.
void canonical_codes(const uint8_t* lens, int n, uint32_t* codes) {
  uint32_t count[16] = {}, next[16] = {};
  for (int i = 0; i < n; ++i) count[lens[i]]++;
  count[0] = 0;
  uint32_t code = 0;
  for (int len = 1; len <= 15; ++len) {
    code = (code + count[len - 1]) << 1;
    next[len] = code;
  }
  for (int i = 0; i < n; ++i)
    if (lens[i]) codes[i] = reverse_bits(next[lens[i]]++, lens[i]);
}

void stored_block(BitOut& bo, const uint8_t* p, size_t n, bool last) {
  bo.put(last ? 1u : 0u, 1);
  bo.put(0, 2);
  bo.align();
  bo.put((uint32_t)n, 16);
  bo.put((uint32_t)(n ^ 0xFFFFu), 16);
  bo.bytes.insert(bo.bytes.end(), p, p + n);
}

// One part of the deflate stream: `n` (<= 65535) filtered bytes, ending on a
// byte boundary.  The last part carries BFINAL.
void encode_part(const uint8_t* p, size_t n, int level, bool last, std::vector<uint8_t>& out) {
  BitOut bo;
  bo.bytes.reserve(n + 64);
  if (level > 0 && n > 0) {
    uint32_t freq[257] = {};
    for (size_t i = 0; i < n; ++i) freq[p[i]]++;
    freq[256] = 1;
    uint8_t ll[259];
    huff_lengths(freq, 257, 15, ll);
    ll[257] = ll[258] = 1;  // two distance codes of one bit (a complete, unused distance code)
    uint32_t cfreq[19] = {};
    for (int i = 0; i < 259; ++i) cfreq[ll[i]]++;
    uint8_t cl[19];
    huff_lengths(cfreq, 19, 7, cl);
    int hclen = 19;
    while (hclen > 4 && cl[kClenOrder[hclen - 1]] == 0) --hclen;
    uint64_t bits = 3 + 5 + 5 + 4 + 3ull * hclen;
    for (int i = 0; i < 259; ++i) bits += cl[ll[i]];
    for (int i = 0; i < 257; ++i) bits += (uint64_t)freq[i] * ll[i];
    const uint64_t stored_bits = 3 + 7 + 32 + 8ull * n;  // header, worst-case alignment, LEN/NLEN, data
    if (bits + 3 + 7 + 32 < stored_bits) {  // the Huffman block plus the aligning empty stored block
      uint32_t lcode[257], ccode[19];
      canonical_codes(ll, 257, lcode);
      canonical_codes(cl, 19, ccode);
      bo.put(0, 1);  // BFINAL comes with the aligning block
      bo.put(2, 2);
      bo.put(0, 5);  // HLIT = 257
      bo.put(1, 5);  // HDIST = 2
      bo.put((uint32_t)(hclen - 4), 4);
      for (int i = 0; i < hclen; ++i) bo.put(cl[kClenOrder[i]], 3);
      for (int i = 0; i < 259; ++i) bo.put(ccode[ll[i]], cl[ll[i]]);
      for (size_t i = 0; i < n; ++i) bo.put(lcode[p[i]], ll[p[i]]);
      bo.put(lcode[256], ll[256]);
      stored_block(bo, nullptr, 0, last);
      out.swap(bo.bytes);
      return;
    }
  }
  stored_block(bo, p, n, last);
  out.swap(bo.bytes);
}

inline int paeth_pred(int a, int b, int c) {
  const int pa = std::abs(b - c), pb = std::abs(a - c), pc = std::abs(a + b - 2 * c);
  const int ma = -(int)((pa <= pb) & (pa <= pc));
  const int mb = ~ma & -(int)(pb <= pc);
  return (a & ma) | (b & mb) | (c & ~(ma | mb));
}

// Filter type and residuals of one RGB8 row (libpng's minimum-sum-of-absolute-
// residuals choice): one pass scores all five filters, a second writes the
// chosen one's residuals.
void filter_row(const uint8_t* cur, const uint8_t* prev, size_t rb, uint8_t* dst) {
  constexpr int bpp = 3;
  uint64_t sum[5] = {0, 0, 0, 0, 0};
  auto mag = [](int v) { return (uint64_t)std::abs((int)(int8_t)(uint8_t)v); };
  for (size_t i = 0; i < rb; ++i) {
    const int x = cur[i], a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0,
              c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
    sum[0] += mag(x);
    sum[1] += mag(x - a);
    sum[2] += mag(x - b);
    sum[3] += mag(x - ((a + b) >> 1));
    sum[4] += mag(x - paeth_pred(a, b, c));
  }
  int f = 0;
  for (int k = 1; k < 5; ++k)
    if (sum[k] < sum[f]) f = k;
  dst[0] = (uint8_t)f;
  uint8_t* r = dst + 1;
  const size_t head = std::min<size_t>(bpp, rb);
  switch (f) {
    case 0:
      std::memcpy(r, cur, rb);
      break;
    case 1:
      for (size_t i = 0; i < head; ++i) r[i] = cur[i];
      for (size_t i = bpp; i < rb; ++i) r[i] = (uint8_t)(cur[i] - cur[i - bpp]);
      break;
    case 2:
      for (size_t i = 0; i < rb; ++i) r[i] = (uint8_t)(cur[i] - (prev ? prev[i] : 0));
      break;
    case 3:
      for (size_t i = 0; i < rb; ++i) {
        const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0;
        r[i] = (uint8_t)(cur[i] - ((a + b) >> 1));
      }
      break;
    default:
      for (size_t i = 0; i < rb; ++i) {
        const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0,
                  c = (prev && i >= (size_t)bpp) ? prev[i - bpp] : 0;
        r[i] = (uint8_t)(cur[i] - paeth_pred(a, b, c));
      }
      break;
  }
}

constexpr size_t kPart = 65535;
constexpr size_t kIdatMax = 1u << 20;

size_t encode_bound(int w, int h) {
  if (w <= 0 || h <= 0) return 0;
  const size_t raw = (size_t)h * (1 + 3 * (size_t)w);
  const size_t parts = (raw + kPart - 1) / kPart;
  const size_t z = 2 + raw + 5 * parts + 16 + 4;  // zlib header, stored worst case, Adler-32
  return 8 + 25 + (12 + 4 + 16 * parts) + z + 12 * (z / kIdatMax + 1) + 12;  // ... + the mgIX index
}

int encode_png(const uint8_t* rgb, int w, int h, int64_t stride, int level, int threads, uint8_t* out, size_t cap,
               size_t* len, Status& st) {
  if (!rgb || w <= 0 || h <= 0 || stride < 3ll * w) return st.bad(MG_ERR_ARG, "invalid image"), st.code;
  if (level < 0 || level > 1) return st.bad(MG_ERR_ARG, "level must be 0 or 1"), st.code;
  if (!len) return st.bad(MG_ERR_ARG, "null length"), st.code;
  const size_t bound = encode_bound(w, h);
  if (!out || cap < bound) {
    *len = bound;
    return st.bad(MG_ERR_ARG, "output buffer smaller than mg_png_encode_bound"), st.code;
  }
  try {
    const size_t rb = 3 * (size_t)w, raw = (size_t)h * (rb + 1);
    std::vector<uint8_t> filt(raw);
    parallel_for((size_t)h, threads, [&](size_t r) {
      const uint8_t* cur = rgb + r * (size_t)stride;
      const uint8_t* prev = r ? rgb + (r - 1) * (size_t)stride : nullptr;
      filter_row(cur, prev, rb, filt.data() + r * (rb + 1));
    });
    const size_t parts = (raw + kPart - 1) / kPart;
    std::vector<std::vector<uint8_t>> enc(parts);
    std::vector<uint32_t> adl(parts);
    parallel_for(parts, threads, [&](size_t i) {
      const size_t off = i * kPart, n = std::min(kPart, raw - off);
      encode_part(filt.data() + off, n, level, i + 1 == parts, enc[i]);
      adl[i] = adler32(1, filt.data() + off, n);
    });
    uint32_t adler = adl[0];
    for (size_t i = 1; i < parts; ++i) adler = adler32_combine(adler, adl[i], std::min(kPart, raw - i * kPart));
    // IDAT chunks of kIdatMax bytes of the zlib stream (2-byte header, the
    // parts, the Adler-32), each gathered and check-summed on its own thread
    std::vector<size_t> part_at(parts + 1, 2);  // stream offset of each part
    for (size_t i = 0; i < parts; ++i) part_at[i + 1] = part_at[i] + enc[i].size();
    const size_t zlen = part_at[parts] + 4;
    uint8_t zhead[2] = {0x78, 0x01}, ztail[4];
    put_be32(ztail, adler);
    uint8_t* o = out;
    std::memcpy(o, kSignature, 8);
    o += 8;
    put_be32(o, 13);
    std::memcpy(o + 4, "IHDR", 4);
    put_be32(o + 8, (uint32_t)w);
    put_be32(o + 12, (uint32_t)h);
    o[16] = 8;  // bit depth
    o[17] = 2;  // RGB
    o[18] = 0;  // deflate
    o[19] = 0;  // adaptive filtering
    o[20] = 0;  // no interlace
    put_be32(o + 21, crc32_update(0, o + 4, 17));
    o += 25;
    {  // mgIX: where each independent part starts in the zlib stream and in the rows
      const uint32_t ilen = (uint32_t)(4 + 16 * parts);
      put_be32(o, ilen);
      std::memcpy(o + 4, "mgIX", 4);
      uint8_t* q = o + 8;
      put_be32(q, (uint32_t)parts);
      for (size_t i = 0; i < parts; ++i) {
        uint8_t* e = q + 4 + 16 * i;
        const uint64_t zoff = part_at[i], roff = (uint64_t)i * kPart;
        put_be32(e, (uint32_t)(zoff >> 32));
        put_be32(e + 4, (uint32_t)zoff);
        put_be32(e + 8, (uint32_t)(roff >> 32));
        put_be32(e + 12, (uint32_t)roff);
      }
      put_be32(o + 8 + ilen, crc32_update(0, o + 4, 4 + ilen));
      o += 12 + ilen;
    }
    const size_t chunks = (zlen + kIdatMax - 1) / kIdatMax;
    parallel_for(chunks, threads, [&](size_t c) {
      const size_t z0 = c * kIdatMax, clen = std::min(kIdatMax, zlen - z0);
      uint8_t* co = o + c * (kIdatMax + 12);
      put_be32(co, (uint32_t)clen);
      std::memcpy(co + 4, "IDAT", 4);
      uint8_t* dst = co + 8;
      // stream bytes [z0, z0 + clen): the header, the parts from the one holding z0, the tail
      size_t zp = z0, left = clen;
      size_t i = (size_t)(std::upper_bound(part_at.begin(), part_at.end(), zp) - part_at.begin());
      while (left) {
        const uint8_t* src;
        size_t avail;
        if (zp < 2) {
          src = zhead + zp;
          avail = 2 - zp;
        } else if (zp < part_at[parts]) {
          while (part_at[i] <= zp) ++i;  // part i - 1 holds zp
          src = enc[i - 1].data() + (zp - part_at[i - 1]);
          avail = part_at[i] - zp;
        } else {
          src = ztail + (zp - part_at[parts]);
          avail = zlen - zp;
        }
        const size_t take = std::min(avail, left);
        std::memcpy(dst, src, take);
        dst += take;
        zp += take;
        left -= take;
      }
      put_be32(co + 8 + clen, crc32_update(0, co + 4, 4 + clen));
    });
    o += (chunks - 1) * (kIdatMax + 12) + (zlen - (chunks - 1) * kIdatMax) + 12;
    put_be32(o, 0);
    std::memcpy(o + 4, "IEND", 4);
    put_be32(o + 8, crc32_update(0, o + 4, 4));
    o += 12;
    *len = (size_t)(o - out);
  } catch (const std::bad_alloc&) {
    return st.bad(MG_ERR_OOM, "out of host memory"), st.code;
  } catch (const std::exception& e) {
    return st.bad(MG_ERR_ARG, e.what()), st.code;
  }
  return MG_OK;
}

int report(const Status& st) {
  if (st.code != MG_OK) mg::set_error(st.msg);
  return st.code;
}

}  // namespace

extern "C" {

int mg_png_info(const uint8_t* data, size_t n, int* w, int* h) {
  Status st;
  Header H;
  if (!parse_header(data, n, H, st)) return report(st);
  if (w) *w = (int)H.w;
  if (h) *h = (int)H.h;
  return MG_OK;
}

int mg_png_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride) {
  Status st;
  decode_png(data, n, out, stride, st, true);
  return report(st);
}

int mg_png_decode_batch(const uint8_t* const* data, const size_t* n, int count, uint8_t* const* out,
                        const int64_t* stride, int threads, int* status) {
  Status st;
  if (count < 0 || (count > 0 && (!data || !n || !out || !stride))) return st.bad(MG_ERR_ARG, "invalid batch"), report(st);
  std::vector<Status> each((size_t)count);
  try {
    parallel_for((size_t)count, threads,
                 [&](size_t i) { decode_png(data[i], n[i], out[i], stride[i], each[i], count == 1); });
  } catch (const std::exception&) {
    return st.bad(MG_ERR_OOM, "could not start decoding threads"), report(st);
  }
  int first = MG_OK;
  for (int i = 0; i < count; ++i) {
    if (status) status[i] = each[i].code;
    if (each[i].code != MG_OK && first == MG_OK) {
      first = each[i].code;
      st.code = first;
      st.msg = "file " + std::to_string(i) + ": " + each[i].msg;
    }
  }
  return report(st);
}

size_t mg_png_encode_bound(int w, int h) { return encode_bound(w, h); }

int mg_png_encode(const uint8_t* rgb, int w, int h, int64_t stride, int level, int threads, uint8_t* out, size_t cap,
                  size_t* len) {
  Status st;
  encode_png(rgb, w, h, stride, level, threads, out, cap, len, st);
  return report(st);
}

}  // extern "C"
