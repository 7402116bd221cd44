// io_jpeg.cpp -- JPEG files at the input end of the path (host code), and
// decoding by file signature.
//
// Reference: main.rs:172-185 load_tiles accepts png, jpg, jpeg and webp
// materials and main.rs:492 / 548 open them with image::open (+ to_rgb8);
// for JPEG that is zune-jpeg 0.4.18 behind image 0.25.6.  This decoder is the
// library's own, from ITU-T T.81 (the JPEG standard) and JFIF 1.02:
//   * DCT with Huffman coding, 8-bit samples: sequential (SOF0 baseline, SOF1
//     extended) and progressive (SOF2: spectral selection and successive
//     approximation, T.81 G.1.2 -- DC first and refinement scans, AC first
//     scans with end-of-band runs, AC refinement scans with correction bits);
//     lossless, hierarchical and arithmetic-coded files are refused with
//     MG_ERR_ARG;
//   * one component (grey, replicated to RGB) or three (YCbCr per JFIF, or
//     R, G, B when an Adobe segment says "no transform" or, without JFIF or
//     Adobe segments, the components are named 'R', 'G', 'B');
//     sampling factors 1 or 2 in each direction; interleaved and
//     one-component scans; 8- and 16-bit quantisation tables; restart
//     intervals;
//   * the inverse DCT is the separable 8-point form of T.81 A.3.3 in FP32
//     with a cosine table computed in FP64; chroma is upsampled by
//     replication; YCbCr -> RGB with the JFIF equations; each sample rounded
//     to nearest and clamped.
// zune-jpeg's own integer IDCT, its upsampling filter and its colour
// conversion are not pinned (the crate is not here to run): decoded pixels
// may differ from the reference's by a few levels; the tests hold this
// decoder to +-1 of a float64 restatement of the same steps and to the exact
// pixels of files whose content survives the codec unchanged.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mosaic_gpu.h"

namespace mg {
void set_error(const std::string& msg);
}

namespace {

struct Err {
  int code = MG_OK;
  std::string msg;
  bool bad(const std::string& m) {
    code = MG_ERR_ARG;
    msg = "JPEG: " + m;
    return false;
  }
};

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// A Huffman table (T.81 C / F.2.2.3): canonical codes from the code-length
// counts; decoding with a 9-bit lookup and the canonical limits beyond it.
struct Huff {
  static constexpr int kFast = 9;
  uint16_t fast[1 << kFast];  // (length << 8 | symbol) + 1, 0: longer than kFast bits
  int maxcode[18];
  int valptr[17];
  int mincode[17];
  uint8_t vals[256];
  bool present = false;
  bool build(const uint8_t counts[16], const uint8_t* symbols, int nsym) {
    std::memset(fast, 0, sizeof(fast));
    int code = 0, k = 0;
    for (int len = 1; len <= 16; ++len) {
      valptr[len] = k;
      mincode[len] = code;
      code += counts[len - 1];
      k += counts[len - 1];
      if (code > (1 << len)) return false;  // over-subscribed
      maxcode[len] = counts[len - 1] ? code - 1 : -1;
      code <<= 1;
    }
    maxcode[17] = 0x7FFFFFFF;
    if (k != nsym) return false;
    std::memcpy(vals, symbols, (size_t)nsym);
    // fast table
    code = 0;
    k = 0;
    for (int len = 1; len <= kFast; ++len) {
      for (int i = 0; i < counts[len - 1]; ++i, ++k, ++code) {
        const int shift = kFast - len;
        for (int j = 0; j < (1 << shift); ++j) fast[(code << shift) | j] = (uint16_t)(((len << 8) | vals[k]) + 1);
      }
      code <<= 1;
    }
    present = true;
    return true;
  }
};

// Entropy-coded data: bits MSB first, 0xFF 0x00 stuffing removed; a marker
// ends the data (later reads give zero bits and flag an overrun).
struct Bits {
  const uint8_t* p;
  const uint8_t* end;
  uint64_t buf = 0;
  int cnt = 0;
  bool hit_marker = false;
  int marker = 0;
  int overrun = 0;  // bits fed past the data
  void fill() {
    while (cnt <= 56) {
      int b = 0;
      if (!hit_marker && p < end) {
        b = *p;
        if (b == 0xFF) {
          const int nxt = p + 1 < end ? p[1] : -1;
          if (nxt == 0x00) {
            p += 2;
          } else {
            hit_marker = true;
            marker = nxt;
            b = 0;
            overrun += 8;
          }
        } else {
          ++p;
        }
      } else {
        overrun += 8;
      }
      buf |= (uint64_t)b << (56 - cnt);
      cnt += 8;
    }
  }
  uint32_t get(int n) {  // n <= 16
    if (n == 0) return 0;
    if (cnt < n) fill();
    const uint32_t v = (uint32_t)(buf >> (64 - n));
    buf <<= n;
    cnt -= n;
    return v;
  }
  int decode(const Huff& h) {
    if (cnt < 16) fill();
    const uint16_t e = h.fast[buf >> (64 - Huff::kFast)];
    if (e) {
      const int len = (e - 1) >> 8;
      buf <<= len;
      cnt -= len;
      return (e - 1) & 0xFF;
    }
    for (int len = Huff::kFast + 1; len <= 16; ++len) {
      const int code = (int)(buf >> (64 - len));
      if (code <= h.maxcode[len]) {
        buf <<= len;
        cnt -= len;
        return h.vals[h.valptr[len] + code - h.mincode[len]];
      }
    }
    return -1;
  }
  // bits consumed beyond the real data (zeros fed after a marker or the end)
  bool past_end() const { return overrun > cnt; }
  // At a restart boundary: drop the padding bits and step over marker RSTn
  // (the reader stops at a marker without consuming it).
  bool restart(int expect) {
    buf = 0;
    cnt = 0;
    overrun = 0;
    hit_marker = false;
    const uint8_t* q = p;
    while (q + 1 < end && !(q[0] == 0xFF && q[1] != 0x00 && q[1] != 0xFF)) ++q;
    if (q + 1 >= end || q[1] != 0xD0 + expect) return false;
    p = q + 2;
    return true;
  }
};

// v rounded to the nearest integer (ties to even, as lrintf) and clamped to
// 0..255: v is clamped to [-1, 256] first (which rounds to the same clamped
// byte), then 1.5 * 2^23 + v, whose unit in the last place is 1, rounds it.
inline uint8_t round_clamp_u8(float v) {
  v = v < -1.0f ? -1.0f : (v > 256.0f ? 256.0f : v);
  const int iv = (int)((v + 12582912.0f) - 12582912.0f);
  return (uint8_t)(iv < 0 ? 0 : (iv > 255 ? 255 : iv));
}

inline int extend(uint32_t v, int s) { return s == 0 ? 0 : (v < (1u << (s - 1)) ? (int)v - (1 << s) + 1 : (int)v); }

struct Component {
  int id = 0, h = 1, v = 1, tq = 0;
  int td = 0, ta = 0;      // Huffman tables of the current scan
  int bw = 0, bh = 0;      // blocks across / down, padded to whole MCUs
  int pred = 0;            // DC prediction
  std::vector<int16_t> coef;  // bw * bh blocks x 64, natural order, quantised
};

struct Decoder {
  const uint8_t* d;
  size_t n;
  Err& err;
  int width = 0, height = 0, ncomp = 0, hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
  bool have_frame = false;
  bool progressive = false;
  bool jfif = false;         // an APP0 "JFIF" segment (YCbCr by definition)
  int adobe_transform = -1;  // the APP14 "Adobe" segment's colour transform, -1 without one
  // the current progressive scan: spectral band ss..se, successive approximation ah / al
  int ss = 0, se = 63, ah = 0, al = 0;
  int eobrun = 0;  // blocks left in the current end-of-band run
  int restart = 0;
  uint16_t qt[4][64];
  bool qt_set[4] = {false, false, false, false};
  Huff dc[4], ac[4];
  Component comp[3];
  Decoder(const uint8_t* data, size_t size, Err& e) : d(data), n(size), err(e) {}

  bool header_only(int* w, int* h) {
    size_t pos = 0;
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) return err.bad("not a JPEG file");
    pos = 2;
    while (pos + 4 <= n) {
      if (d[pos] != 0xFF) return err.bad("marker expected");
      const int m = d[pos + 1];
      if (m == 0xFF) {
        ++pos;
        continue;
      }
      const size_t len = (size_t)d[pos + 2] << 8 | d[pos + 3];
      if (len < 2 || pos + 2 + len > n) return err.bad("segment runs past the end of the file");
      if (m == 0xC0 || m == 0xC1 || m == 0xC2 || m == 0xC3) {
        if (len < 8) return err.bad("short frame header");
        *h = d[pos + 5] << 8 | d[pos + 6];
        *w = d[pos + 7] << 8 | d[pos + 8];
        if (*w <= 0 || *h <= 0) return err.bad("empty image (or a height given later by DNL, not supported)");
        return true;
      }
      pos += 2 + len;
    }
    return err.bad("no frame header");
  }

  bool frame(const uint8_t* s, size_t len, int m) {
    if (m != 0xC0 && m != 0xC1 && m != 0xC2)
      return err.bad("lossless, hierarchical or arithmetic-coded JPEG is not supported");
    if (have_frame) return err.bad("second frame header");
    progressive = m == 0xC2;
    if (len < 6) return err.bad("short frame header");
    if (s[0] != 8) return err.bad("only 8-bit samples are supported");
    height = s[1] << 8 | s[2];
    width = s[3] << 8 | s[4];
    ncomp = s[5];
    if (width <= 0 || height <= 0) return err.bad("empty image (or a height given later by DNL, not supported)");
    if (ncomp != 1 && ncomp != 3) return err.bad("only grey and three-component images are supported");
    if (len < 6 + 3 * (size_t)ncomp) return err.bad("short frame header");
    if ((int64_t)width * height > (1ll << 28)) return err.bad("image too large");
    hmax = vmax = 1;
    for (int i = 0; i < ncomp; ++i) {
      Component& c = comp[i];
      c.id = s[6 + 3 * i];
      c.h = s[7 + 3 * i] >> 4;
      c.v = s[7 + 3 * i] & 15;
      c.tq = s[8 + 3 * i];
      if (c.h < 1 || c.h > 2 || c.v < 1 || c.v > 2) return err.bad("sampling factors other than 1 and 2");
      if (c.tq > 3) return err.bad("bad quantisation table index");
      hmax = std::max(hmax, c.h);
      vmax = std::max(vmax, c.v);
    }
    if (ncomp == 1) comp[0].h = comp[0].v = hmax = vmax = 1;  // a single component is never subsampled
    mcux = (width + 8 * hmax - 1) / (8 * hmax);
    mcuy = (height + 8 * vmax - 1) / (8 * vmax);
    for (int i = 0; i < ncomp; ++i) {
      Component& c = comp[i];
      c.bw = mcux * c.h;
      c.bh = mcuy * c.v;
      c.coef.assign((size_t)c.bw * c.bh * 64, 0);
    }
    have_frame = true;
    return true;
  }

  bool dqt(const uint8_t* s, size_t len) {
    size_t i = 0;
    while (i < len) {
      const int pq = s[i] >> 4, tq = s[i] & 15;
      if (tq > 3 || pq > 1) return err.bad("bad quantisation table");
      const size_t need = 1 + 64 * (pq ? 2 : 1);
      if (i + need > len) return err.bad("short quantisation table");
      for (int k = 0; k < 64; ++k)
        qt[tq][kZigzag[k]] = pq ? (uint16_t)(s[i + 1 + 2 * k] << 8 | s[i + 2 + 2 * k]) : s[i + 1 + k];
      qt_set[tq] = true;
      i += need;
    }
    return true;
  }

  bool dht(const uint8_t* s, size_t len) {
    size_t i = 0;
    while (i < len) {
      if (i + 17 > len) return err.bad("short Huffman table");
      const int tc = s[i] >> 4, th = s[i] & 15;
      if (tc > 1 || th > 3) return err.bad("bad Huffman table");
      int total = 0;
      for (int k = 0; k < 16; ++k) total += s[i + 1 + k];
      if (total > 256 || i + 17 + total > len) return err.bad("bad Huffman table");
      if (!(tc ? ac[th] : dc[th]).build(s + i + 1, s + i + 17, total)) return err.bad("bad Huffman code lengths");
      i += 17 + total;
    }
    return true;
  }

  // One block: DC difference and AC run/size codes (T.81 F.2.2), natural order.
  bool block(Bits& b, Component& c, int16_t* out) {
    const Huff& hd = dc[c.td];
    const Huff& ha = ac[c.ta];
    const int t = b.decode(hd);
    if (t < 0 || t > 11) return err.bad("bad DC code");
    c.pred += extend(b.get(t), t);
    if (c.pred < -32768 || c.pred > 32767) return err.bad("DC value out of range");
    out[0] = (int16_t)c.pred;
    for (int k = 1; k < 64;) {
      const int rs = b.decode(ha);
      if (rs < 0) return err.bad("bad AC code");
      const int r = rs >> 4, sz = rs & 15;
      if (sz == 0) {
        if (r == 15) {
          k += 16;
          continue;
        }
        break;  // end of block
      }
      k += r;
      if (k > 63) return err.bad("AC coefficients run past the block");
      out[kZigzag[k]] = (int16_t)extend(b.get(sz), sz);
      ++k;
    }
    return true;
  }

  // Progressive scans (T.81 G.1.2), one block each; coefficients kept in
  // natural order, scaled by 2^al as they arrive.
  bool put_coef(int16_t* out, int z, int v) {
    if (v < -32768 || v > 32767) return err.bad("coefficient out of range");
    out[z] = (int16_t)v;
    return true;
  }
  // DC first scan: the DC difference, the prediction, the value << al.
  bool dc_first(Bits& b, Component& c, int16_t* out) {
    const int t = b.decode(dc[c.td]);
    if (t < 0 || t > 11) return err.bad("bad DC code");
    c.pred += extend(b.get(t), t);
    if (c.pred < -32768 || c.pred > 32767) return err.bad("DC value out of range");
    return put_coef(out, 0, c.pred * (1 << al));
  }
  // DC refinement: one bit, bit al of the DC value.
  void dc_refine(Bits& b, int16_t* out) {
    if (b.get(1)) out[0] = (int16_t)(out[0] | (1 << al));
  }
  // AC first scan of band ss..se: run/size codes, ZRL, and end-of-band runs
  // (symbol r << 4 with r < 15: 2^r blocks plus r more bits, this one included).
  bool ac_first(Bits& b, Component& c, int16_t* out) {
    if (eobrun > 0) {
      --eobrun;
      return true;
    }
    const Huff& ha = ac[c.ta];
    for (int k = ss; k <= se;) {
      const int rs = b.decode(ha);
      if (rs < 0) return err.bad("bad AC code");
      const int r = rs >> 4, sz = rs & 15;
      if (sz == 0) {
        if (r == 15) {
          k += 16;
          continue;
        }
        eobrun = (1 << r) - 1;
        if (r) eobrun += (int)b.get(r);
        break;
      }
      k += r;
      if (k > se) return err.bad("AC coefficients run past the band");
      if (!put_coef(out, kZigzag[k], extend(b.get(sz), sz) * (1 << al))) return false;
      ++k;
    }
    return true;
  }
  // A correction bit for a coefficient already nonzero: when set, bit al is
  // added to its magnitude (if not there yet).
  bool correct(Bits& b, int16_t* out, int z) {
    if (!b.get(1)) return true;
    const int p1 = 1 << al, v = out[z];
    if ((v & p1) != 0) return true;
    return put_coef(out, z, v >= 0 ? v + p1 : v - p1);
  }
  // AC refinement of band ss..se at bit al: each code places one new
  // coefficient of magnitude 2^al (its sign the next bit) after r zero-history
  // positions, or skips 16 of them (ZRL), or starts an end-of-band run; every
  // already-nonzero coefficient passed on the way takes a correction bit, as do
  // those of the rest of the block in an end-of-band run.
  bool ac_refine(Bits& b, Component& c, int16_t* out) {
    const int p1 = 1 << al;
    int k = ss;
    if (eobrun == 0) {
      const Huff& ha = ac[c.ta];
      while (k <= se) {
        const int rs = b.decode(ha);
        if (rs < 0) return err.bad("bad AC code");
        int r = rs >> 4;
        const int sz = rs & 15;
        int val = 0;
        if (sz != 0) {
          if (sz != 1) return err.bad("bad refinement code");
          val = b.get(1) ? p1 : -p1;
        } else if (r != 15) {
          eobrun = 1 << r;
          if (r) eobrun += (int)b.get(r);
          break;
        }
        bool placed = false;
        while (k <= se) {
          const int z = kZigzag[k];
          if (out[z] != 0) {
            if (!correct(b, out, z)) return false;
          } else {
            if (r == 0) {
              if (val) out[z] = (int16_t)val;
              ++k;
              placed = true;
              break;
            }
            --r;
          }
          ++k;
        }
        if (!placed && (val != 0 || r > 0)) return err.bad("refinement runs past the band");
      }
    }
    if (eobrun > 0) {
      for (; k <= se; ++k) {
        const int z = kZigzag[k];
        if (out[z] != 0 && !correct(b, out, z)) return false;
      }
      --eobrun;
    }
    return true;
  }
  bool prog_block(Bits& b, Component& c, int16_t* out) {
    if (ss == 0) {
      if (ah == 0) return dc_first(b, c, out);
      dc_refine(b, out);
      return true;
    }
    return ah == 0 ? ac_first(b, c, out) : ac_refine(b, c, out);
  }

  bool scan(const uint8_t* s, size_t len, size_t& pos) {
    if (!have_frame) return err.bad("scan before the frame header");
    if (len < 1) return err.bad("short scan header");
    const int ns = s[0];
    if (ns < 1 || ns > ncomp || len < 4 + 2 * (size_t)ns) return err.bad("bad scan header");
    Component* sc[3];
    for (int i = 0; i < ns; ++i) {
      const int id = s[1 + 2 * i];
      int j = 0;
      while (j < ncomp && comp[j].id != id) ++j;
      if (j == ncomp) return err.bad("scan names an unknown component");
      sc[i] = &comp[j];
      sc[i]->td = s[2 + 2 * i] >> 4;
      sc[i]->ta = s[2 + 2 * i] & 15;
      if (sc[i]->td > 3 || sc[i]->ta > 3) return err.bad("bad Huffman table index");
      sc[i]->pred = 0;
    }
    ss = s[1 + 2 * ns];
    se = s[2 + 2 * ns];
    ah = s[3 + 2 * ns] >> 4;
    al = s[3 + 2 * ns] & 15;
    eobrun = 0;
    if (!progressive) {
      if (ss != 0 || se != 63 || ah != 0 || al != 0)
        return err.bad("spectral selection or successive approximation in a sequential scan");
    } else {
      if (ss == 0 ? se != 0 : (se < ss || se > 63 || ns != 1))
        return err.bad("bad spectral selection in a progressive scan");
      if (al > 13 || (ah != 0 && ah != al + 1)) return err.bad("bad successive approximation");
    }
    // the tables a scan decodes with: DC codes in sequential and first DC
    // scans, AC codes in sequential and AC scans (a DC refinement uses none)
    for (int i = 0; i < ns; ++i) {
      const bool need_dc = !progressive || (ss == 0 && ah == 0), need_ac = !progressive || ss > 0;
      if ((need_dc && !dc[sc[i]->td].present) || (need_ac && !ac[sc[i]->ta].present))
        return err.bad("scan uses a missing Huffman table");
    }
    // entropy-coded data
    Bits b{d + pos, d + n};
    int mx, my;
    if (ns == 1) {  // one component: its own block grid (T.81 A.2.2), not padded to whole MCUs
      mx = (int)std::ceil((double)width * sc[0]->h / hmax / 8.0);
      my = (int)std::ceil((double)height * sc[0]->v / vmax / 8.0);
    } else {
      mx = mcux;
      my = mcuy;
    }
    const int64_t units = (int64_t)mx * my;
    int64_t left = restart;
    int next_rst = 0;
    for (int64_t u = 0; u < units; ++u) {
      if (restart && left == 0) {
        if (!b.restart(next_rst)) return err.bad("restart marker missing or out of order");
        next_rst = (next_rst + 1) & 7;
        for (int i = 0; i < ns; ++i) sc[i]->pred = 0;
        eobrun = 0;
        left = restart;
      }
      if (ns == 1) {
        Component& c = *sc[0];
        const int bx = (int)(u % mx), by = (int)(u / mx);
        int16_t* blk = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
        if (!(progressive ? prog_block(b, c, blk) : block(b, c, blk))) return false;
      } else {
        const int ux = (int)(u % mx), uy = (int)(u / mx);
        for (int i = 0; i < ns; ++i) {
          Component& c = *sc[i];
          for (int y = 0; y < c.v; ++y)
            for (int x = 0; x < c.h; ++x) {
              const int bx = ux * c.h + x, by = uy * c.v + y;
              int16_t* blk = c.coef.data() + ((size_t)by * c.bw + bx) * 64;
              if (!(progressive ? prog_block(b, c, blk) : block(b, c, blk))) return false;
            }
        }
      }
      if (b.past_end()) return err.bad("entropy-coded data truncated");
      if (restart) --left;
    }
    // continue after the scan's data at the next marker (RSTn and fill bytes skipped)
    const uint8_t* q = b.p;
    while (q + 1 < d + n && !(q[0] == 0xFF && q[1] != 0x00 && !(q[1] >= 0xD0 && q[1] <= 0xD7) && q[1] != 0xFF)) ++q;
    pos = (size_t)(q - d);
    return true;
  }

  bool parse() {
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) return err.bad("not a JPEG file");
    size_t pos = 2;
    bool scanned = false;
    while (pos + 2 <= n) {
      if (d[pos] != 0xFF) return err.bad("marker expected");
      const int m = d[pos + 1];
      if (m == 0xFF) {
        ++pos;
        continue;
      }
      if (m == 0xD9) break;  // EOI
      if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7) || m == 0x01) {
        pos += 2;
        continue;
      }
      if (pos + 4 > n) return err.bad("truncated segment");
      const size_t len = (size_t)d[pos + 2] << 8 | d[pos + 3];
      if (len < 2 || pos + 2 + len > n) return err.bad("segment runs past the end of the file");
      const uint8_t* s = d + pos + 4;
      const size_t sl = len - 2;
      pos += 2 + len;
      if (m >= 0xC0 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
        if (!frame(s, sl, m)) return false;
      } else if (m == 0xC4) {
        if (!dht(s, sl)) return false;
      } else if (m == 0xCC) {
        return err.bad("arithmetic-coded JPEG is not supported");
      } else if (m == 0xDB) {
        if (!dqt(s, sl)) return false;
      } else if (m == 0xDD) {
        if (sl < 2) return err.bad("short restart interval");
        restart = s[0] << 8 | s[1];
      } else if (m == 0xDA) {
        if (!scan(s, sl, pos)) return false;
        scanned = true;
      } else if (m == 0xDC) {
        return err.bad("DNL (height defined later) is not supported");
      } else if (m == 0xE0 && sl >= 5 && std::memcmp(s, "JFIF", 5) == 0) {
        jfif = true;
      } else if (m == 0xEE && sl >= 12 && std::memcmp(s, "Adobe", 5) == 0) {
        adobe_transform = s[11];  // 0: no colour transform, 1: YCbCr, 2: YCCK
      }
      // other APPn, COM and the rest: skipped
    }
    if (!have_frame) return err.bad("no frame header");
    if (!scanned) return err.bad("no scan");
    for (int i = 0; i < ncomp; ++i)
      if (!qt_set[comp[i].tq]) return err.bad("missing quantisation table");
    return true;
  }

  // T.81 A.3.3 inverse DCT of one dequantised block, rows then columns, FP32,
  // + 128, rounded to nearest, clamped.  Each output is a sum from 0 over the
  // eight frequencies in order; the loops run the eight outputs of a row (or
  // column pass) side by side (ct[u][x] = cs[x][u]) so that the compiler can
  // keep them in vector lanes without reordering any sum.
  static void idct(const int16_t* in, const uint16_t* q, uint8_t* out, int stride, const float (&ct)[8][8]) {
    float t[64];
    for (int u = 0; u < 64; ++u) t[u] = (float)in[u] * (float)q[u];
    float r[64];
    for (int y = 0; y < 8; ++y) {  // 1-D over the horizontal frequency of each row
      float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
      for (int u = 0; u < 8; ++u) {
        const float tu = t[y * 8 + u];
        for (int x = 0; x < 8; ++x) s[x] += ct[u][x] * tu;
      }
      for (int x = 0; x < 8; ++x) r[y * 8 + x] = s[x];
    }
    for (int y = 0; y < 8; ++y) {  // then over the vertical frequency of each column
      float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
      for (int v = 0; v < 8; ++v) {
        const float c = ct[v][y];
        for (int x = 0; x < 8; ++x) s[x] += c * r[v * 8 + x];
      }
      for (int x = 0; x < 8; ++x) out[y * stride + x] = round_clamp_u8(s[x] + 128.0f);
    }
  }

  // Three components stored as R, G, B rather than YCbCr: an Adobe segment
  // saying "no transform", or no JFIF or Adobe segment and components named
  // 'R', 'G', 'B' (the conventions of T.872 and libjpeg-era writers).
  bool rgb_samples() const {
    if (ncomp != 3) return false;
    if (adobe_transform >= 0) return adobe_transform == 0;
    return !jfif && comp[0].id == 'R' && comp[1].id == 'G' && comp[2].id == 'B';
  }

  bool output(uint8_t* out, int64_t stride) {
    float ct[8][8];  // ct[u][x] = C(u)/2 cos((2x+1) u pi / 16)
    for (int x = 0; x < 8; ++x)
      for (int u = 0; u < 8; ++u)
        ct[u][x] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * M_PI / 16.0));
    std::vector<std::vector<uint8_t>> plane(ncomp);
    for (int i = 0; i < ncomp; ++i) {
      Component& c = comp[i];
      const int pw = c.bw * 8, ph = c.bh * 8;
      plane[i].assign((size_t)pw * ph, 0);
      for (int by = 0; by < c.bh; ++by)
        for (int bx = 0; bx < c.bw; ++bx)
          idct(c.coef.data() + ((size_t)by * c.bw + bx) * 64, qt[c.tq], plane[i].data() + (size_t)by * 8 * pw + bx * 8,
               pw, ct);
    }
    for (int y = 0; y < height; ++y) {
      uint8_t* o = out + (int64_t)y * stride;
      if (ncomp == 1) {
        const uint8_t* p = plane[0].data() + (size_t)y * comp[0].bw * 8;
        for (int x = 0; x < width; ++x) o[3 * x] = o[3 * x + 1] = o[3 * x + 2] = p[x];
        continue;
      }
      if (rgb_samples()) {  // three components that are R, G and B themselves
        const uint8_t* row[3];
        int sh[3];
        for (int i = 0; i < 3; ++i) {
          const Component& c = comp[i];
          row[i] = plane[i].data() + (size_t)(y * c.v / vmax) * c.bw * 8;
          sh[i] = hmax / c.h == 2 ? 1 : 0;
        }
        for (int x = 0; x < width; ++x)
          for (int i = 0; i < 3; ++i) o[3 * x + i] = row[i][x >> sh[i]];
        continue;
      }
      const uint8_t* row[3];
      int sh[3];  // horizontal replication: x >> sh (factors 1 or 2)
      for (int i = 0; i < 3; ++i) {
        const Component& c = comp[i];
        const int yy = y * c.v / vmax;  // replication
        row[i] = plane[i].data() + (size_t)yy * c.bw * 8;
        sh[i] = hmax / c.h == 2 ? 1 : 0;
      }
      for (int x = 0; x < width; ++x) {
        const float Y = row[0][x >> sh[0]], cb = row[1][x >> sh[1]] - 128.0f, cr = row[2][x >> sh[2]] - 128.0f;
        o[3 * x] = round_clamp_u8(Y + 1.402f * cr);
        o[3 * x + 1] = round_clamp_u8(Y - 0.344136f * cb - 0.714136f * cr);
        o[3 * x + 2] = round_clamp_u8(Y + 1.772f * cb);
      }
    }
    return true;
  }
};

int jpeg_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride, Err& e) {
  if (!data || !out) return e.bad("null argument"), e.code;
  Decoder dec(data, n, e);
  if (!dec.parse()) return e.code;
  if (stride < 3ll * dec.width) return e.bad("output stride below 3 * width"), e.code;
  dec.output(out, stride);
  return MG_OK;
}

bool is_jpeg(const uint8_t* d, size_t n) { return d && n >= 3 && d[0] == 0xFF && d[1] == 0xD8 && d[2] == 0xFF; }
bool is_png(const uint8_t* d, size_t n) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  return d && n >= 8 && std::memcmp(d, sig, 8) == 0;
}

// ---- encoder (the output end: image::save of a .jpg / .jpeg path) ----------------
//
// Baseline JFIF (T.81 sequential DCT, Huffman): YCbCr with 4:2:0 chroma (the
// mean of each 2x2 box), the forward DCT in FP32 with the decoder's cosine
// table, the T.81 Annex K.1 quantisation tables scaled by quality with the
// IJG rule (q < 50: 5000 / q percent, else 200 - 2q), rounding half away from
// zero; Huffman codes built from this image's own symbol counts (T.81 Annex
// K.2: code sizes, then lengths limited to 16 bits); one restart interval per
// row of MCUs, so the rows are entropy-coded on all threads and joined with
// RSTn markers.  The output bytes are not those of the crate's encoder (not
// pinned); any JPEG reader decodes them.

const uint8_t kQLuma[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                            14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                            18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                            49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
const uint8_t kQChroma[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                              24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                              99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

void scaled_quant(const uint8_t* base, int quality, uint8_t* q) {
  const int scale = quality < 50 ? 5000 / quality : 200 - 2 * quality;
  for (int i = 0; i < 64; ++i) q[i] = (uint8_t)std::min(255, std::max(1, (base[i] * scale + 50) / 100));
}

// A Huffman code from symbol counts (T.81 K.2): code sizes by repeatedly
// merging the two least frequent nodes, a reserved symbol (count 1) keeping
// the all-ones code out, then lengths limited to 16 bits (Adjust_BITS) and the
// reserved code dropped from the longest length.
struct HuffCode {
  uint8_t bits[16] = {};   // codes per length 1..16
  uint8_t vals[256] = {};  // symbols in code order
  int nvals = 0;
  uint16_t code[256] = {};
  uint8_t size[256] = {};
  void build(const uint64_t* freq_in) {
    uint64_t freq[257];
    for (int i = 0; i < 256; ++i) freq[i] = freq_in[i];
    freq[256] = 1;
    int codesize[257] = {}, others[257];
    for (int i = 0; i < 257; ++i) others[i] = -1;
    for (;;) {
      int c1 = -1, c2 = -1;  // least, then next least nonzero count (ties: the larger symbol first)
      for (int i = 0; i < 257; ++i) {
        if (freq[i] == 0) continue;
        if (c1 < 0 || freq[i] <= freq[c1]) {
          c2 = c1;
          c1 = i;
        } else if (c2 < 0 || freq[i] <= freq[c2]) {
          c2 = i;
        }
      }
      if (c2 < 0) break;
      freq[c1] += freq[c2];
      freq[c2] = 0;
      ++codesize[c1];
      while (others[c1] >= 0) {
        c1 = others[c1];
        ++codesize[c1];
      }
      others[c1] = c2;
      ++codesize[c2];
      while (others[c2] >= 0) {
        c2 = others[c2];
        ++codesize[c2];
      }
    }
    int count[258] = {};  // a code size is at most 256 (257 symbols)
    int maxsize = 0;
    for (int i = 0; i < 257; ++i)
      if (codesize[i]) {
        ++count[codesize[i]];
        maxsize = std::max(maxsize, codesize[i]);
      }
    for (int i = maxsize; i > 16; --i)
      while (count[i] > 0) {
        int j = i - 2;
        while (count[j] == 0) --j;
        count[i] -= 2;
        count[i - 1] += 1;
        count[j + 1] += 2;
        count[j] -= 1;
      }
    int longest = 16;
    while (longest > 0 && count[longest] == 0) --longest;
    if (longest > 0) --count[longest];  // the reserved symbol's code
    for (int i = 0; i < 16; ++i) bits[i] = (uint8_t)count[i + 1];
    nvals = 0;
    for (int len = 1; len <= maxsize; ++len)
      for (int sym = 0; sym < 256; ++sym)
        if (codesize[sym] == len) vals[nvals++] = (uint8_t)sym;
    int k = 0, c = 0;
    for (int len = 1; len <= 16; ++len) {
      for (int i = 0; i < bits[len - 1]; ++i, ++k, ++c) {
        code[vals[k]] = (uint16_t)c;
        size[vals[k]] = (uint8_t)len;
      }
      c <<= 1;
    }
  }
};

struct BitSink {
  std::vector<uint8_t> out;
  uint32_t acc = 0;
  int n = 0;
  void put(uint32_t v, int bits) {  // bits <= 16
    acc = (acc << bits) | (v & ((1u << bits) - 1u));
    n += bits;
    while (n >= 8) {
      const uint8_t b = (uint8_t)(acc >> (n - 8));
      out.push_back(b);
      if (b == 0xFF) out.push_back(0x00);
      n -= 8;
    }
    acc &= (1u << n) - 1u;
  }
  void pad() {
    if (n) put((1u << (8 - n)) - 1u, 8 - n);
  }
};

inline int category(int v) {
  int a = v < 0 ? -v : v, s = 0;
  while (a) {
    ++s;
    a >>= 1;
  }
  return s;
}

struct Encoder {
  int w, h, mcux, mcuy;
  uint8_t qt[2][64];  // natural order
  // quantised coefficients, natural order: Y blocks (2 mcux x 2 mcuy), Cb, Cr (mcux x mcuy)
  std::vector<int16_t> coef[3];
  int bw[3], bh[3];

  // One MCU row: pixel rows 16 my .. 16 my + 15 (edges replicated) to YCbCr,
  // chroma averaged over 2x2, forward DCT, quantisation.
  void transform_row(const uint8_t* rgb, int64_t stride, int my, const float (&ct)[8][8]) {
    const int pw = mcux * 16;
    std::vector<float> Y((size_t)16 * pw), cb((size_t)16 * pw), cr((size_t)16 * pw);
    for (int y = 0; y < 16; ++y) {
      const int sy = std::min(h - 1, my * 16 + y);
      const uint8_t* row = rgb + (int64_t)sy * stride;
      for (int x = 0; x < pw; ++x) {
        const uint8_t* px = row + 3 * std::min(w - 1, x);
        const float r = px[0], g = px[1], b = px[2];
        Y[(size_t)y * pw + x] = 0.299f * r + 0.587f * g + 0.114f * b - 128.0f;
        cb[(size_t)y * pw + x] = -0.168736f * r - 0.331264f * g + 0.5f * b;
        cr[(size_t)y * pw + x] = 0.5f * r - 0.418688f * g - 0.081312f * b;
      }
    }
    float blk[64];
    for (int bx = 0; bx < 2 * mcux; ++bx)
      for (int by = 0; by < 2; ++by) {
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x) blk[y * 8 + x] = Y[(size_t)(by * 8 + y) * pw + bx * 8 + x];
        fdct_quant(blk, qt[0], coef[0].data() + ((size_t)(2 * my + by) * bw[0] + bx) * 64, ct);
      }
    for (int c = 1; c < 3; ++c) {
      const std::vector<float>& p = c == 1 ? cb : cr;
      for (int bx = 0; bx < mcux; ++bx) {
        for (int y = 0; y < 8; ++y)
          for (int x = 0; x < 8; ++x) {
            const size_t o = (size_t)(2 * y) * pw + 2 * (bx * 8 + x);
            blk[y * 8 + x] = 0.25f * (p[o] + p[o + 1] + p[o + pw] + p[o + pw + 1]);
          }
        fdct_quant(blk, qt[1], coef[c].data() + ((size_t)my * bw[c] + bx) * 64, ct);
      }
    }
  }
  // F(u, v) = sum_y ct[v][y] sum_x ct[u][x] f(x, y), then F / Q rounded half away from zero.
  static void fdct_quant(const float* f, const uint8_t* q, int16_t* out, const float (&ct)[8][8]) {
    float r[64];
    for (int y = 0; y < 8; ++y) {
      float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
      for (int x = 0; x < 8; ++x) {
        const float fx = f[y * 8 + x];
        for (int u = 0; u < 8; ++u) s[u] += ct[u][x] * fx;
      }
      for (int u = 0; u < 8; ++u) r[y * 8 + u] = s[u];
    }
    for (int v = 0; v < 8; ++v) {
      float s[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
      for (int y = 0; y < 8; ++y) {
        const float c = ct[v][y];
        for (int u = 0; u < 8; ++u) s[u] += c * r[y * 8 + u];
      }
      for (int u = 0; u < 8; ++u) {
        const float t = s[u] / (float)q[v * 8 + u];
        const int r = t >= 0.0f ? (int)(t + 0.5f) : -(int)(0.5f - t);
        const int lim = u + v ? 1023 : 2047;  // baseline: AC categories up to 10, DC up to 11
        out[v * 8 + u] = (int16_t)std::max(-lim, std::min(lim, r));
      }
    }
  }
  // The blocks of MCU row my in scan order (Y 2x2, Cb, Cr per MCU), calling
  // f(component, block coefficients).
  template <class F>
  void walk_row(int my, F&& f) const {
    for (int mx = 0; mx < mcux; ++mx) {
      for (int by = 0; by < 2; ++by)
        for (int bx = 0; bx < 2; ++bx) f(0, coef[0].data() + ((size_t)(2 * my + by) * bw[0] + 2 * mx + bx) * 64);
      for (int c = 1; c < 3; ++c) f(c, coef[c].data() + ((size_t)my * bw[c] + mx) * 64);
    }
  }
  // Symbol counts of MCU row my (DC prediction restarts with the row): [table][symbol]
  void count_row(int my, uint64_t (*freq)[256]) const {
    int pred[3] = {0, 0, 0};
    walk_row(my, [&](int c, const int16_t* b) {
      const int t = c ? 1 : 0;
      ++freq[2 * t][category(b[0] - pred[c])];
      pred[c] = b[0];
      int run = 0;
      for (int k = 1; k < 64; ++k) {
        const int v = b[kZigzag[k]];
        if (v == 0) {
          ++run;
          continue;
        }
        while (run > 15) {
          ++freq[2 * t + 1][0xF0];
          run -= 16;
        }
        ++freq[2 * t + 1][(run << 4) | category(v)];
        run = 0;
      }
      if (run) ++freq[2 * t + 1][0x00];
    });
  }
  void code_row(int my, const HuffCode* hc, BitSink& bs) const {
    int pred[3] = {0, 0, 0};
    walk_row(my, [&](int c, const int16_t* b) {
      const HuffCode& dc = hc[c ? 2 : 0];
      const HuffCode& ac = hc[c ? 3 : 1];
      const int diff = b[0] - pred[c];
      pred[c] = b[0];
      int s = category(diff);
      bs.put(dc.code[s], dc.size[s]);
      if (s) bs.put((uint32_t)(diff < 0 ? diff + (1 << s) - 1 : diff), s);
      int run = 0;
      for (int k = 1; k < 64; ++k) {
        const int v = b[kZigzag[k]];
        if (v == 0) {
          ++run;
          continue;
        }
        while (run > 15) {
          bs.put(ac.code[0xF0], ac.size[0xF0]);
          run -= 16;
        }
        s = category(v);
        const int sym = (run << 4) | s;
        bs.put(ac.code[sym], ac.size[sym]);
        bs.put((uint32_t)(v < 0 ? v + (1 << s) - 1 : v), s);
        run = 0;
      }
      if (run) bs.put(ac.code[0x00], ac.size[0x00]);
    });
    bs.pad();
  }
};

template <class F>
void run_threads(int threads, int items, F&& f) {
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int i; (i = next.fetch_add(1)) < items;) f(i);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) {
    try {
      pool.emplace_back(work);
    } catch (const std::exception&) {
      break;  // the threads running (and this one) take the rest
    }
  }
  work();
  for (auto& t : pool) t.join();
}

void put_segment(std::vector<uint8_t>& o, int marker, const std::vector<uint8_t>& body) {
  o.push_back(0xFF);
  o.push_back((uint8_t)marker);
  o.push_back((uint8_t)((body.size() + 2) >> 8));
  o.push_back((uint8_t)(body.size() + 2));
  o.insert(o.end(), body.begin(), body.end());
}

// The whole file into `file` (MG_OK) or an error code.
int jpeg_encode(const uint8_t* rgb, int w, int h, int64_t stride, int quality, int threads, std::vector<uint8_t>& file) {
  Encoder E;
  E.w = w;
  E.h = h;
  E.mcux = (w + 15) / 16;
  E.mcuy = (h + 15) / 16;
  scaled_quant(kQLuma, quality, E.qt[0]);
  scaled_quant(kQChroma, quality, E.qt[1]);
  E.bw[0] = 2 * E.mcux;
  E.bh[0] = 2 * E.mcuy;
  E.bw[1] = E.bw[2] = E.mcux;
  E.bh[1] = E.bh[2] = E.mcuy;
  for (int c = 0; c < 3; ++c) E.coef[c].assign((size_t)E.bw[c] * E.bh[c] * 64, 0);
  float ct[8][8];  // ct[u][x] = C(u)/2 cos((2x+1) u pi / 16), as the decoder's
  for (int x = 0; x < 8; ++x)
    for (int u = 0; u < 8; ++u)
      ct[u][x] = (float)((u == 0 ? std::sqrt(0.5) : 1.0) * 0.5 * std::cos((2 * x + 1) * u * M_PI / 16.0));
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::max(1, std::min(threads, E.mcuy));
  run_threads(threads, E.mcuy, [&](int my) { E.transform_row(rgb, stride, my, ct); });
  std::vector<std::array<std::array<uint64_t, 256>, 4>> counts((size_t)E.mcuy);
  run_threads(threads, E.mcuy, [&](int my) {
    uint64_t f[4][256] = {};
    E.count_row(my, f);
    for (int t = 0; t < 4; ++t)
      for (int s = 0; s < 256; ++s) counts[my][t][s] = f[t][s];
  });
  uint64_t total[4][256] = {};
  for (const auto& c : counts)
    for (int t = 0; t < 4; ++t)
      for (int s = 0; s < 256; ++s) total[t][s] += c[t][s];
  HuffCode hc[4];  // DC luma, AC luma, DC chroma, AC chroma
  for (int t = 0; t < 4; ++t) hc[t].build(total[t]);
  std::vector<BitSink> rows((size_t)E.mcuy);
  run_threads(threads, E.mcuy, [&](int my) { E.code_row(my, hc, rows[my]); });
  // headers
  file.clear();
  file.insert(file.end(), {0xFF, 0xD8});
  put_segment(file, 0xE0, {'J', 'F', 'I', 'F', 0, 1, 2, 0, 0, 1, 0, 1, 0, 0});
  std::vector<uint8_t> dqt;
  for (int t = 0; t < 2; ++t) {
    dqt.push_back((uint8_t)t);
    for (int k = 0; k < 64; ++k) dqt.push_back(E.qt[t][kZigzag[k]]);
  }
  put_segment(file, 0xDB, dqt);
  put_segment(file, 0xC0,
              {8, (uint8_t)(h >> 8), (uint8_t)h, (uint8_t)(w >> 8), (uint8_t)w, 3, 1, 0x22, 0, 2, 0x11, 1, 3, 0x11, 1});
  std::vector<uint8_t> dht;
  for (int t = 0; t < 4; ++t) {
    dht.push_back((uint8_t)(((t & 1) << 4) | (t >> 1)));
    dht.insert(dht.end(), hc[t].bits, hc[t].bits + 16);
    dht.insert(dht.end(), hc[t].vals, hc[t].vals + hc[t].nvals);
  }
  put_segment(file, 0xC4, dht);
  put_segment(file, 0xDD, {(uint8_t)(E.mcux >> 8), (uint8_t)E.mcux});
  put_segment(file, 0xDA, {3, 1, 0x00, 2, 0x11, 3, 0x11, 0, 63, 0});
  for (int my = 0; my < E.mcuy; ++my) {
    if (my) file.insert(file.end(), {0xFF, (uint8_t)(0xD0 + ((my - 1) & 7))});
    file.insert(file.end(), rows[my].out.begin(), rows[my].out.end());
  }
  file.insert(file.end(), {0xFF, 0xD9});
  return MG_OK;
}

}  // namespace

extern "C" {

int mg_jpeg_info(const uint8_t* data, size_t n, int* w, int* h) {
  Err e;
  if (!data || !w || !h) {
    mg::set_error("null argument");
    return MG_ERR_ARG;
  }
  try {
    Decoder dec(data, n, e);
    if (!dec.header_only(w, h)) {
      mg::set_error(e.msg);
      return e.code;
    }
    return MG_OK;
  } catch (const std::exception& x) {
    mg::set_error(std::string("JPEG: ") + x.what());
    return MG_ERR_OOM;
  }
}

int mg_jpeg_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride) {
  Err e;
  try {
    const int rc = jpeg_decode(data, n, out, stride, e);
    if (rc != MG_OK) mg::set_error(e.msg);
    return rc;
  } catch (const std::bad_alloc&) {
    mg::set_error("JPEG: out of memory");
    return MG_ERR_OOM;
  } catch (const std::exception& x) {
    mg::set_error(std::string("JPEG: ") + x.what());
    return MG_ERR_ARG;
  }
}

int mg_image_info(const uint8_t* data, size_t n, int* w, int* h) {
  if (is_png(data, n)) return mg_png_info(data, n, w, h);
  if (is_jpeg(data, n)) return mg_jpeg_info(data, n, w, h);
  mg::set_error("neither a PNG nor a JPEG file");
  return MG_ERR_ARG;
}

int mg_image_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride) {
  if (is_png(data, n)) return mg_png_decode(data, n, out, stride);
  if (is_jpeg(data, n)) return mg_jpeg_decode(data, n, out, stride);
  mg::set_error("neither a PNG nor a JPEG file");
  return MG_ERR_ARG;
}

int mg_image_decode_batch(const uint8_t* const* data, const size_t* n, int count, uint8_t* const* out,
                          const int64_t* stride, int threads, int* status) {
  if (count < 0 || (count > 0 && (!data || !n || !out || !stride))) {
    mg::set_error("invalid arguments");
    return MG_ERR_ARG;
  }
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::max(1, std::min(threads, count));
  std::vector<int> st((size_t)std::max(count, 1), MG_OK);
  std::vector<std::string> msg((size_t)std::max(count, 1));
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int i; (i = next.fetch_add(1)) < count;) {
      st[i] = mg_image_decode(data[i], n[i], out[i], stride[i]);
      if (st[i] != MG_OK) msg[i] = mg_last_error();
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) {
    try {
      pool.emplace_back(work);
    } catch (const std::exception&) {
      break;  // the threads running (and this one) take the rest
    }
  }
  work();
  for (auto& t : pool) t.join();
  int first = MG_OK;
  for (int i = 0; i < count; ++i) {
    if (status) status[i] = st[i];
    if (st[i] != MG_OK && first == MG_OK) {
      first = st[i];
      mg::set_error("file " + std::to_string(i) + ": " + msg[i]);
    }
  }
  return first;
}

size_t mg_jpeg_encode_bound(int w, int h) {
  if (w <= 0 || h <= 0 || w > 65535 || h > 65535) return 0;
  const size_t mcus = (size_t)((w + 15) / 16) * ((h + 15) / 16);
  // per block at most 16 + 11 bits of DC and 63 x (16 + 10) bits of AC, doubled for 0xFF stuffing
  return 4096 + mcus * 6 * 2 * ((27 + 63 * 26 + 7) / 8) + 2 * (size_t)((h + 15) / 16);
}

int mg_jpeg_encode(const uint8_t* rgb, int w, int h, int64_t stride, int quality, int threads, uint8_t* out,
                   size_t cap, size_t* len) {
  const size_t bound = mg_jpeg_encode_bound(w, h);
  if (!rgb || !out || !len || bound == 0 || stride < 3ll * w || quality < 1 || quality > 100) {
    mg::set_error("invalid arguments (sizes 1..65535, quality 1..100)");
    return MG_ERR_ARG;
  }
  if (cap < bound) {
    *len = bound;
    mg::set_error("output buffer smaller than mg_jpeg_encode_bound");
    return MG_ERR_ARG;
  }
  try {
    std::vector<uint8_t> file;
    const int st = jpeg_encode(rgb, w, h, stride, quality, threads, file);
    if (st != MG_OK) return st;
    if (file.size() > cap) {  // cannot happen within the bound; kept as a guard
      mg::set_error("JPEG larger than its bound");
      return MG_ERR_ARG;
    }
    std::memcpy(out, file.data(), file.size());
    *len = file.size();
    return MG_OK;
  } catch (const std::bad_alloc&) {
    mg::set_error("out of host memory");
    return MG_ERR_OOM;
  } catch (const std::exception& e) {
    mg::set_error(e.what());
    return MG_ERR_ARG;
  }
}

}  // extern "C"
