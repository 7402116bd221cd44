// oracle.cpp -- CPU restatement of mosaic-art-rust's tile matching-and-placement
// path.  TEST INFRASTRUCTURE ONLY (the checker for the CUDA library, and the
// timed CPU baseline); the shipped library never links or calls this file.
//
// Build: oracle/Makefile (g++ -O2 -ffp-contract=off, no -march flags, so x86 and
// Arm hosts give identical bits).  FMA contraction is off; every fused
// multiply-add below is an explicit std::fmaf, which is correctly rounded.
//
// Parity: pinned only by the reference's known-answer tests (see oracle.h);
// third-party arithmetic (palette 0.7.6, kiddo 5.2.2, rand 0.8.5) is restated
// from the published algorithms, and its last-bit agreement is unpinned.

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }

// Rust f32::clamp (NaN passes through).
inline float rclamp(float v, float lo, float hi) {
  if (v < lo) v = lo;
  if (v > hi) v = hi;
  return v;
}
// Rust `f as u8`: saturating, truncating toward zero, NaN -> 0.
inline uint8_t as_u8(float v) {
  if (!(v == v)) return 0;
  if (v <= 0.0f) return 0;
  if (v >= 255.0f) return 255;
  return (uint8_t)(int)v;
}

template <class F>
void parallel_for(int n, int threads, F fn) {
  if (threads <= 1 || n <= 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  threads = std::min(threads, n);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([=, &fn]() {
      for (int i = t; i < n; i += threads) fn(i);
    });
  for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------------------
// sRGB -> CIE Lab.  palette 0.7.6 `Lab::from_color(Srgb)` (lib.rs:102-107):
// IEC 61966-2-1 transfer function, RGB->XYZ matrix derived from the sRGB
// primaries and the D65 white (0.95047, 1.0, 1.08883), CIE 1976 L*a*b* with
// epsilon = 216/24389 and kappa = 24389/27, then palette's Lab clamp
// (L in [0,100], a and b in [-128,127]).
// ---------------------------------------------------------------------------
const double kWhite[3] = {0.95047, 1.0, 1.08883};
const double kEps = 216.0 / 24389.0;
const double kKappa = 24389.0 / 27.0;

struct Mat3 { double m[3][3]; };

Mat3 srgb_to_xyz_f64() {
  // Primaries' chromaticities (x, y) for R, G, B.
  const double xy[3][2] = {{0.64, 0.33}, {0.30, 0.60}, {0.15, 0.06}};
  double P[3][3];
  for (int c = 0; c < 3; ++c) {
    double x = xy[c][0], y = xy[c][1];
    P[0][c] = x / y;
    P[1][c] = 1.0;
    P[2][c] = (1.0 - x - y) / y;
  }
  // S = P^-1 * W
  double det = P[0][0] * (P[1][1] * P[2][2] - P[1][2] * P[2][1]) -
               P[0][1] * (P[1][0] * P[2][2] - P[1][2] * P[2][0]) +
               P[0][2] * (P[1][0] * P[2][1] - P[1][1] * P[2][0]);
  double inv[3][3];
  inv[0][0] = (P[1][1] * P[2][2] - P[1][2] * P[2][1]) / det;
  inv[0][1] = (P[0][2] * P[2][1] - P[0][1] * P[2][2]) / det;
  inv[0][2] = (P[0][1] * P[1][2] - P[0][2] * P[1][1]) / det;
  inv[1][0] = (P[1][2] * P[2][0] - P[1][0] * P[2][2]) / det;
  inv[1][1] = (P[0][0] * P[2][2] - P[0][2] * P[2][0]) / det;
  inv[1][2] = (P[0][2] * P[1][0] - P[0][0] * P[1][2]) / det;
  inv[2][0] = (P[1][0] * P[2][1] - P[1][1] * P[2][0]) / det;
  inv[2][1] = (P[0][1] * P[2][0] - P[0][0] * P[2][1]) / det;
  inv[2][2] = (P[0][0] * P[1][1] - P[0][1] * P[1][0]) / det;
  double S[3];
  for (int i = 0; i < 3; ++i)
    S[i] = inv[i][0] * kWhite[0] + inv[i][1] * kWhite[1] + inv[i][2] * kWhite[2];
  Mat3 M;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) M.m[r][c] = P[r][c] * S[c];
  return M;
}

double srgb_decode_f64(double c) {
  return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4);
}

double lab_f_f64(double t) { return t > kEps ? std::cbrt(t) : (kKappa * t + 16.0) / 116.0; }

struct SpecConsts {
  float lut[256];    // sRGB8 -> linear, FP64 then rounded
  float ms[3][3];    // RGB->XYZ rows divided by the white point, rounded
  float eps, k1, k2;
  SpecConsts() {
    for (int v = 0; v < 256; ++v) lut[v] = (float)srgb_decode_f64(v / 255.0);
    Mat3 M = srgb_to_xyz_f64();
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) ms[r][c] = (float)(M.m[r][c] / kWhite[r]);
    eps = (float)kEps;
    k1 = (float)(kKappa / 116.0);
    k2 = (float)(16.0 / 116.0);
  }
};
const SpecConsts& spec() {
  static SpecConsts s;
  return s;
}

// Cube root on (216/24389, ~1.1], the build's own definition (identical op
// sequence in the CUDA library): bit-level initial guess for t^(-1/3), two
// Newton steps r += r/3 * (1 - t r^3), y = t r^2, one Newton polish of y.
// Max error 0.77 ulp against FP64 cbrt on that interval.
float cbrt_spec(float t) {
  float r = u2f(0x54A2FA8Cu - f2u(t) / 3u);
  for (int k = 0; k < 2; ++k) {
    float r2 = r * r;
    float r3 = r2 * r;
    float e = std::fmaf(-t, r3, 1.0f);
    r = std::fmaf(r * (1.0f / 3.0f), e, r);
  }
  float rr = r * r;
  float y = t * rr;
  float y2 = y * y;
  float res = std::fmaf(-y2, y, t);
  return std::fmaf(res, rr * (1.0f / 3.0f), y);
}

inline float lab_f_spec(float t) {
  const SpecConsts& S = spec();
  return t > S.eps ? cbrt_spec(t) : std::fmaf(S.k1, t, S.k2);
}

inline void lab_pixel_spec(int r, int g, int b, float out[3]) {
  const SpecConsts& S = spec();
  float R = S.lut[r], G = S.lut[g], B = S.lut[b];
  float t[3];
  for (int i = 0; i < 3; ++i)
    t[i] = std::fmaf(S.ms[i][2], B, std::fmaf(S.ms[i][1], G, S.ms[i][0] * R));
  float fx = lab_f_spec(t[0]), fy = lab_f_spec(t[1]), fz = lab_f_spec(t[2]);
  out[0] = rclamp(std::fmaf(116.0f, fy, -16.0f), 0.0f, 100.0f);
  out[1] = rclamp(500.0f * (fx - fy), -128.0f, 127.0f);
  out[2] = rclamp(200.0f * (fy - fz), -128.0f, 127.0f);
}

// Fixed-point summation: each pixel's L, a, b is scaled by 2^20 and rounded
// to the nearest integer (ties to even), summed exactly in int64.  The sum is
// therefore independent of order, which is what lets many GPU threads reduce
// a cell and still agree bit for bit with this sequential loop.
const float kQ = 1048576.0f;          // 2^20
const float kInvQ = 9.5367431640625e-07f;  // 2^-20

inline int64_t quantize(float v) { return (int64_t)std::llrintf(v * kQ); }

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
// ---------------------------------------------------------------------------
void philox4x32_10(const uint32_t in[4], const uint32_t k_in[2], uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = k_in[0], k1 = k_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// exp(x) in f32, the build's own definition (identical op sequence in the
// CUDA library): Cody-Waite reduction x = k ln2 + r with ln2 split into a
// 24-bit head and a tail, Taylor polynomial of degree 7 on |r| <= ln2/2 in
// Horner form with fused multiply-adds, scaling by 2^k.  NaN passes through,
// x > 88.7 gives +inf, x < -87 gives 0.
float exp_spec(float x) {
  if (!(x == x)) return x;
  if (x > 88.7f) return INFINITY;
  if (x < -87.0f) return 0.0f;
  float k = std::rintf(x * 1.44269504088896341f);
  float r = std::fmaf(-k, 0.693145751953125f, x);
  r = std::fmaf(-k, 1.428606820309417232e-6f, r);
  float p = 1.0f / 5040.0f;
  p = std::fmaf(p, r, 1.0f / 720.0f);
  p = std::fmaf(p, r, 1.0f / 120.0f);
  p = std::fmaf(p, r, 1.0f / 24.0f);
  p = std::fmaf(p, r, 1.0f / 6.0f);
  p = std::fmaf(p, r, 0.5f);
  p = std::fmaf(p, r, 1.0f);
  p = std::fmaf(p, r, 1.0f);
  int ki = (int)k;
  if (ki > 127) return (p * 2.0f) * u2f((uint32_t)(127 + 127) << 23);
  return p * u2f((uint32_t)(ki + 127) << 23);
}

inline uint32_t mulhi_range(uint32_t r, uint32_t n) { return (uint32_t)(((uint64_t)r * n) >> 32); }

// ---------------------------------------------------------------------------
// Similarity: similarity.rs:141-146 calculate_lab_distance, and the lookup of
// similarity.rs:85-103 (same tile -> Some(0.0)); adjacency weight 1/(sim+1)
// (adjacency.rs:83, 110, 121, 168-207).
// ---------------------------------------------------------------------------
inline float lab_dist(const float* a, const float* b) {
  float dl = a[0] - b[0];
  float da = a[1] - b[1];
  float db = a[2] - b[2];
  return std::sqrt(dl * dl + da * da + db * db);
}
inline float sim_of(const float* pal, int i, int j) {
  if (i == j) return 0.0f;
  int lo = std::min(i, j), hi = std::max(i, j);
  return lab_dist(pal + 3 * lo, pal + 3 * hi);
}
inline float wgt(const float* pal, int i, int j) { return 1.0f / (sim_of(pal, i, j) + 1.0f); }

// adjacency.rs:17-45 get_adjacent_positions: up, down, left, right.
int adjacent(int x, int y, int gw, int gh, int nx[4], int ny[4]) {
  int n = 0;
  if (y > 0) { nx[n] = x; ny[n] = y - 1; ++n; }
  if (y < gh - 1) { nx[n] = x; ny[n] = y + 1; ++n; }
  if (x > 0) { nx[n] = x - 1; ny[n] = y; ++n; }
  if (x < gw - 1) { nx[n] = x + 1; ny[n] = y; ++n; }
  return n;
}

// kiddo SquaredEuclidean::dist(query, point): sum over dims of (q-p)^2, folded
// from zero in dimension order.
inline float sq_dist(const float* q, const float* p) {
  float d0 = q[0] - p[0], d1 = q[1] - p[1], d2 = q[2] - p[2];
  return (d0 * d0 + d1 * d1) + d2 * d2;
}

}  // namespace

extern "C" {

void orc_srgb_lut(float out[256]) { std::memcpy(out, spec().lut, sizeof(float) * 256); }

void orc_lab_pixel_f64(int r, int g, int b, double out[3]) {
  static const Mat3 M = srgb_to_xyz_f64();
  double lin[3] = {srgb_decode_f64(r / 255.0), srgb_decode_f64(g / 255.0), srgb_decode_f64(b / 255.0)};
  double f[3];
  for (int i = 0; i < 3; ++i) {
    double t = (M.m[i][0] * lin[0] + M.m[i][1] * lin[1] + M.m[i][2] * lin[2]) / kWhite[i];
    f[i] = lab_f_f64(t);
  }
  out[0] = std::min(std::max(116.0 * f[1] - 16.0, 0.0), 100.0);
  out[1] = std::min(std::max(500.0 * (f[0] - f[1]), -128.0), 127.0);
  out[2] = std::min(std::max(200.0 * (f[1] - f[2]), -128.0), 127.0);
}

// lib.rs:94-119 in FP64 (the accuracy reference for the 1e-4 gate).
void orc_lab_mean_f64(const uint8_t* rgb, int w, int h, long stride, double out[3]) {
  double s[3] = {0, 0, 0};
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = rgb + (long)y * stride + 3L * x;
      double l[3];
      orc_lab_pixel_f64(p[0], p[1], p[2], l);
      s[0] += l[0]; s[1] += l[1]; s[2] += l[2];
    }
  double n = (double)w * (double)h;
  out[0] = s[0] / n; out[1] = s[1] / n; out[2] = s[2] / n;
}

// lib.rs:94-119 as the reference writes it: per-pixel palette conversion in
// f32 (powf transfer function, cbrtf), then a sequential f32 fold and one
// division by the pixel count.  Used only to report how far the reference's
// own f32 fold drifts from FP64.
void orc_lab_mean_reffold(const uint8_t* rgb, int w, int h, long stride, float out[3]) {
  Mat3 M = srgb_to_xyz_f64();
  float m[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m[r][c] = (float)M.m[r][c];
  const float wp[3] = {0.95047f, 1.0f, 1.08883f};
  const float eps = 216.0f / 24389.0f, kappa = 24389.0f / 27.0f;
  float sl = 0, sa = 0, sb = 0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = rgb + (long)y * stride + 3L * x;
      float lin[3];
      for (int c = 0; c < 3; ++c) {
        float v = (float)p[c] / 255.0f;
        lin[c] = v <= 0.04045f ? v / 12.92f : std::pow((v + 0.055f) / 1.055f, 2.4f);
      }
      float f[3];
      for (int i = 0; i < 3; ++i) {
        float t = (m[i][0] * lin[0] + m[i][1] * lin[1] + m[i][2] * lin[2]) / wp[i];
        f[i] = t > eps ? std::cbrt(t) : (kappa * t + 16.0f) / 116.0f;
      }
      sl += rclamp(116.0f * f[1] - 16.0f, 0.0f, 100.0f);
      sa += rclamp(500.0f * (f[0] - f[1]), -128.0f, 127.0f);
      sb += rclamp(200.0f * (f[1] - f[2]), -128.0f, 127.0f);
    }
  float n = (float)(w * h);
  out[0] = sl / n; out[1] = sa / n; out[2] = sb / n;
}

void orc_lab_pixel_spec(int r, int g, int b, float out[3]) { lab_pixel_spec(r, g, b, out); }

// The constants of the defined conversion: transfer table, white-normalised
// RGB -> XYZ matrix (row major), and eps, kappa / 116, 16 / 116.
void orc_lab_consts(float lut[256], float ms[9], float k[3]) {
  const SpecConsts& S = spec();
  std::memcpy(lut, S.lut, sizeof(float) * 256);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) ms[3 * r + c] = S.ms[r][c];
  k[0] = S.eps;
  k[1] = S.k1;
  k[2] = S.k2;
}

// The fixed-point summands of n pixels (L, a, b of each, scaled by 2^20 and
// rounded as orc_lab_mean_spec sums them).
void orc_lab_pixels_q(const uint8_t* rgb, long n, int32_t* q) {
  for (long i = 0; i < n; ++i) {
    float l[3];
    lab_pixel_spec(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], l);
    for (int c = 0; c < 3; ++c) q[3 * i + c] = (int32_t)quantize(l[c]);
  }
}

// lib.rs:94-119 in the build's defined arithmetic (FP32 per pixel, exact
// fixed-point sum, one FP32 division).  The CUDA reduction must equal this.
void orc_lab_mean_spec(const uint8_t* rgb, int w, int h, long stride, float out[3]) {
  int64_t s[3] = {0, 0, 0};
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = rgb + (long)y * stride + 3L * x;
      float l[3];
      lab_pixel_spec(p[0], p[1], p[2], l);
      s[0] += quantize(l[0]); s[1] += quantize(l[1]); s[2] += quantize(l[2]);
    }
  float n = (float)((int64_t)w * h);
  for (int c = 0; c < 3; ++c) out[c] = ((float)s[c] / n) * kInvQ;
}

// main.rs:710-738 resize_image: fast_image_resize's default Lanczos3
// convolution, restated from the published resampler it follows (Pillow's
// ImagingResample): per output coordinate of a dimension in -> out, taps at
// pixel centres over a support of 3 * max(in / out, 1), lanczos3 weights
// normalised to sum 1 and rounded half away from zero to 22-bit fixed point;
// the horizontal pass into an 8-bit image first, then the vertical pass; a
// dimension that keeps its size is copied.
namespace {
double resize_sinc(double x) {
  if (x == 0.0) return 1.0;
  x = x * M_PI;
  return std::sin(x) / x;
}
double resize_lanczos3(double x) {
  if (x < -3.0 || x >= 3.0) return 0.0;
  return resize_sinc(x) * resize_sinc(x / 3.0);
}
struct Taps {
  std::vector<int> first, count;
  std::vector<std::vector<int32_t>> k;
};
Taps resize_taps(int in, int out) {
  Taps T;
  const double scale = (double)in / (double)out;
  const double fs = std::max(scale, 1.0);
  const double support = 3.0 * fs;
  for (int o = 0; o < out; ++o) {
    const double centre = (o + 0.5) * scale;
    const int lo = std::max(0, (int)(centre - support + 0.5));
    const int hi = std::min(in, (int)(centre + support + 0.5));
    std::vector<double> w;
    double sum = 0.0;
    for (int i = lo; i < hi; ++i) {
      w.push_back(resize_lanczos3((i - centre + 0.5) / fs));
      sum += w.back();
    }
    std::vector<int32_t> q;
    for (double v : w) {
      if (sum != 0.0) v /= sum;
      q.push_back((int32_t)(v < 0.0 ? v * 4194304.0 - 0.5 : v * 4194304.0 + 0.5));
    }
    T.first.push_back(lo);
    T.count.push_back(hi - lo);
    T.k.push_back(q);
  }
  return T;
}
uint8_t resize_clip(int32_t acc) {
  const int32_t v = acc >> 22;
  return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
}
}  // namespace

void orc_resize_lanczos3(const uint8_t* rgb, int w, int h, long stride, int dw, int dh, uint8_t* out) {
  // horizontal: h rows of dw pixels
  std::vector<uint8_t> mid((size_t)h * dw * 3);
  if (dw == w) {
    for (int y = 0; y < h; ++y) std::memcpy(&mid[(size_t)y * dw * 3], rgb + (long)y * stride, (size_t)w * 3);
  } else {
    const Taps T = resize_taps(w, dw);
    for (int y = 0; y < h; ++y)
      for (int x = 0; x < dw; ++x)
        for (int c = 0; c < 3; ++c) {
          int32_t acc = 1 << 21;
          for (int t = 0; t < T.count[x]; ++t) acc += T.k[x][t] * rgb[(long)y * stride + 3L * (T.first[x] + t) + c];
          mid[((size_t)y * dw + x) * 3 + c] = resize_clip(acc);
        }
  }
  // vertical: dh rows
  if (dh == h) {
    std::memcpy(out, mid.data(), mid.size());
    return;
  }
  const Taps T = resize_taps(h, dh);
  for (int y = 0; y < dh; ++y)
    for (int x = 0; x < dw; ++x)
      for (int c = 0; c < 3; ++c) {
        int32_t acc = 1 << 21;
        for (int t = 0; t < T.count[y]; ++t) acc += T.k[y][t] * mid[((size_t)(T.first[y] + t) * dw + x) * 3 + c];
        out[((size_t)y * dw + x) * 3 + c] = resize_clip(acc);
      }
}

// main.rs:687-708 calculate_average_rgb: u64 sums, truncating division.
void orc_avg_rgb(const uint8_t* rgb, int w, int h, long stride, uint8_t out[3]) {
  uint64_t s[3] = {0, 0, 0};
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = rgb + (long)y * stride + 3L * x;
      s[0] += p[0]; s[1] += p[1]; s[2] += p[2];
    }
  uint64_t n = (uint64_t)w * (uint64_t)h;
  for (int c = 0; c < 3; ++c) out[c] = (uint8_t)(s[c] / n);
}

// main.rs:495-496, 529-541: cell geometry img/grid (integer division, the
// right and bottom remainder ignored), row-major cells.
int orc_cells(const uint8_t* img, int w, int h, long stride, int gw, int gh, float* lab_out,
              uint8_t* avg_rgb_out) {
  if (gw <= 0 || gh <= 0) return -1;
  int cw = w / gw, ch = h / gh;
  if (cw <= 0 || ch <= 0) return -1;
  for (int y = 0; y < gh; ++y)
    for (int x = 0; x < gw; ++x) {
      const uint8_t* base = img + (long)y * ch * stride + 3L * x * cw;
      int c = y * gw + x;
      if (lab_out) orc_lab_mean_spec(base, cw, ch, stride, lab_out + 3 * c);
      if (avg_rgb_out) orc_avg_rgb(base, cw, ch, stride, avg_rgb_out + 3 * c);
    }
  return 0;
}

// lib.rs:121-123.
int orc_is_aspect_ratio_match(float img_aspect, float target_aspect, float tol) {
  return std::fabs(img_aspect - target_aspect) <= tol;
}

// main.rs:166-261 load_tiles: aspect filter in input order; if nothing
// matches, the first min(n, 2*max_materials) unfiltered; then truncate to
// max_materials.
int orc_select_palette(const int* widths, const int* heights, int n, float target_aspect, float tol,
                       int max_materials, int* selected) {
  int cnt = 0;
  for (int i = 0; i < n; ++i) {
    float a = (float)widths[i] / (float)heights[i];
    if (orc_is_aspect_ratio_match(a, target_aspect, tol)) selected[cnt++] = i;
  }
  if (cnt == 0) {
    long lim = std::min((long)n, 2L * (long)max_materials);
    for (long i = 0; i < lim; ++i) selected[cnt++] = (int)i;
  }
  if (cnt > max_materials) cnt = max_materials;
  return cnt;
}

float orc_lab_distance(const float a[3], const float b[3]) { return lab_dist(a, b); }

// similarity.rs:69-82: strict upper triangle, row order.
void orc_similarity_tri(const float* lab, int p, float* out) {
  long pos = 0;
  for (int i = 0; i < p; ++i)
    for (int j = i + 1; j < p; ++j) out[pos++] = lab_dist(lab + 3 * i, lab + 3 * j);
}

// Full symmetric P x P view of the same values (similarity.rs:85-103).
void orc_similarity_full(const float* lab, int p, float* out) {
  for (int i = 0; i < p; ++i)
    for (int j = 0; j < p; ++j) out[(long)i * p + j] = sim_of(lab, i, j);
}

// kiddo nearest_n::<SquaredEuclidean> (main.rs:348-352): the k nearest by
// squared distance, ascending; ties broken to the lowest palette index.
void orc_nearest_n(const float* pal, int p, const float q[3], int k, uint32_t* idx, float* dist) {
  std::vector<uint64_t> keys(p);
  for (int j = 0; j < p; ++j) keys[j] = ((uint64_t)f2u(sq_dist(q, pal + 3 * j)) << 32) | (uint32_t)j;
  k = std::min(k, p);
  std::partial_sort(keys.begin(), keys.begin() + k, keys.end());
  for (int i = 0; i < k; ++i) {
    idx[i] = (uint32_t)keys[i];
    dist[i] = u2f((uint32_t)(keys[i] >> 32));
  }
}

// adjacency.rs:63-88 calculate_penalty (weighted).
float orc_penalty(const float* pal, int p, int cand, int x, int y, const int32_t* grid, int gw, int gh,
                  float weight) {
  (void)p;
  int nx[4], ny[4];
  int n = adjacent(x, y, gw, gh, nx, ny);
  float pen = 0.0f;
  for (int i = 0; i < n; ++i) {
    int nb = grid[ny[i] * gw + nx[i]];
    if (nb >= 0) pen += wgt(pal, cand, nb);
  }
  return pen * weight;
}

// adjacency.rs:91-130 calculate_total_cost (unweighted, right and down pairs).
float orc_total_cost(const float* pal, int p, const int32_t* grid, int gw, int gh) {
  (void)p;
  if (gh == 0) return 0.0f;
  float total = 0.0f;
  for (int y = 0; y < gh; ++y)
    for (int x = 0; x < gw; ++x) {
      int cur = grid[y * gw + x];
      if (cur < 0) continue;
      if (x < gw - 1) {
        int r = grid[y * gw + x + 1];
        if (r >= 0) total += wgt(pal, cur, r);
      }
      if (y < gh - 1) {
        int d = grid[(y + 1) * gw + x];
        if (d >= 0) total += wgt(pal, cur, d);
      }
    }
  return total;
}

// adjacency.rs:133-214 calculate_swap_delta (unweighted).
float orc_swap_delta(const float* pal, int p, const int32_t* grid, int gw, int gh, int x1, int y1, int x2,
                     int y2) {
  (void)p;
  if (gh == 0) return 0.0f;
  int p1 = grid[y1 * gw + x1], p2 = grid[y2 * gw + x2];
  if (p1 < 0 || p2 < 0) return 0.0f;
  if (p1 == p2) return 0.0f;
  float old_cost = 0.0f, new_cost = 0.0f;
  int nx[4], ny[4];
  int n1 = adjacent(x1, y1, gw, gh, nx, ny);
  bool adj12 = false;
  for (int i = 0; i < n1; ++i) {
    if (nx[i] == x2 && ny[i] == y2) { adj12 = true; continue; }
    int a = grid[ny[i] * gw + nx[i]];
    if (a >= 0) {
      old_cost += wgt(pal, p1, a);
      new_cost += wgt(pal, p2, a);
    }
  }
  int n2 = adjacent(x2, y2, gw, gh, nx, ny);
  for (int i = 0; i < n2; ++i) {
    if (nx[i] == x1 && ny[i] == y1) continue;
    int a = grid[ny[i] * gw + nx[i]];
    if (a >= 0) {
      old_cost += wgt(pal, p2, a);
      new_cost += wgt(pal, p1, a);
    }
  }
  if (adj12) {
    float c = wgt(pal, p1, p2);
    old_cost += c;
    new_cost += c;
  }
  return new_cost - old_cost;
}

// main.rs:335-475: find_and_use_best_tile_with_position + fallback, row-major
// over the grid (main.rs:529-545).  Candidates are the min(P,100) nearest by
// squared Lab distance; score = squared distance + weighted penalty; strict <
// keeps the first of equal scores.  Fallback: global usage reset, first
// candidate that passes the same-neighbour ban, else the nearest one.
//
// gui: the GUI generator's selection instead (gui/app_full.rs:1396-1470
// find_best_tile_primary, with the same two fallbacks at :1475-1568): score =
// sqrt of the squared distance (the candidate's distance recomputed as
// (dl^2 + da^2) + db^2, the same bits) + the penalty, computed for every weight;
// best starts at +inf, so a candidate only wins with a score below it.
static int place_greedy(const float* pal, int p, const float* cell_lab, int gw, int gh, int max_usage,
                        float weight, bool gui, int32_t* grid, int* n_resets) {
  const int n = gw * gh;
  for (int i = 0; i < n; ++i) grid[i] = -1;
  int resets = 0;
  if (p <= 0) {
    if (n_resets) *n_resets = 0;
    return 0;
  }
  std::vector<uint32_t> usage(p, 0);
  const int k = std::min(p, 100);
  std::vector<uint32_t> cidx(k);
  std::vector<float> cdist(k);
  auto can_place = [&](int t, int x, int y) {  // main.rs:309-333
    const int dx[4] = {-1, 1, 0, 0}, dy[4] = {0, 0, -1, 1};
    for (int i = 0; i < 4; ++i) {
      int nx = x + dx[i], ny = y + dy[i];
      if (nx < 0 || ny < 0 || nx >= gw || ny >= gh) continue;
      if (grid[ny * gw + nx] == t) return false;
    }
    return true;
  };
  for (int y = 0; y < gh; ++y)
    for (int x = 0; x < gw; ++x) {
      orc_nearest_n(pal, p, cell_lab + 3 * (y * gw + x), k, cidx.data(), cdist.data());
      int best = -1;
      float best_score = gui ? INFINITY : 0.0f;
      for (int j = 0; j < k; ++j) {
        int t = (int)cidx[j];
        if (!(usage[t] < (uint32_t)max_usage)) continue;
        if (!can_place(t, x, y)) continue;
        float pen = gui || weight > 0.0f ? orc_penalty(pal, p, t, x, y, grid, gw, gh, weight) : 0.0f;
        float score = (gui ? std::sqrt(cdist[j]) : cdist[j]) + pen;
        if ((!gui && best < 0) || score < best_score) { best = t; best_score = score; }
      }
      if (best >= 0) {
        usage[best] += 1;
        grid[y * gw + x] = best;
        continue;
      }
      ++resets;
      std::fill(usage.begin(), usage.end(), 0u);
      int chosen = -1;
      for (int j = 0; j < k; ++j)
        if (can_place((int)cidx[j], x, y)) { chosen = (int)cidx[j]; break; }
      if (chosen < 0) chosen = (int)cidx[0];  // nearest_one: lowest-index nearest
      usage[chosen] += 1;
      grid[y * gw + x] = chosen;
    }
  if (n_resets) *n_resets = resets;
  return 0;
}

int orc_place_greedy(const float* pal, int p, const float* cell_lab, int gw, int gh, int max_usage,
                     float weight, int32_t* grid, int* n_resets) {
  return place_greedy(pal, p, cell_lab, gw, gh, max_usage, weight, false, grid, n_resets);
}

int orc_place_greedy_gui(const float* pal, int p, const float* cell_lab, int gw, int gh, int max_usage,
                         float weight, int32_t* grid, int* n_resets) {
  return place_greedy(pal, p, cell_lab, gw, gh, max_usage, weight, true, grid, n_resets);
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox4x32_10(ctr, key, out); }

float orc_exp(float x) { return exp_spec(x); }

// optimizer.rs:41-129 optimize (greedy_only: optimizer.rs:132-198).  The
// reference's unseeded thread_rng is replaced by a counter-based stream: at
// iteration t of chain c, Philox4x32-10 with key (seed lo, seed hi) and counter
// (t, c, stream, 2*(t>>32)) gives x1, y1, x2, y2 by multiply-high range
// reduction, and counter (t, c, stream, 2*(t>>32)+1) gives the acceptance
// uniform (word0 >> 8) * 2^-24 (rand's f32 construction).  An iteration that
// draws pos1 == pos2 or an empty cell is skipped without cooling, as in the
// reference.
// libm_exp: the acceptance test with the C library's expf (what Rust's
// f32::exp calls, optimizer.rs:81) instead of the defined exp_spec.
void orc_anneal_ex(const float* pal, int p, int32_t* grid, int gw, int gh, long iters, float t0, float decay,
                   uint64_t seed, uint32_t stream, uint32_t chain, int greedy_only, int libm_exp, float res[3],
                   int64_t counts[3]) {
  res[0] = res[1] = res[2] = 0.0f;
  counts[0] = counts[1] = counts[2] = 0;
  if (gh == 0 || gw == 0) return;
  float current = orc_total_cost(pal, p, grid, gw, gh);
  float initial = current, best = current;
  int64_t improved = 0, accepted = 0, cooled = 0;
  float temp = t0;
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  for (long it = 0; it < iters; ++it) {
    uint32_t hi = (uint32_t)((uint64_t)it >> 32);
    uint32_t ctr[4] = {(uint32_t)it, chain, stream, 2u * hi};
    uint32_t r[4];
    philox4x32_10(ctr, key, r);
    int x1 = (int)mulhi_range(r[0], (uint32_t)gw), y1 = (int)mulhi_range(r[1], (uint32_t)gh);
    int x2 = (int)mulhi_range(r[2], (uint32_t)gw), y2 = (int)mulhi_range(r[3], (uint32_t)gh);
    if (x1 == x2 && y1 == y2) continue;
    if (grid[y1 * gw + x1] < 0 || grid[y2 * gw + x2] < 0) continue;
    float delta = orc_swap_delta(pal, p, grid, gw, gh, x1, y1, x2, y2);
    bool accept;
    if (greedy_only) {
      accept = delta < 0.0f;
    } else if (delta < 0.0f) {
      accept = true;
    } else {
      uint32_t ctr2[4] = {(uint32_t)it, chain, stream, 2u * hi + 1u};
      uint32_t u[4];
      philox4x32_10(ctr2, key, u);
      float uf = (float)(u[0] >> 8) * 5.9604644775390625e-08f;
      const float arg = -delta / temp;
      accept = uf < (libm_exp ? std::exp(arg) : exp_spec(arg));
    }
    if (accept) {
      std::swap(grid[y1 * gw + x1], grid[y2 * gw + x2]);
      current += delta;
      ++accepted;
      if (current < best) {
        best = current;
        ++improved;
      }
    }
    if (!greedy_only) temp *= decay;
    ++cooled;
  }
  res[0] = initial;
  res[1] = current;
  res[2] = greedy_only ? current : best;
  counts[0] = accepted;
  counts[1] = greedy_only ? accepted : improved;
  counts[2] = cooled;
}

void orc_anneal(const float* pal, int p, int32_t* grid, int gw, int gh, long iters, float t0, float decay,
                uint64_t seed, uint32_t stream, uint32_t chain, int greedy_only, float res[3],
                int64_t counts[3]) {
  orc_anneal_ex(pal, p, grid, gw, gh, iters, t0, decay, seed, stream, chain, greedy_only, 0, res, counts);
}

// palette 0.7.6 Hsv::from_color(Rgb) -- hexcone, hue in raw degrees (may be
// negative), then palette's clamp of saturation and value to [0,1].
void orc_rgb_to_hsv(float r, float g, float b, float out[3]) {
  float red = std::max(r, 0.0f), green = std::max(g, 0.0f), blue = std::max(b, 0.0f);
  float mx, mn, sep, coeff;
  if (red > green) { mx = red; mn = green; sep = green - blue; coeff = 0.0f; }
  else { mx = green; mn = red; sep = blue - red; coeff = 2.0f; }
  if (blue > mx) { mx = blue; sep = red - green; coeff = 4.0f; }
  else if (blue < mn) { mn = blue; }
  float h = 0.0f, s = 0.0f;
  if (mx != mn) {
    float d = mx - mn;
    h = (sep / d + coeff) * 60.0f;
    s = d / mx;
  }
  out[0] = h;
  out[1] = rclamp(s, 0.0f, 1.0f);
  out[2] = rclamp(mx, 0.0f, 1.0f);
}

// palette 0.7.6 Rgb::from_color(Hsv): hue normalised to [0,360), six zones,
// then palette's clamp of each channel to [0,1].
void orc_hsv_to_rgb(float hue, float s, float v, float out[3]) {
  float pos = hue - std::floor(hue / 360.0f) * 360.0f;
  float c = v * s;
  float h = pos / 60.0f;
  float hm2 = h - std::floor(h * 0.5f) * 2.0f;
  float x = c * (1.0f - std::fabs(hm2 - 1.0f));
  float m = v - c;
  bool z0 = h >= 0.0f && h < 1.0f, z1 = h >= 1.0f && h < 2.0f, z2 = h >= 2.0f && h < 3.0f;
  bool z3 = h >= 3.0f && h < 4.0f, z4 = h >= 4.0f && h < 5.0f;
  float red = (z1 || z4) ? x : ((z2 || z3) ? 0.0f : c);
  float green = (z0 || z3) ? x : ((z1 || z2) ? c : 0.0f);
  float blue = (z0 || z1) ? 0.0f : ((z3 || z4) ? c : x);
  out[0] = rclamp(red + m, 0.0f, 1.0f);
  out[1] = rclamp(green + m, 0.0f, 1.0f);
  out[2] = rclamp(blue + m, 0.0f, 1.0f);
}

// color_adjustment.rs:30-37 ColorAdjustment::new clamps.
void orc_adjustment_new(float br, float co, float hue, float sat, float out[4]) {
  out[0] = rclamp(br, -1.0f, 1.0f);
  out[1] = rclamp(co, 0.0f, 2.0f);
  out[2] = rclamp(hue, -180.0f, 180.0f);
  out[3] = rclamp(sat, 0.0f, 2.0f);
}

// color_adjustment.rs:99-154 calculate_optimal_adjustment.
void orc_optimal_adjustment(const uint8_t tile[3], const uint8_t target[3], float strength, float out[4]) {
  float tr = (float)tile[0] / 255.0f, tg = (float)tile[1] / 255.0f, tb = (float)tile[2] / 255.0f;
  float gr = (float)target[0] / 255.0f, gg = (float)target[1] / 255.0f, gb = (float)target[2] / 255.0f;
  float tile_luma = 0.299f * tr + 0.587f * tg + 0.114f * tb;
  float target_luma = 0.299f * gr + 0.587f * gg + 0.114f * gb;
  float brightness = (target_luma - tile_luma) * strength;
  float th[3], gh[3];
  orc_rgb_to_hsv(tr, tg, tb, th);
  orc_rgb_to_hsv(gr, gg, gb, gh);
  float hue = 0.0f;
  if (th[1] > 0.1f && gh[1] > 0.1f) {
    float diff = gh[0] - th[0];
    float wrapped = diff > 180.0f ? diff - 360.0f : (diff < -180.0f ? diff + 360.0f : diff);
    hue = wrapped * strength * 0.5f;
  }
  float sat = 1.0f;
  if (th[1] > 0.01f) {
    float ratio = gh[1] / th[1];
    sat = 1.0f + (ratio - 1.0f) * strength * 0.7f;
  }
  orc_adjustment_new(brightness, 1.0f, hue, sat, out);
}

// color_adjustment.rs:53-96 adjust_pixel / apply_brightness_contrast.
void orc_adjust_pixel(const float adj[4], const uint8_t in[3], uint8_t out[3]) {
  float c[3];
  for (int i = 0; i < 3; ++i) {
    float v = (float)in[i] / 255.0f;
    float con = rclamp((v - 0.5f) * adj[1] + 0.5f, 0.0f, 1.0f);
    c[i] = rclamp(con + adj[0], 0.0f, 1.0f);
  }
  float f[3] = {c[0], c[1], c[2]};
  if (adj[2] != 0.0f || adj[3] != 1.0f) {
    float hsv[3];
    orc_rgb_to_hsv(c[0], c[1], c[2], hsv);
    float hh = hsv[0] + adj[2];
    float rem = std::fmod(hh, 360.0f);
    if (rem < 0.0f) rem += 360.0f;  // f32::rem_euclid
    float ss = rclamp(hsv[1] * adj[3], 0.0f, 1.0f);
    orc_hsv_to_rgb(rem, ss, hsv[2], f);
  }
  for (int i = 0; i < 3; ++i) out[i] = as_u8(rclamp(f[i] * 255.0f, 0.0f, 255.0f));
}

// orc_adjust_pixel of n pixels.
void orc_adjust_pixels(const float adj[4], const uint8_t* in, long n, uint8_t* out) {
  for (long i = 0; i < n; ++i) orc_adjust_pixel(adj, in + 3 * i, out + 3 * i);
}

// main.rs:548-592 (first composite) and main.rs:627-664 (rebuild after the
// optimiser): per cell, the material's thumbnail, colour-adjusted when the
// strength is positive, written at (x*tw, y*th).  Cells without a tile stay 0.
int orc_composite(const int32_t* grid, int gw, int gh, const uint8_t* thumbs, int tw, int th,
                  const uint8_t* cell_avg_rgb, const uint8_t* thumb_avg_rgb, float strength, uint8_t* out) {
  const long ow = (long)gw * tw;
  std::memset(out, 0, (size_t)ow * gh * th * 3);
  for (int y = 0; y < gh; ++y)
    for (int x = 0; x < gw; ++x) {
      int m = grid[y * gw + x];
      if (m < 0) continue;
      const uint8_t* src = thumbs + (size_t)m * tw * th * 3;
      float adj[4] = {0.0f, 1.0f, 0.0f, 1.0f};
      bool do_adj = strength > 0.0f;
      if (do_adj) orc_optimal_adjustment(thumb_avg_rgb + 3 * m, cell_avg_rgb + 3 * (y * gw + x), strength, adj);
      for (int dy = 0; dy < th; ++dy)
        for (int dx = 0; dx < tw; ++dx) {
          const uint8_t* s = src + 3L * (dy * tw + dx);
          uint8_t* d = out + 3L * (((long)y * th + dy) * ow + (long)x * tw + dx);
          if (do_adj) orc_adjust_pixel(adj, s, d);
          else { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }
        }
    }
  return 0;
}

// main.rs:105-164 (MosaicGenerator::new) + main.rs:477-685 (generate_mosaic),
// minus file I/O and resizing: thumbnails at the output tile size are an input.
// Material Lab runs across threads (main.rs:193-208 uses Rayon); the greedy
// pass is sequential; the K annealing chains run across threads.
int orc_generate(const orc_job* J, orc_out* O) {
  if (J->gw <= 0 || J->gh <= 0) return -1;
  const int cw = J->tw_img / J->gw, ch = J->th_img / J->gh;
  if (cw <= 0 || ch <= 0) return -1;
  const int N = J->gw * J->gh;
  const float target_aspect = (float)J->tw_img / (float)J->th_img;
  std::vector<int> sel(std::max(J->n_mats, 1));
  int P = orc_select_palette(J->mat_w, J->mat_h, J->n_mats, target_aspect, J->aspect_tol,
                             J->max_materials, sel.data());
  // ref_arith: Lab as lib.rs:99-118 folds it (per-pixel FP32 conversion, a
  // sequential FP32 sum, one division) instead of the defined fixed-point mean
  auto lab_mean = [&](const uint8_t* img, int w, int h, long stride, float* out) {
    if (J->ref_arith) orc_lab_mean_reffold(img, w, h, stride, out);
    else orc_lab_mean_spec(img, w, h, stride, out);
  };
  std::vector<float> pal(3 * (size_t)std::max(P, 1));
  parallel_for(P, J->threads, [&](int i) {
    int m = sel[i];
    lab_mean(J->mats + J->mat_off[m], J->mat_w[m], J->mat_h[m], 3L * J->mat_w[m], pal.data() + 3 * i);
  });
  std::vector<float> cell_lab(3 * (size_t)N);
  std::vector<uint8_t> cell_rgb(3 * (size_t)N);
  // Cells are sequential, as in the reference's row-major loop (main.rs:529-541).
  parallel_for(J->gh, 1, [&](int y) {
    for (int x = 0; x < J->gw; ++x) {
      const uint8_t* base = J->target + (long)y * ch * J->tstride + 3L * x * cw;
      int c = y * J->gw + x;
      lab_mean(base, cw, ch, J->tstride, cell_lab.data() + 3 * c);
      orc_avg_rgb(base, cw, ch, J->tstride, cell_rgb.data() + 3 * c);
    }
  });
  std::vector<int32_t> grid(N);
  int resets = 0;
  place_greedy(pal.data(), P, cell_lab.data(), J->gw, J->gh, J->max_usage, J->weight, J->gui_scoring != 0, grid.data(),
               &resets);
  if (O->greedy_grid) std::memcpy(O->greedy_grid, grid.data(), sizeof(int32_t) * N);

  std::vector<int32_t> final_grid = grid;
  int best_chain = -1;
  float ic = 0, fc = 0, bc = 0;
  if (J->enable_opt && J->weight > 0.0f && J->chains > 0) {
    const int K = J->chains;
    std::vector<std::vector<int32_t>> g(K, grid);
    std::vector<float> res(3 * K);
    parallel_for(K, J->threads, [&](int c) {
      int64_t cnt[3];
      orc_anneal_ex(pal.data(), P, g[c].data(), J->gw, J->gh, J->iters, J->t0, J->decay, J->seed, J->stream,
                    (uint32_t)c, 0, J->ref_arith, res.data() + 3 * c, cnt);
    });
    best_chain = 0;
    for (int c = 1; c < K; ++c)
      if (res[3 * c + 1] < res[3 * best_chain + 1]) best_chain = c;
    final_grid = g[best_chain];
    ic = res[3 * best_chain]; fc = res[3 * best_chain + 1]; bc = res[3 * best_chain + 2];
    if (O->chain_res) std::memcpy(O->chain_res, res.data(), sizeof(float) * 3 * K);
  }
  // thumbnails of the selected palette, and their mean RGB (main.rs:557)
  const size_t tb = (size_t)J->thumb_w * J->thumb_h * 3;
  std::vector<uint8_t> pthumb(tb * std::max(P, 1));
  std::vector<uint8_t> pavg(3 * (size_t)std::max(P, 1));
  for (int i = 0; i < P; ++i) {
    std::memcpy(pthumb.data() + tb * i, J->thumbs + tb * sel[i], tb);
    orc_avg_rgb(pthumb.data() + tb * i, J->thumb_w, J->thumb_h, 3L * J->thumb_w, pavg.data() + 3 * i);
  }
  float strength = rclamp(J->color_strength, 0.0f, 1.0f);  // main.rs:162
  if (O->image)
    orc_composite(final_grid.data(), J->gw, J->gh, pthumb.data(), J->thumb_w, J->thumb_h, cell_rgb.data(),
                  pavg.data(), strength, O->image);
  for (int i = 0; i < N; ++i) O->grid[i] = final_grid[i] < 0 ? -1 : sel[final_grid[i]];
  if (O->pal_lab) std::memcpy(O->pal_lab, pal.data(), sizeof(float) * 3 * P);
  if (O->cell_lab) std::memcpy(O->cell_lab, cell_lab.data(), sizeof(float) * 3 * N);
  O->p = P;
  O->n_resets = resets;
  O->best_chain = best_chain;
  O->initial_cost = ic; O->final_cost = fc; O->best_cost = bc;
  return 0;
}

}  // extern "C"
