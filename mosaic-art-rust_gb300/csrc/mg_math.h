// mg_math.h -- the arithmetic of the tile matching-and-placement path, written
// once for host and device.  Every rounding step is explicit (MG_MUL, MG_ADD,
// MG_FMA, ...), so a host build with -ffp-contract=off and a device build give
// the same bits.  Nothing here calls a CUDA or libm transcendental: the cube
// root and exp are this library's own (methods named at each function).
#pragma once
#include <stdint.h>

#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define MG_HD __host__ __device__ __forceinline__
#define MG_UNROLL _Pragma("unroll")
#else
#define MG_HD inline
#define MG_UNROLL
#endif

#if defined(__CUDA_ARCH__)
#define MG_MUL(a, b) __fmul_rn((a), (b))
#define MG_ADD(a, b) __fadd_rn((a), (b))
#define MG_SUB(a, b) __fsub_rn((a), (b))
#define MG_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define MG_DIV(a, b) __fdiv_rn((a), (b))
#define MG_SQRT(a) __fsqrt_rn((a))
#define MG_FLOOR(a) floorf((a))
#define MG_RINT(a) rintf((a))
#define MG_FMOD(a, b) fmodf((a), (b))
#else
#define MG_MUL(a, b) ((a) * (b))
#define MG_ADD(a, b) ((a) + (b))
#define MG_SUB(a, b) ((a) - (b))
#define MG_FMA(a, b, c) std::fmaf((a), (b), (c))
#define MG_DIV(a, b) ((a) / (b))
#define MG_SQRT(a) std::sqrt((a))
#define MG_FLOOR(a) std::floor((a))
#define MG_RINT(a) std::rintf((a))
#define MG_FMOD(a, b) std::fmod((a), (b))
#endif

namespace mg {

MG_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
MG_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}

// Rust f32::clamp semantics (NaN passes through).
MG_HD float rclamp(float v, float lo, float hi) {
  v = (v < lo) ? lo : v;
  v = (v > hi) ? hi : v;
  return v;
}
// Rust `f as u8`: saturating, truncating toward zero, NaN -> 0.
MG_HD uint8_t as_u8(float v) {
  if (!(v == v) || v <= 0.0f) return 0;
  if (v >= 255.0f) return 255;
  return (uint8_t)(int)v;
}

// --------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror & Shaw, SC'11).
// --------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

MG_HD void mulhilo(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
  hi = __umulhi(a, b);
  lo = a * b;
#else
  uint64_t p = (uint64_t)a * b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
#endif
}

MG_HD u32x4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
MG_UNROLL
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(0xD2511F53u, c0, hi0, lo0);
    mulhilo(0xCD9E8D57u, c2, hi1, lo1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return u32x4{c0, c1, c2, c3};
}

// Uniform integer in [0, n) by multiply-high range reduction.
MG_HD uint32_t range_u32(uint32_t r, uint32_t n) {
#if defined(__CUDA_ARCH__)
  return __umulhi(r, n);
#else
  return (uint32_t)(((uint64_t)r * n) >> 32);
#endif
}
// Uniform float in [0,1) from the top 24 bits (rand's f32 construction).
MG_HD float unit_f32(uint32_t r) { return MG_MUL((float)(r >> 8), 5.9604644775390625e-08f); }

// --------------------------------------------------------------------------
// exp(x): Cody-Waite reduction x = k ln2 + r (ln2 split into a 24-bit head
// and a tail), degree-7 Taylor polynomial on |r| <= ln2/2 in Horner form
// with fused multiply-adds, scaling by 2^k.  Max error 0.87 ulp on
// [-87, 88.7] against FP64 exp.  NaN passes through, x > 88.7 -> +inf,
// x < -87 -> 0.
// --------------------------------------------------------------------------
MG_HD float exp_spec(float x) {
  if (!(x == x)) return x;
  if (x > 88.7f) return u2f(0x7f800000u);
  if (x < -87.0f) return 0.0f;
  float k = MG_RINT(MG_MUL(x, 1.44269504088896341f));
  float r = MG_FMA(-k, 0.693145751953125f, x);
  r = MG_FMA(-k, 1.428606820309417232e-6f, r);
  float p = 1.0f / 5040.0f;
  p = MG_FMA(p, r, 1.0f / 720.0f);
  p = MG_FMA(p, r, 1.0f / 120.0f);
  p = MG_FMA(p, r, 1.0f / 24.0f);
  p = MG_FMA(p, r, 1.0f / 6.0f);
  p = MG_FMA(p, r, 0.5f);
  p = MG_FMA(p, r, 1.0f);
  p = MG_FMA(p, r, 1.0f);
  int ki = (int)k;
  if (ki > 127) return MG_MUL(MG_MUL(p, 2.0f), u2f((uint32_t)(127 + 127) << 23));
  return MG_MUL(p, u2f((uint32_t)(ki + 127) << 23));
}

// --------------------------------------------------------------------------
// Cube root on (216/24389, ~1.1]: bit-level first guess for t^(-1/3) (within
// 3.3%), two Newton steps r += r/3 (1 - t r^3) (relative error then below
// 1e-5), y = t r^2, one Newton polish of y.  Max error 0.77 ulp against FP64
// cbrt on that interval (every float checked), mean error -0.004 ulp.
// --------------------------------------------------------------------------
constexpr int kCbrtNewton = 2;
MG_HD float cbrt_spec(float t) {
  float r = u2f(0x54A2FA8Cu - f2u(t) / 3u);
MG_UNROLL
  for (int k = 0; k < kCbrtNewton; ++k) {
    float r2 = MG_MUL(r, r);
    float r3 = MG_MUL(r2, r);
    float e = MG_FMA(-t, r3, 1.0f);
    r = MG_FMA(MG_MUL(r, 1.0f / 3.0f), e, r);
  }
  float rr = MG_MUL(r, r);
  float y = MG_MUL(t, rr);
  float y2 = MG_MUL(y, y);
  float res = MG_FMA(-y2, y, t);
  return MG_FMA(res, MG_MUL(rr, 1.0f / 3.0f), y);
}

// Constants of the sRGB8 -> Lab conversion.  Filled on the host in FP64
// (transfer-function table, RGB->XYZ matrix from the sRGB primaries and the
// D65 white divided by the white point) and rounded once to FP32.
struct LabConsts {
  float lut[256];
  float ms[9];
  float eps, k1, k2;
};

// Fixed-point scale of the per-pixel Lab sums: values are scaled by 2^20 and
// rounded to integers, so a sum is exact and order-independent.
constexpr float kLabQ = 1048576.0f;
constexpr float kLabInvQ = 9.5367431640625e-07f;

MG_HD float lab_f(float t, float eps, float k1, float k2) {
  return t > eps ? cbrt_spec(t) : MG_FMA(k1, t, k2);
}

// One sRGB8 pixel -> Lab (palette's Lab::from_color semantics: CIE 1976,
// D65, then L clamped to [0,100], a and b to [-128,127]).
MG_HD void lab_pixel(const float* lut, const float* ms, float eps, float k1, float k2,
                     uint32_t r8, uint32_t g8, uint32_t b8, float& L, float& A, float& B) {
  float R = lut[r8], G = lut[g8], Bl = lut[b8];
  float tx = MG_FMA(ms[2], Bl, MG_FMA(ms[1], G, MG_MUL(ms[0], R)));
  float ty = MG_FMA(ms[5], Bl, MG_FMA(ms[4], G, MG_MUL(ms[3], R)));
  float tz = MG_FMA(ms[8], Bl, MG_FMA(ms[7], G, MG_MUL(ms[6], R)));
  float fx = lab_f(tx, eps, k1, k2), fy = lab_f(ty, eps, k1, k2), fz = lab_f(tz, eps, k1, k2);
  L = rclamp(MG_FMA(116.0f, fy, -16.0f), 0.0f, 100.0f);
  A = rclamp(MG_MUL(500.0f, MG_SUB(fx, fy)), -128.0f, 127.0f);
  B = rclamp(MG_MUL(200.0f, MG_SUB(fy, fz)), -128.0f, 127.0f);
}

MG_HD long long lab_quant(float v) {
#if defined(__CUDA_ARCH__)
  // |v| <= 128, so v * 2^20 fits a 32-bit integer: the 32-bit conversion
  // (round to nearest even, as llrint) is exact and cheaper than the 64-bit one.
  return (long long)__float2int_rn(__fmul_rn(v, kLabQ));
#else
  return (long long)std::llrintf(v * kLabQ);
#endif
}

// The quantised Lab of one pixel as the reduction kernels compute it:
// lab_quant of each lab_pixel component, rearranged without changing a
// result.  The 2^20 scale is folded into the L, a, b constants (scaling by a
// power of two commutes with rounding), and the clamps are left out: for all
// 2^24 sRGB8 colours a and b stay inside [-128, 127] and L inside [0, 100]
// except for black, whose L of -6e-8 quantises to 0 as the clamped value
// does.  The kernels evaluate this on pairs of pixels with packed FP32x2
// arithmetic (each component rounded as here).  The cube root is cbrt_spec
// with the seed's division by 3 as a multiply-high (div3_u31: equal for
// inputs below 2^31, and t >= 0 here).
constexpr float kLabQL = 121634816.0f;   // 116 * 2^20
constexpr float kLabQL0 = -16777216.0f;  // -16 * 2^20
constexpr float kLabQA = 524288000.0f;   // 500 * 2^20
constexpr float kLabQB = 209715200.0f;   // 200 * 2^20
MG_HD uint32_t div3_u31(uint32_t x) {  // x / 3 for x < 2^31
#if defined(__CUDA_ARCH__)
  return __umulhi(x, 0x55555556u);
#else
  return (uint32_t)(((uint64_t)x * 0x55555556u) >> 32);
#endif
}
MG_HD int quant_rn(float v) {
#if defined(__CUDA_ARCH__)
  return __float2int_rn(v);
#else
  return (int)std::lrintf(v);
#endif
}
MG_HD void lab_pixel_q(const float* lut, const float* ms, float eps, float k1, float k2, uint32_t r8, uint32_t g8,
                       uint32_t b8, int& qL, int& qA, int& qB) {
  float R = lut[r8], G = lut[g8], Bl = lut[b8];
  float t[3];
  for (int i = 0; i < 3; ++i) t[i] = MG_FMA(ms[3 * i + 2], Bl, MG_FMA(ms[3 * i + 1], G, MG_MUL(ms[3 * i], R)));
  float f[3];
  for (int i = 0; i < 3; ++i) {
    float r = u2f(0x54A2FA8Cu - div3_u31(f2u(t[i])));
    for (int k = 0; k < kCbrtNewton; ++k) {
      float r2 = MG_MUL(r, r);
      float r3 = MG_MUL(r2, r);
      float e = MG_FMA(-t[i], r3, 1.0f);
      r = MG_FMA(MG_MUL(r, 1.0f / 3.0f), e, r);
    }
    float rr = MG_MUL(r, r);
    float y = MG_MUL(t[i], rr);
    float y2 = MG_MUL(y, y);
    float res = MG_FMA(-y2, y, t[i]);
    float c = MG_FMA(res, MG_MUL(rr, 1.0f / 3.0f), y);
    float l = MG_FMA(k1, t[i], k2);
    f[i] = t[i] > eps ? c : l;
  }
  qL = quant_rn(MG_FMA(kLabQL, f[1], kLabQL0));
  qA = quant_rn(MG_MUL(MG_ADD(f[0], -f[1]), kLabQA));
  qB = quant_rn(MG_MUL(MG_ADD(f[1], -f[2]), kLabQB));
}

// Sum (fixed point) / pixel count -> mean, in FP32.
MG_HD float lab_mean(long long sum, long long n) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(__fdiv_rn(__ll2float_rn(sum), __ll2float_rn(n)), kLabInvQ);
#else
  return ((float)sum / (float)n) * kLabInvQ;
#endif
}

// --------------------------------------------------------------------------
// Lab distances.  similarity.rs:141-146 (Euclidean, sqrt) and kiddo's
// SquaredEuclidean (no sqrt), both summed in dimension order with no fused
// multiply-add.
// --------------------------------------------------------------------------
MG_HD float sq_dist(float q0, float q1, float q2, float p0, float p1, float p2) {
  float d0 = MG_SUB(q0, p0), d1 = MG_SUB(q1, p1), d2 = MG_SUB(q2, p2);
  return MG_ADD(MG_ADD(MG_MUL(d0, d0), MG_MUL(d1, d1)), MG_MUL(d2, d2));
}
MG_HD float lab_distance(float a0, float a1, float a2, float b0, float b1, float b2) {
  return MG_SQRT(sq_dist(a0, a1, a2, b0, b1, b2));
}
// 1/(sim+1) of adjacency.rs:83/110/121/168-207; sim(i,i) = 0 (similarity.rs:90-92).
MG_HD float adj_weight_from_sim(float sim) { return MG_DIV(1.0f, MG_ADD(sim, 1.0f)); }

// --------------------------------------------------------------------------
// HSV (palette 0.7.6 hexcone on non-linear sRGB) and the colour adjustment of
// color_adjustment.rs.
// --------------------------------------------------------------------------
MG_HD void rgb_to_hsv(float r, float g, float b, float& h, float& s, float& v) {
  float red = r < 0.0f ? 0.0f : r, green = g < 0.0f ? 0.0f : g, blue = b < 0.0f ? 0.0f : b;
  float mx, mn, sep, coeff;
  if (red > green) { mx = red; mn = green; sep = MG_SUB(green, blue); coeff = 0.0f; }
  else { mx = green; mn = red; sep = MG_SUB(blue, red); coeff = 2.0f; }
  if (blue > mx) { mx = blue; sep = MG_SUB(red, green); coeff = 4.0f; }
  else if (blue < mn) { mn = blue; }
  float hh = 0.0f, ss = 0.0f;
  if (mx != mn) {
    float d = MG_SUB(mx, mn);
    hh = MG_MUL(MG_ADD(MG_DIV(sep, d), coeff), 60.0f);
    ss = MG_DIV(d, mx);
  }
  h = hh;
  s = rclamp(ss, 0.0f, 1.0f);
  v = rclamp(mx, 0.0f, 1.0f);
}

MG_HD void hsv_to_rgb(float hue, float s, float v, float& r, float& g, float& b) {
  // hue - floor(hue / 360) * 360: for 0 < hue < 360 the rounded quotient is
  // below 1 (at most 1 - 2^-24), so the expression is hue itself.
  float pos = (hue > 0.0f && hue < 360.0f) ? hue : MG_SUB(hue, MG_MUL(MG_FLOOR(MG_DIV(hue, 360.0f)), 360.0f));
  float c = MG_MUL(v, s);
  float h = MG_DIV(pos, 60.0f);
  float hm2 = MG_SUB(h, MG_MUL(MG_FLOOR(MG_MUL(h, 0.5f)), 2.0f));
  float t = MG_SUB(hm2, 1.0f);
  t = t < 0.0f ? -t : t;
  float x = MG_MUL(c, MG_SUB(1.0f, t));
  float m = MG_SUB(v, c);
  bool z0 = h >= 0.0f && h < 1.0f, z1 = h >= 1.0f && h < 2.0f, z2 = h >= 2.0f && h < 3.0f;
  bool z3 = h >= 3.0f && h < 4.0f, z4 = h >= 4.0f && h < 5.0f;
  float red = (z1 || z4) ? x : ((z2 || z3) ? 0.0f : c);
  float green = (z0 || z3) ? x : ((z1 || z2) ? c : 0.0f);
  float blue = (z0 || z1) ? 0.0f : ((z3 || z4) ? c : x);
  r = rclamp(MG_ADD(red, m), 0.0f, 1.0f);
  g = rclamp(MG_ADD(green, m), 0.0f, 1.0f);
  b = rclamp(MG_ADD(blue, m), 0.0f, 1.0f);
}

struct Adjust { float brightness, contrast, hue_shift, saturation; };

// color_adjustment.rs:30-37.
MG_HD Adjust adjustment_new(float br, float co, float hue, float sat) {
  return Adjust{rclamp(br, -1.0f, 1.0f), rclamp(co, 0.0f, 2.0f), rclamp(hue, -180.0f, 180.0f),
                rclamp(sat, 0.0f, 2.0f)};
}

// v/255 for v in 0..255, as the reference's `x as f32 / 255.0`.
MG_HD float u8_unit(uint32_t v) { return MG_DIV((float)v, 255.0f); }

// color_adjustment.rs:99-154 calculate_optimal_adjustment.
MG_HD Adjust optimal_adjustment(uint32_t tr8, uint32_t tg8, uint32_t tb8, uint32_t gr8, uint32_t gg8,
                                uint32_t gb8, float strength) {
  float tr = u8_unit(tr8), tg = u8_unit(tg8), tb = u8_unit(tb8);
  float gr = u8_unit(gr8), gg = u8_unit(gg8), gb = u8_unit(gb8);
  float tile_luma = MG_ADD(MG_ADD(MG_MUL(0.299f, tr), MG_MUL(0.587f, tg)), MG_MUL(0.114f, tb));
  float target_luma = MG_ADD(MG_ADD(MG_MUL(0.299f, gr), MG_MUL(0.587f, gg)), MG_MUL(0.114f, gb));
  float brightness = MG_MUL(MG_SUB(target_luma, tile_luma), strength);
  float th, ts, tv, gh, gs, gv;
  rgb_to_hsv(tr, tg, tb, th, ts, tv);
  rgb_to_hsv(gr, gg, gb, gh, gs, gv);
  float hue = 0.0f;
  if (ts > 0.1f && gs > 0.1f) {
    float diff = MG_SUB(gh, th);
    float wrapped = diff > 180.0f ? MG_SUB(diff, 360.0f) : (diff < -180.0f ? MG_ADD(diff, 360.0f) : diff);
    hue = MG_MUL(MG_MUL(wrapped, strength), 0.5f);
  }
  float sat = 1.0f;
  if (ts > 0.01f) {
    float ratio = MG_DIV(gs, ts);
    sat = MG_ADD(1.0f, MG_MUL(MG_MUL(MG_SUB(ratio, 1.0f), strength), 0.7f));
  }
  (void)tv; (void)gv;
  return adjustment_new(brightness, 1.0f, hue, sat);
}

// color_adjustment.rs:91-96 apply_brightness_contrast.
MG_HD float brightness_contrast(float v, float brightness, float contrast) {
  float c = rclamp(MG_ADD(MG_MUL(MG_SUB(v, 0.5f), contrast), 0.5f), 0.0f, 1.0f);
  return rclamp(MG_ADD(c, brightness), 0.0f, 1.0f);
}

// fmod(x, 360).  For |x| < 720 it is x itself below 360 in magnitude, else
// x -+ 360 with x's sign, which is exact (Sterbenz: 360 <= |x| <= 720).
// adjust_pixel's hues stay within (-240, 540).
MG_HD float fmod_360(float x) {
  const float ax = x < 0.0f ? -x : x;
  if (ax < 360.0f) return x;
  if (ax < 720.0f) {
    const float r = MG_SUB(ax, 360.0f);
    return x < 0.0f ? -r : r;
  }
  return MG_FMOD(x, 360.0f);
}

// color_adjustment.rs:53-87 adjust_pixel after the brightness/contrast step:
// c0..c2 are brightness_contrast of the pixel's channels (a function of the
// byte alone, so the composite tabulates it per tile).
MG_HD void adjust_from_bc(const Adjust& a, float c0, float c1, float c2, uint8_t& o0, uint8_t& o1, uint8_t& o2) {
  if (a.hue_shift != 0.0f || a.saturation != 1.0f) {
    float h, s, v;
    rgb_to_hsv(c0, c1, c2, h, s, v);
    float hh = MG_ADD(h, a.hue_shift);
    float rem = fmod_360(hh);
    if (rem < 0.0f) rem = MG_ADD(rem, 360.0f);
    float ss = rclamp(MG_MUL(s, a.saturation), 0.0f, 1.0f);
    hsv_to_rgb(rem, ss, v, c0, c1, c2);
  }
  o0 = as_u8(rclamp(MG_MUL(c0, 255.0f), 0.0f, 255.0f));
  o1 = as_u8(rclamp(MG_MUL(c1, 255.0f), 0.0f, 255.0f));
  o2 = as_u8(rclamp(MG_MUL(c2, 255.0f), 0.0f, 255.0f));
}

// x / 60, correctly rounded, as a multiply and one FMA correction: equal to
// the division for every float in [0x1p-120, 360] (checked exhaustively); the
// division itself below that.
MG_HD float div60(float x) {
  if (x < 0x1p-120f) return MG_DIV(x, 60.0f);
  const float q = MG_MUL(x, 1.0f / 60.0f);
  return MG_FMA(MG_FMA(-q, 60.0f, x), 1.0f / 60.0f, q);
}

// adjust_from_bc for channels in [0, 1] (the brightness/contrast table's
// values: clamped, possibly -0), rearranged without changing a result:
//  - rgb_to_hsv's clamps cannot bind: channels >= 0 (or -0, which the max
//    with 0 keeps), the value is the largest channel <= 1, the saturation
//    d / max is in [0, 1] as d = fl(max - min) <= max;
//  - the hue reaching hsv_to_rgb is in [-0, 360] (fmod_360 of the shifted hue,
//    then + 360 below zero), so its normalisation is the hue itself inside
//    (0, 360) and 0 at the ends (0 - 0 * 360, -0 - (-0) * 360, 360 - 360);
//  - pos / 60 through div60;
//  - the sector tests h in [i, i + 1) become the truncated index of h >= 0
//    (index 6 for h = 6 takes the last sector's branch, as before);
//  - each channel red + m is >= 0 (red in {c, x, 0}, x = c (1 - t) with t in
//    [0, 1], m = v - c >= 0 as c = v s <= v), so only the clamp at 1 can bind;
//  - the output v * 255 of a channel in [-0, 1] lies in [0, 255] and is never
//    NaN, so `as u8` is a truncating conversion.
MG_HD uint32_t unit_to_u8(float v) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(__fmul_rn(v, 255.0f));
#else
  return (uint32_t)(v * 255.0f);
#endif
}
MG_HD float min1(float v) { return v > 1.0f ? 1.0f : v; }
MG_HD void adjust_unit(const Adjust& a, float c0, float c1, float c2, uint8_t& o0, uint8_t& o1, uint8_t& o2) {
  if (a.hue_shift != 0.0f || a.saturation != 1.0f) {
    float mx, mn, sep, coeff;
    if (c0 > c1) { mx = c0; mn = c1; sep = MG_SUB(c1, c2); coeff = 0.0f; }
    else { mx = c1; mn = c0; sep = MG_SUB(c2, c0); coeff = 2.0f; }
    if (c2 > mx) { mx = c2; sep = MG_SUB(c0, c1); coeff = 4.0f; }
    else if (c2 < mn) { mn = c2; }
    float hh = 0.0f, s = 0.0f;
    if (mx != mn) {
      const float d = MG_SUB(mx, mn);
      hh = MG_MUL(MG_ADD(MG_DIV(sep, d), coeff), 60.0f);
      s = MG_DIV(d, mx);
    }
    float rem = fmod_360(MG_ADD(hh, a.hue_shift));
    if (rem < 0.0f) rem = MG_ADD(rem, 360.0f);
    const float pos = (rem > 0.0f && rem < 360.0f) ? rem : 0.0f;
    const float ss = rclamp(MG_MUL(s, a.saturation), 0.0f, 1.0f);
    const float v = mx;
    const float c = MG_MUL(v, ss);
    const float h = div60(pos);
    const float hm2 = MG_SUB(h, MG_MUL(MG_FLOOR(MG_MUL(h, 0.5f)), 2.0f));
    float t = MG_SUB(hm2, 1.0f);
    t = t < 0.0f ? -t : t;
    const float x = MG_MUL(c, MG_SUB(1.0f, t));
    const float m = MG_SUB(v, c);
    const uint32_t bit = 1u << (uint32_t)(int)h;  // h in [0, 6]
    const float red = (bit & 0x12u) ? x : ((bit & 0x0Cu) ? 0.0f : c);
    const float green = (bit & 0x09u) ? x : ((bit & 0x06u) ? c : 0.0f);
    const float blue = (bit & 0x03u) ? 0.0f : ((bit & 0x18u) ? c : x);
    c0 = min1(MG_ADD(red, m));
    c1 = min1(MG_ADD(green, m));
    c2 = min1(MG_ADD(blue, m));
  }
  o0 = (uint8_t)unit_to_u8(c0);
  o1 = (uint8_t)unit_to_u8(c1);
  o2 = (uint8_t)unit_to_u8(c2);
}

// y in [-0, 2^23): the bits of the float 2^23 + trunc(y) (the sum rounded
// toward zero: floats in [2^23, 2^24) are the integers), whose low byte is
// trunc(y) mod 256.
MG_HD uint32_t trunc_word(float y) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(__fadd_rz(y, 8388608.0f));
#else
  return 0x4B000000u + (uint32_t)y;
#endif
}
// h in [-0, 2^21): the bits of the float 2^21 + floor(4h) / 4 (the sum rounded
// toward zero: floats in [2^21, 2^22) step by 1/4), 0x4A000000 + floor(4h).
MG_HD uint32_t quarter_word(float h) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(__fadd_rz(h, 2097152.0f));
#else
  return 0x4A000000u + (uint32_t)(h * 4.0f);
#endif
}
// Bytes of the 8-byte value hi:lo picked by the nibbles of sel (each 0..7).
MG_HD uint32_t perm_bytes(uint32_t lo, uint32_t hi, uint32_t sel) {
#if defined(__CUDA_ARCH__)
  return __byte_perm(lo, hi, sel);
#else
  const uint64_t v = (uint64_t)hi << 32 | lo;
  uint32_t r = 0;
  for (int k = 0; k < 4; ++k) r |= (uint32_t)((v >> (8 * ((sel >> (4 * k)) & 7u))) & 0xFFu) << (8 * k);
  return r;
#endif
}
// The byte selector of hue sector i for adjust_word: channel r, g, b (result
// bytes 0, 1, 2) takes c (selector 0), x (1) or 0 (4), as hsv_to_rgb's sectors
// (c, x, 0), (x, c, 0), (0, c, x), (0, x, c), (x, 0, c), (c, 0, x), and h = 6
// the last sector's.
MG_HD uint32_t sector_perm(uint32_t i) {
  return i == 0 ? 0x410u : i == 1 ? 0x401u : i == 2 ? 0x104u : i == 3 ? 0x014u : i == 4 ? 0x041u : 0x140u;
}
// The hue shift and saturation for which adjust_word equals adjust_unit
// (adjustment_new's ranges, the HSV step active).
MG_HD bool adjust_word_applies(const Adjust& a) {
  return (a.hue_shift != 0.0f || a.saturation != 1.0f) && a.hue_shift >= -180.0f && a.hue_shift <= 180.0f &&
         a.saturation >= 0.0f && a.saturation <= 2.0f;
}

// adjust_unit for adjustments with adjust_word_applies, the output bytes as
// one word (r | g << 8 | b << 16; byte 3 is not part of the result).  `perm`
// holds sector_perm(i) at index i (0..7; device code: shared memory).
// Rearranged further without changing a result:
//  - the shifted hue x = hh + shift lies in [-240, 480] (hh in [-60, 300]), so
//    fmod_360 and the wrap below zero are x - 360 from 360 up (exact), x + 360
//    below zero, x itself between;
//  - pos / 60 by div60's multiply and FMA correction at every pos: below
//    2^-120 both quotients are below 2^-126, and a quotient that small
//    reaches the output only through sector 0 and t = |h - 1| = 1;
//  - floor(h) and 2 floor(h / 2) read from quarter_word(h);
//  - each output channel is one of c + m, x + m and m (min1(0 + m) = m, as
//    0 <= m = v - c <= v <= 1), each converted once by trunc_word, and the
//    sector's byte permutation picks them.
MG_HD uint32_t adjust_word(const Adjust& a, float c0, float c1, float c2, const uint32_t* perm) {
  float mx, mn, sep, coeff;
  if (c0 > c1) { mx = c0; mn = c1; sep = MG_SUB(c1, c2); coeff = 0.0f; }
  else { mx = c1; mn = c0; sep = MG_SUB(c2, c0); coeff = 2.0f; }
  if (c2 > mx) { mx = c2; sep = MG_SUB(c0, c1); coeff = 4.0f; }
  else if (c2 < mn) { mn = c2; }
  float hh = 0.0f, s = 0.0f;
  if (mx != mn) {
    const float d = MG_SUB(mx, mn);
    hh = MG_MUL(MG_ADD(MG_DIV(sep, d), coeff), 60.0f);
    s = MG_DIV(d, mx);
  }
  const float xs = MG_ADD(hh, a.hue_shift);
  float pos = MG_ADD(xs, xs < 0.0f ? 360.0f : (xs >= 360.0f ? -360.0f : 0.0f));
  pos = (pos > 0.0f && pos < 360.0f) ? pos : 0.0f;
  const float v = mx;
  const float c = MG_MUL(v, min1(MG_MUL(s, a.saturation)));
  const float q = MG_MUL(pos, 1.0f / 60.0f);
  const float h = MG_FMA(MG_FMA(-q, 60.0f, pos), 1.0f / 60.0f, q);
  const uint32_t hq = quarter_word(h);
  const float hm2 = MG_SUB(h, MG_SUB(u2f(hq & ~7u), 2097152.0f));
  float t = MG_SUB(hm2, 1.0f);
  t = t < 0.0f ? -t : t;
  const float x = MG_MUL(c, MG_SUB(1.0f, t));
  const float m = MG_SUB(v, c);
  const uint32_t wc = trunc_word(MG_MUL(min1(MG_ADD(c, m)), 255.0f));
  const uint32_t wx = trunc_word(MG_MUL(min1(MG_ADD(x, m)), 255.0f));
  const uint32_t wz = trunc_word(MG_MUL(m, 255.0f));
#if defined(__CUDA_ARCH__)
  const uint32_t sel = *reinterpret_cast<const uint32_t*>(reinterpret_cast<const char*>(perm) + (hq & 0x1Cu));
#else
  const uint32_t sel = perm[(hq >> 2) & 7u];
#endif
  return perm_bytes(perm_bytes(wc, wx, 0x40u), wz, sel);
}

// color_adjustment.rs:53-87 adjust_pixel.  r, g, b are the channels as v/255.
MG_HD void adjust_pixel(const Adjust& a, float r, float g, float b, uint8_t& o0, uint8_t& o1, uint8_t& o2) {
  adjust_from_bc(a, brightness_contrast(r, a.brightness, a.contrast), brightness_contrast(g, a.brightness, a.contrast),
                 brightness_contrast(b, a.brightness, a.contrast), o0, o1, o2);
}

}  // namespace mg
