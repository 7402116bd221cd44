// lab_reduce.cuh -- per-pixel Lab and mean-RGB sums over rows of an RGB8
// region, one warp at a time.  Shared by the region kernel (k_lab.cu: target
// cells, materials, thumbnails) and the batch kernel (k_batch.cu: the cells
// of many targets).
//
// Reference: lib.rs:94-119 calculate_average_lab (per-pixel sRGB8 -> Lab,
// summed, divided by the pixel count) and main.rs:687-708
// calculate_average_rgb (integer sums).
//
// The reduction is issue-bound (three cube roots per pixel), so the design
// minimises issued instructions per pixel:
//   * pixels are converted two at a time in packed FP32x2 arithmetic
//     (__ffma2_rn / __fmul2_rn / __fadd2_rn, each component rounded exactly
//     as the scalar op), one pixel per component, so the result is
//     mg_math.h's lab_pixel_q bit for bit;
//   * a lane loads a group of 16, 8 or 4 pixels per step as three 16-, 8- or
//     4-byte vectors (48, 24 or 12 bytes), the widest the row's alignment and
//     width allow; other rows go pixel pair by pixel pair;
//   * quantised Lab is summed in 32-bit registers within a group (at most 16
//     pixels of |value| < 109 * 2^20) and folded into 64-bit sums once per
//     group;
//   * the sRGB transfer table sits in shared memory (one load per channel).
// Integer sums are exact, so the result does not depend on how pixels are
// split over lanes, warps or CTAs.
#pragma once
#include "mg_internal.h"

namespace mg {

// The conversion constants, held per thread as packed pairs.
struct LabK {
  float2 m[9];
  float eps, k1, k2;
};

__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

__device__ __forceinline__ LabK make_lab_k(const float* ms, float eps, float k1, float k2) {
  LabK K;
#pragma unroll
  for (int i = 0; i < 9; ++i) K.m[i] = dup2(ms[i]);
  K.eps = eps;
  K.k1 = k1;
  K.k2 = k2;
  return K;
}

// cbrt_spec of both components (mg_math.h), the seed's division by 3 as a
// multiply-high (t >= 0, so its bits are below 2^31).
__device__ __forceinline__ float2 cbrt_pair(float2 t) {
  float2 r = make_float2(__uint_as_float(0x54A2FA8Cu - div3_u31(__float_as_uint(t.x))),
                         __uint_as_float(0x54A2FA8Cu - div3_u31(__float_as_uint(t.y))));
  const float2 nt = neg2(t);
  const float2 third = dup2(1.0f / 3.0f);
#pragma unroll
  for (int k = 0; k < kCbrtNewton; ++k) {
    const float2 r2 = __fmul2_rn(r, r);
    const float2 r3 = __fmul2_rn(r2, r);
    const float2 e = __ffma2_rn(nt, r3, dup2(1.0f));
    r = __ffma2_rn(__fmul2_rn(r, third), e, r);
  }
  const float2 rr = __fmul2_rn(r, r);
  const float2 y = __fmul2_rn(t, rr);
  const float2 y2 = __fmul2_rn(y, y);
  const float2 res = __ffma2_rn(neg2(y2), y, t);
  return __ffma2_rn(res, __fmul2_rn(rr, third), y);
}

// CIE f(t) of both components: the cube root above eps, else k1 t + k2.
__device__ __forceinline__ float2 lab_f_pair(float2 t, const LabK& K) {
  const float2 c = cbrt_pair(t);
  const float2 l = __ffma2_rn(dup2(K.k1), t, dup2(K.k2));
  return make_float2(t.x > K.eps ? c.x : l.x, t.y > K.eps ? c.y : l.y);
}

// Quantised L, a, b of pixels (ra, ga, ba) and (rb, gb, bb), as lab_pixel_q.
// Component x belongs to the first pixel, y to the second.
__device__ __forceinline__ void lab_pair(const float* __restrict__ lut, const LabK& K, uint32_t ra, uint32_t ga,
                                         uint32_t ba, uint32_t rb, uint32_t gb, uint32_t bb, int2& qL, int2& qA,
                                         int2& qB) {
  const float2 R = make_float2(lut[ra], lut[rb]);
  const float2 G = make_float2(lut[ga], lut[gb]);
  const float2 B = make_float2(lut[ba], lut[bb]);
  const float2 tx = __ffma2_rn(K.m[2], B, __ffma2_rn(K.m[1], G, __fmul2_rn(K.m[0], R)));
  const float2 ty = __ffma2_rn(K.m[5], B, __ffma2_rn(K.m[4], G, __fmul2_rn(K.m[3], R)));
  const float2 tz = __ffma2_rn(K.m[8], B, __ffma2_rn(K.m[7], G, __fmul2_rn(K.m[6], R)));
  const float2 fx = lab_f_pair(tx, K), fy = lab_f_pair(ty, K), fz = lab_f_pair(tz, K);
  const float2 L = __ffma2_rn(dup2(kLabQL), fy, dup2(kLabQL0));
  const float2 A = __fmul2_rn(__fadd2_rn(fx, neg2(fy)), dup2(kLabQA));
  const float2 Bq = __fmul2_rn(__fadd2_rn(fy, neg2(fz)), dup2(kLabQB));
  qL = make_int2(__float2int_rn(L.x), __float2int_rn(L.y));
  qA = make_int2(__float2int_rn(A.x), __float2int_rn(A.y));
  qB = make_int2(__float2int_rn(Bq.x), __float2int_rn(Bq.y));
}

// One lane's running sums.
struct LabAcc {
  long long L = 0, A = 0, B = 0;
  unsigned R = 0, G = 0, Bc = 0;
};

// Byte i of a little-endian word array.
template <int I, int N>
__device__ __forceinline__ uint32_t byte_of(const uint32_t (&w)[N]) {
  return (w[I >> 2] >> (8 * (I & 3))) & 0xFFu;
}

// kG pixels held as 3 kG / 4 words (R G B R G B ...).
template <int kG, bool kLab, int P = 0>
struct GroupSum {
  static __device__ __forceinline__ void run(const uint32_t (&w)[3 * kG / 4], const float* lut, const LabK& K,
                                             int& sL, int& sA, int& sB, unsigned& sR, unsigned& sG, unsigned& sBc) {
    if constexpr (P < kG) {
      const uint32_t ra = byte_of<3 * P + 0>(w), ga = byte_of<3 * P + 1>(w), ba = byte_of<3 * P + 2>(w);
      const uint32_t rb = byte_of<3 * P + 3>(w), gb = byte_of<3 * P + 4>(w), bb = byte_of<3 * P + 5>(w);
      sR += ra + rb;
      sG += ga + gb;
      sBc += ba + bb;
      if constexpr (kLab) {
        int2 qL, qA, qB;
        lab_pair(lut, K, ra, ga, ba, rb, gb, bb, qL, qA, qB);
        sL += qL.x + qL.y;
        sA += qA.x + qA.y;
        sB += qB.x + qB.y;
      }
      GroupSum<kG, kLab, P + 2>::run(w, lut, K, sL, sA, sB, sR, sG, sBc);
    }
  }
};

template <int kG>
__device__ __forceinline__ void load_group(const uint8_t* p, uint32_t (&w)[3 * kG / 4]) {
  if constexpr (kG == 16) {
    const uint4* v = reinterpret_cast<const uint4*>(p);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const uint4 a = v[i];
      w[4 * i] = a.x; w[4 * i + 1] = a.y; w[4 * i + 2] = a.z; w[4 * i + 3] = a.w;
    }
  } else if constexpr (kG == 8) {
    const uint2* v = reinterpret_cast<const uint2*>(p);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const uint2 a = v[i];
      w[2 * i] = a.x; w[2 * i + 1] = a.y;
    }
  } else {
    const uint32_t* v = reinterpret_cast<const uint32_t*>(p);
#pragma unroll
    for (int i = 0; i < 3; ++i) w[i] = v[i];
  }
}

// Rows [y0, y1) of a region w pixels wide, in groups of kG pixels (w a
// multiple of kG; img and stride multiples of kG bytes).  Lane l takes groups
// l, l + 32, ... in row-major order.
template <int kG, bool kLab>
__device__ __forceinline__ void rows_groups(const uint8_t* __restrict__ img, int w, int64_t stride, int y0, int y1,
                                            int lane, const float* lut, const LabK& K, LabAcc& acc) {
  const int gpr = w / kG;
  const int ng = (y1 - y0) * gpr;
  int gx = lane % gpr, y = y0 + lane / gpr;
  const int dgx = 32 % gpr, dgy = 32 / gpr;
  for (int q = lane; q < ng; q += 32) {
    uint32_t wv[3 * kG / 4];
    load_group<kG>(img + (int64_t)y * stride + 3 * kG * gx, wv);
    int sL = 0, sA = 0, sB = 0;
    unsigned sR = 0, sG = 0, sBc = 0;
    GroupSum<kG, kLab>::run(wv, lut, K, sL, sA, sB, sR, sG, sBc);
    acc.L += sL;
    acc.A += sA;
    acc.B += sB;
    acc.R += sR;
    acc.G += sG;
    acc.Bc += sBc;
    gx += dgx;
    y += dgy;
    if (gx >= gpr) {
      gx -= gpr;
      ++y;
    }
  }
}

// Any row geometry: pixel pairs (x, x + 1) of each row, byte loads; a row of
// odd width ends in a pair whose second pixel repeats the first and counts 0.
template <bool kLab>
__device__ __forceinline__ void rows_pairs(const uint8_t* __restrict__ img, int w, int64_t stride, int y0, int y1,
                                           int lane, const float* lut, const LabK& K, LabAcc& acc) {
  const int ppr = (w + 1) >> 1;
  const int np = (y1 - y0) * ppr;
  for (int q = lane; q < np; q += 32) {
    const int row = q / ppr;
    const int x = 2 * (q - row * ppr);
    const uint8_t* p = img + (int64_t)(y0 + row) * stride + 3 * x;
    const bool two = x + 1 < w;
    const uint32_t ra = p[0], ga = p[1], ba = p[2];
    const uint32_t rb = two ? p[3] : ra, gb = two ? p[4] : ga, bb = two ? p[5] : ba;
    acc.R += ra + (two ? rb : 0u);
    acc.G += ga + (two ? gb : 0u);
    acc.Bc += ba + (two ? bb : 0u);
    if constexpr (kLab) {
      int2 qL, qA, qB;
      lab_pair(lut, K, ra, ga, ba, rb, gb, bb, qL, qA, qB);
      acc.L += (long long)qL.x + (two ? qL.y : 0);
      acc.A += (long long)qA.x + (two ? qA.y : 0);
      acc.B += (long long)qB.x + (two ? qB.y : 0);
    }
  }
}

// The lane's share of rows [y0, y1) of a region, by the widest group form the
// geometry allows (warp-uniform: every lane sees the same region).
template <bool kLab>
__device__ __forceinline__ void reduce_rows(const uint8_t* img, int w, int64_t stride, int y0, int y1, int lane,
                                            const float* lut, const LabK& K, LabAcc& acc) {
  const uint64_t align = (uint64_t)(uintptr_t)img | (uint64_t)stride;
  if ((w & 15) == 0 && (align & 15) == 0) rows_groups<16, kLab>(img, w, stride, y0, y1, lane, lut, K, acc);
  else if ((w & 7) == 0 && (align & 7) == 0) rows_groups<8, kLab>(img, w, stride, y0, y1, lane, lut, K, acc);
  else if ((w & 3) == 0 && (align & 3) == 0) rows_groups<4, kLab>(img, w, stride, y0, y1, lane, lut, K, acc);
  else rows_pairs<kLab>(img, w, stride, y0, y1, lane, lut, K, acc);
}

// Sums of the whole warp, in every lane (RGB widened to 64 bits).
struct LabSums {
  long long L, A, B;
  unsigned long long R, G, Bc;
};
template <bool kLab>
__device__ __forceinline__ LabSums warp_sums(const LabAcc& a) {
  LabSums s{a.L, a.A, a.B, a.R, a.G, a.Bc};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (kLab) {
      s.L += __shfl_xor_sync(0xffffffffu, s.L, o);
      s.A += __shfl_xor_sync(0xffffffffu, s.A, o);
      s.B += __shfl_xor_sync(0xffffffffu, s.B, o);
    }
    s.R += __shfl_xor_sync(0xffffffffu, s.R, o);
    s.G += __shfl_xor_sync(0xffffffffu, s.G, o);
    s.Bc += __shfl_xor_sync(0xffffffffu, s.Bc, o);
  }
  return s;
}

}  // namespace mg
