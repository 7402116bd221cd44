// composite.cuh -- one tile of the composite, by one CTA, shared by the
// single-mosaic kernel (k_composite.cu) and the batch kernel (k_batch.cu):
// main.rs:583-592 copies the adjusted tile into the output;
// color_adjustment.rs:53-87 adjust_pixel on each pixel.
//
// The brightness/contrast step of adjust_pixel is a function of one byte, so
// the CTA tabulates it for the tile's adjustment (256 entries) and each pixel
// looks its three channels up; the HSV part stays per pixel, as adjust_word
// for adjustments in adjustment_new's ranges (every adjustment the composite
// computes) and adjust_unit otherwise (mg_math.h: adjust_from_bc rearranged
// for channels in [0, 1] without changing a result -- fewer comparisons,
// selects and clamps, the division by 60 as a multiply and one correction,
// the sector's channels as one byte permutation of three converted values,
// the conversions as additions rounded toward zero).
// With tile widths a multiple of 4, four pixels of a tile row are 12 bytes,
// 4-byte aligned in the thumbnail and in the output, and move as three 32-bit
// words.
#pragma once
#include "mg_internal.h"

namespace mg {

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int i) { return (w >> (8 * i)) & 0xFFu; }

// brightness_contrast (color_adjustment.rs:91-96) of v/255 for every byte v.
__device__ __forceinline__ void tile_bc_table(float* s_bc, const Adjust& a) {
  for (int v = threadIdx.x; v < 256; v += blockDim.x) s_bc[v] = brightness_contrast(u8_unit((uint32_t)v), a.brightness, a.contrast);
}

// The sector permutations of adjust_word in shared memory (threads 0..7).
__device__ __forceinline__ void sector_perm_table(uint32_t* s_perm) {
  if (threadIdx.x < 8) s_perm[threadIdx.x] = sector_perm(threadIdx.x);
}

// Per-pixel arithmetic of a tile: 0 a copy, 1 adjust_unit, 2 adjust_word.
enum TileMode { kTileCopy = 0, kTileUnit = 1, kTileWord = 2 };

// One pixel (channels b0, b1, b2) as r | g << 8 | b << 16 (byte 3 not used).
template <int kMode>
__device__ __forceinline__ uint32_t tile_pixel(uint32_t b0, uint32_t b1, uint32_t b2, const Adjust& a,
                                               const float* s_bc, const uint32_t* s_perm) {
  if (kMode == kTileCopy) return b0 | b1 << 8 | b2 << 16;
  if (kMode == kTileWord) return adjust_word(a, s_bc[b0], s_bc[b1], s_bc[b2], s_perm);
  uint8_t o0, o1, o2;
  adjust_unit(a, s_bc[b0], s_bc[b1], s_bc[b2], o0, o1, o2);
  return (uint32_t)o0 | (uint32_t)o1 << 8 | (uint32_t)o2 << 16;
}

template <int kMode>
__device__ __forceinline__ void tile_pixels(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int tw,
                                            int th, size_t pitch, const Adjust& a, const float* s_bc,
                                            const uint32_t* s_perm) {
  if ((tw & 3) == 0) {
    const int gpr = tw >> 2, total = gpr * th;
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
      const int row = q / gpr, gx = (q - row * gpr) << 2;
      uint32_t* d = reinterpret_cast<uint32_t*>(dst + row * pitch + (size_t)gx * 3);
      const uint32_t* s = reinterpret_cast<const uint32_t*>(src + ((size_t)row * tw + gx) * 3);
      const uint32_t w0 = __ldg(s), w1 = __ldg(s + 1), w2 = __ldg(s + 2);
      if (kMode == kTileCopy) {
        d[0] = w0;
        d[1] = w1;
        d[2] = w2;
        continue;
      }
      // pixel k: bytes 3k .. 3k + 2 of w0:w1:w2; results packed back as bytes 0-2 of each
      const uint32_t p0 = tile_pixel<kMode>(byte_of(w0, 0), byte_of(w0, 1), byte_of(w0, 2), a, s_bc, s_perm);
      const uint32_t p1 = tile_pixel<kMode>(byte_of(w0, 3), byte_of(w1, 0), byte_of(w1, 1), a, s_bc, s_perm);
      const uint32_t p2 = tile_pixel<kMode>(byte_of(w1, 2), byte_of(w1, 3), byte_of(w2, 0), a, s_bc, s_perm);
      const uint32_t p3 = tile_pixel<kMode>(byte_of(w2, 1), byte_of(w2, 2), byte_of(w2, 3), a, s_bc, s_perm);
      d[0] = __byte_perm(p0, p1, 0x4210);
      d[1] = __byte_perm(p1, p2, 0x5421);
      d[2] = __byte_perm(p2, p3, 0x6542);
    }
    return;
  }
  const int total = tw * th;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int row = q / tw, x = q - row * tw;
    uint8_t* d = dst + row * pitch + (size_t)x * 3;
    const uint8_t* s = src + ((size_t)row * tw + x) * 3;
    const uint32_t p = tile_pixel<kMode>(s[0], s[1], s[2], a, s_bc, s_perm);
    d[0] = (uint8_t)p;
    d[1] = (uint8_t)(p >> 8);
    d[2] = (uint8_t)(p >> 16);
  }
}

// The tile of thumbnail `src` (tw x th RGB8; nullptr: an empty cell, black)
// into `dst` (row pitch `pitch` bytes), adjusted when `adjust` (s_bc from
// tile_bc_table for `a`, s_perm from sector_perm_table).  `adjust` and `a` are
// uniform over the CTA.
__device__ __forceinline__ void composite_tile(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int tw,
                                               int th, size_t pitch, bool adjust, const Adjust& a,
                                               const float* s_bc, const uint32_t* s_perm) {
  if (!src) {
    const int per_row = (tw & 3) == 0 ? 3 * tw / 4 : 3 * tw;  // 32-bit words, else bytes
    for (int q = threadIdx.x; q < per_row * th; q += blockDim.x) {
      const int row = q / per_row, k = q - row * per_row;
      if ((tw & 3) == 0) reinterpret_cast<uint32_t*>(dst + row * pitch)[k] = 0u;
      else dst[row * pitch + k] = 0;
    }
    return;
  }
  if (!adjust) tile_pixels<kTileCopy>(src, dst, tw, th, pitch, a, s_bc, s_perm);
  else if (adjust_word_applies(a)) tile_pixels<kTileWord>(src, dst, tw, th, pitch, a, s_bc, s_perm);
  else tile_pixels<kTileUnit>(src, dst, tw, th, pitch, a, s_bc, s_perm);
}

// Threads per CTA for tiles of tw x th: the fewest passes over the tile's
// pixel groups at up to 256 threads, in whole warps.
inline int tile_threads(int tw, int th) {
  const int groups = (tw & 3) == 0 ? (tw >> 2) * th : tw * th;
  const int passes = (groups + 255) / 256;
  const int per = (groups + passes - 1) / passes;
  return ((per + 31) / 32) * 32;
}

}  // namespace mg
