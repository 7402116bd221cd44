// composite.cuh -- one tile of the composite, by one CTA, shared by the
// single-mosaic kernel (k_composite.cu) and the batch kernel (k_batch.cu):
// main.rs:583-592 copies the adjusted tile into the output;
// color_adjustment.rs:53-87 adjust_pixel on each pixel.
//
// The brightness/contrast step of adjust_pixel is a function of one byte, so
// the CTA tabulates it for the tile's adjustment (256 entries) and each pixel
// looks its three channels up; the HSV part stays per pixel, as adjust_unit
// (mg_math.h: adjust_from_bc rearranged for channels in [0, 1] without
// changing a result -- fewer comparisons, selects and clamps, the division by
// 60 as a multiply and one correction, the output a truncating conversion).
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

// The tile of thumbnail `src` (tw x th RGB8; nullptr: an empty cell, black)
// into `dst` (row pitch `pitch` bytes), adjusted when `adjust` (s_bc from
// tile_bc_table for `a`).  `adjust` is uniform over the CTA.
__device__ __forceinline__ void composite_tile(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int tw,
                                               int th, size_t pitch, bool adjust, const Adjust& a,
                                               const float* s_bc) {
  if ((tw & 3) == 0) {
    const int gpr = tw >> 2, total = gpr * th;
    for (int q = threadIdx.x; q < total; q += blockDim.x) {
      const int row = q / gpr, gx = (q - row * gpr) << 2;
      uint32_t* d = reinterpret_cast<uint32_t*>(dst + row * pitch + (size_t)gx * 3);
      if (!src) {
        d[0] = d[1] = d[2] = 0u;
        continue;
      }
      const uint32_t* s = reinterpret_cast<const uint32_t*>(src + ((size_t)row * tw + gx) * 3);
      uint32_t w[3] = {__ldg(s), __ldg(s + 1), __ldg(s + 2)};
      if (adjust) {
        uint32_t o[3] = {0u, 0u, 0u};
#pragma unroll
        for (int px = 0; px < 4; ++px) {
          const int b0 = 3 * px, b1 = b0 + 1, b2 = b0 + 2;
          uint8_t o0, o1, o2;
          adjust_unit(a, s_bc[byte_of(w[b0 >> 2], b0 & 3)], s_bc[byte_of(w[b1 >> 2], b1 & 3)],
                         s_bc[byte_of(w[b2 >> 2], b2 & 3)], o0, o1, o2);
          o[b0 >> 2] |= (uint32_t)o0 << (8 * (b0 & 3));
          o[b1 >> 2] |= (uint32_t)o1 << (8 * (b1 & 3));
          o[b2 >> 2] |= (uint32_t)o2 << (8 * (b2 & 3));
        }
        w[0] = o[0];
        w[1] = o[1];
        w[2] = o[2];
      }
      d[0] = w[0];
      d[1] = w[1];
      d[2] = w[2];
    }
    return;
  }
  const int total = tw * th;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int row = q / tw, x = q - row * tw;
    uint8_t* d = dst + row * pitch + (size_t)x * 3;
    uint8_t o0 = 0, o1 = 0, o2 = 0;
    if (src) {
      const uint8_t* s = src + ((size_t)row * tw + x) * 3;
      o0 = s[0];
      o1 = s[1];
      o2 = s[2];
      if (adjust) adjust_unit(a, s_bc[o0], s_bc[o1], s_bc[o2], o0, o1, o2);
    }
    d[0] = o0;
    d[1] = o1;
    d[2] = o2;
  }
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
