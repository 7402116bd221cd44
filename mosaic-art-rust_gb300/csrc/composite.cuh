// composite.cuh -- the composite's inner step, shared by the single-mosaic
// kernel (k_composite.cu) and the batch kernel (k_batch.cu): four consecutive
// output pixels of one tile row (main.rs:583-592 copies the adjusted tile into
// the output; color_adjustment.rs:53-87 adjust_pixel on each pixel).
//
// With tile widths a multiple of 4 the four pixels lie in one tile, and their
// 12 bytes are 4-byte aligned in both the thumbnail and the output, so they
// move as three 32-bit words instead of twelve bytes.
#pragma once
#include "mg_internal.h"

namespace mg {

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int i) { return (w >> (8 * i)) & 0xFFu; }

__device__ __forceinline__ void composite_group4(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                                 bool do_adj, const Adjust& a, const float* unit) {
  const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
  uint32_t w[3] = {__ldg(s), __ldg(s + 1), __ldg(s + 2)};
  if (do_adj) {
    uint32_t o[3] = {0u, 0u, 0u};
#pragma unroll
    for (int px = 0; px < 4; ++px) {
      const int b0 = 3 * px, b1 = b0 + 1, b2 = b0 + 2;
      const uint32_t r = byte_of(w[b0 >> 2], b0 & 3), g = byte_of(w[b1 >> 2], b1 & 3), b = byte_of(w[b2 >> 2], b2 & 3);
      uint8_t o0, o1, o2;
      adjust_pixel(a, unit[r], unit[g], unit[b], o0, o1, o2);
      o[b0 >> 2] |= (uint32_t)o0 << (8 * (b0 & 3));
      o[b1 >> 2] |= (uint32_t)o1 << (8 * (b1 & 3));
      o[b2 >> 2] |= (uint32_t)o2 << (8 * (b2 & 3));
    }
    w[0] = o[0];
    w[1] = o[1];
    w[2] = o[2];
  }
  uint32_t* d = reinterpret_cast<uint32_t*>(dst);
  d[0] = w[0];
  d[1] = w[1];
  d[2] = w[2];
}

}  // namespace mg
