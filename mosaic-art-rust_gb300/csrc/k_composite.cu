// k_composite.cu -- (f) per-cell HSV colour adjustment and compositing of the
// device-resident thumbnails into the output image, in one pass.
//
// Reference: main.rs:548-592 (first composite) and main.rs:627-664 (rebuild
// after the optimiser); color_adjustment.rs:99-154 calculate_optimal_adjustment
// from the thumbnail's mean RGB and the target cell's mean RGB (main.rs:556-563),
// color_adjustment.rs:40-96 apply_to_image / adjust_pixel.  The reference
// composites twice when the optimiser runs and keeps only the second image; the
// device pass composites the final grid once.
//
// Bound: HBM (3*tw*th bytes read + 3*tw*th bytes written per cell) plus the
// per-pixel HSV arithmetic.  One thread per output pixel; each CTA stages the
// byte->[0,1] table (x/255, IEEE division) in shared memory.
#include <algorithm>

#include "composite.cuh"
#include "mg_internal.h"

namespace mg {
namespace {

__global__ void cell_adjust_kernel(const int32_t* __restrict__ grid, int n, const uchar4* __restrict__ thumb_rgb,
                                   const uchar4* __restrict__ cell_rgb, float strength, float4* __restrict__ adj) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int m = grid[c];
  float4 r = make_float4(0.0f, 1.0f, 0.0f, 1.0f);
  if (m >= 0) {
    const uchar4 t = thumb_rgb[m], g = cell_rgb[c];
    const Adjust a = optimal_adjustment(t.x, t.y, t.z, g.x, g.y, g.z, strength);
    r = make_float4(a.brightness, a.contrast, a.hue_shift, a.saturation);
  }
  adj[c] = r;
}

// One CTA per tile (cell), grid-stride over the cells; the brightness/contrast
// table of a tile is built in one of two shared buffers, so one barrier per
// tile orders the build before the lookups and the previous tile's lookups
// before the next build.
template <bool kAdjust>
__global__ void __launch_bounds__(256) composite_kernel(const int32_t* __restrict__ grid, int gw, int gh,
                                                        const uint8_t* __restrict__ thumbs, int tw, int th,
                                                        const float4* __restrict__ adj, uint8_t* __restrict__ out) {
  __shared__ float s_bc[2][256];
  __shared__ uint32_t s_perm[8];
  sector_perm_table(s_perm);
  const int n = gw * gh;
  const size_t pitch = (size_t)gw * tw * 3;
  int it = 0;
  for (int c = blockIdx.x; c < n; c += gridDim.x, ++it) {
    const int m = grid[c];
    float* bc = s_bc[it & 1];
    Adjust a{0.0f, 1.0f, 0.0f, 1.0f};
    if (kAdjust && m >= 0) {
      const float4 a4 = adj[c];
      a = Adjust{a4.x, a4.y, a4.z, a4.w};
      tile_bc_table(bc, a);
    }
    __syncthreads();
    const int cy = c / gw, cx = c - cy * gw;
    uint8_t* dst = out + (size_t)cy * th * pitch + (size_t)cx * tw * 3;
    const uint8_t* src = m >= 0 ? thumbs + (size_t)m * tw * th * 3 : nullptr;
    composite_tile(src, dst, tw, th, pitch, kAdjust, a, bc, s_perm);
  }
}

// apply_to_image: adjust_pixel on every pixel; for adjustments in
// adjustment_new's ranges (and a brightness and contrast that are not NaN,
// so the brightness/contrast table holds channels in [0, 1]) through the
// composite's arithmetic, the table and adjust_word.
__global__ void __launch_bounds__(256) adjust_image_kernel(float4 a4, const uint8_t* __restrict__ in, int w, int h,
                                                           int64_t stride, uint8_t* __restrict__ out) {
  __shared__ float s_unit[256];
  __shared__ uint32_t s_perm[8];
  const Adjust a{a4.x, a4.y, a4.z, a4.w};
  const bool word = adjust_word_applies(a) && a.brightness == a.brightness && a.contrast == a.contrast;
  if (word) s_unit[threadIdx.x] = brightness_contrast(u8_unit(threadIdx.x), a.brightness, a.contrast);
  else s_unit[threadIdx.x] = u8_unit(threadIdx.x);
  sector_perm_table(s_perm);
  __syncthreads();
  const int64_t total = (int64_t)w * h;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(t / w), x = (int)(t - (int64_t)y * w);
    const uint8_t* s = in + (int64_t)y * stride + 3 * x;
    uint8_t* d = out + t * 3;
    if (word) {
      const uint32_t p = adjust_word(a, s_unit[s[0]], s_unit[s[1]], s_unit[s[2]], s_perm);
      d[0] = (uint8_t)p;
      d[1] = (uint8_t)(p >> 8);
      d[2] = (uint8_t)(p >> 16);
      continue;
    }
    uint8_t o0, o1, o2;
    adjust_pixel(a, s_unit[s[0]], s_unit[s[1]], s_unit[s[2]], o0, o1, o2);
    d[0] = o0;
    d[1] = o1;
    d[2] = o2;
  }
}

__global__ void optimal_adjustment_kernel(const uint8_t* __restrict__ tile, const uint8_t* __restrict__ target, int n,
                                          float strength, float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Adjust a = optimal_adjustment(tile[3 * i], tile[3 * i + 1], tile[3 * i + 2], target[3 * i], target[3 * i + 1],
                                      target[3 * i + 2], strength);
  out[i] = make_float4(a.brightness, a.contrast, a.hue_shift, a.saturation);
}

unsigned grid_for(int64_t items) {
  const int64_t blocks = (items + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks, 152 * 32));
}

}  // namespace

int launch_cell_adjust(const int32_t* grid, int n_cells, const uchar4* thumb_rgb, const uchar4* cell_rgb,
                       float strength, float4* adj, cudaStream_t stream) {
  if (n_cells <= 0) return MG_OK;
  cell_adjust_kernel<<<(n_cells + 255) / 256, 256, 0, stream>>>(grid, n_cells, thumb_rgb, cell_rgb, strength, adj);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_composite(const int32_t* grid, int gw, int gh, const uint8_t* thumbs, int tw, int th, const float4* adj,
                     int do_adjust, uint8_t* out, cudaStream_t stream) {
  const int64_t total = (int64_t)gw * tw * gh * th;
  if (total <= 0) return MG_OK;
  int dev = 0, sms = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int cells = gw * gh;
  const unsigned blocks = (unsigned)std::max(1, std::min(cells, sms * 8));
  const int threads = tile_threads(tw, th);
  if (do_adjust) composite_kernel<true><<<blocks, threads, 0, stream>>>(grid, gw, gh, thumbs, tw, th, adj, out);
  else composite_kernel<false><<<blocks, threads, 0, stream>>>(grid, gw, gh, thumbs, tw, th, adj, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_adjust_image(const float4 adj, const uint8_t* in, int w, int h, int64_t stride, uint8_t* out,
                        cudaStream_t stream) {
  const int64_t total = (int64_t)w * h;
  if (total <= 0) return MG_OK;
  adjust_image_kernel<<<grid_for(total), 256, 0, stream>>>(adj, in, w, h, stride, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_optimal_adjustment(const uint8_t* tile_rgb, const uint8_t* target_rgb, int n, float strength, float4* out,
                              cudaStream_t stream) {
  if (n <= 0) return MG_OK;
  optimal_adjustment_kernel<<<(n + 127) / 128, 128, 0, stream>>>(tile_rgb, target_rgb, n, strength, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
