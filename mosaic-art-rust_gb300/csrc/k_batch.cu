// k_batch.cu -- many mosaics of uneven size over one resident palette.
//
// The per-mosaic path (main.rs:477-685 once per target) is sequential inside a
// mosaic -- the greedy walk and each annealing chain -- so a single mosaic
// cannot fill the GPU.  The batch runs the data-parallel stages once over the
// cells of every mosaic (cell statistics and k-nearest here and in k_scan.cu /
// k_nearest_grid.cu, adjustment and composite here), every greedy walk in one
// launch of the walk kernels (k_greedy.cu: one three-CTA cluster per mosaic,
// largest mosaic first), every annealing chain of every mosaic in one launch
// of the chain kernel (k_anneal.cu: one CTA per chain) and one best-chain
// selection per mosaic.  Each walk and chain is the single-mosaic code, so
// batched results equal the one-mosaic-per-launch results bit for bit.
#include "mg_internal.h"
#include "composite.cuh"

namespace mg {
namespace {

__device__ __forceinline__ int find_mosaic(const BatchMosaic* __restrict__ mos, int nm, int cell) {
  int lo = 0, hi = nm - 1;
  while (lo < hi) {  // last mosaic whose cell_base <= cell
    const int mid = (lo + hi + 1) >> 1;
    if (mos[mid].cell_base <= cell) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// One warp per (padded) cell of any mosaic: exact fixed-point Lab sums and u32
// RGB sums over the cell's pixels, reduced by shuffles.  Padding cells get 0.
template <int kWarps>
__global__ void __launch_bounds__(32 * kWarps) batch_cells_kernel(const BatchMosaic* __restrict__ mos, int nm,
                                                                  int total_cells, const LabConsts* __restrict__ C,
                                                                  float4* __restrict__ lab_out,
                                                                  uchar4* __restrict__ rgb_out) {
  __shared__ float s_lut[256];
  __shared__ float s_ms[9];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s_lut[i] = C->lut[i];
  if (threadIdx.x < 9) s_ms[threadIdx.x] = C->ms[threadIdx.x];
  __syncthreads();
  const float eps = C->eps, k1 = C->k1, k2 = C->k2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int cell = blockIdx.x * kWarps + warp; cell < total_cells; cell += gridDim.x * kWarps) {
    const int m = find_mosaic(mos, nm, cell);
    const BatchMosaic& M = mos[m];
    const int local = cell - M.cell_base;
    if (local >= M.n) {
      if (lane == 0) {
        lab_out[cell] = make_float4(0.f, 0.f, 0.f, 0.f);
        rgb_out[cell] = make_uchar4(0, 0, 0, 0);
      }
      continue;
    }
    const int cy = local / M.gw, cx = local - cy * M.gw;
    const uint8_t* base = M.target + (int64_t)cy * M.ch * M.stride + 3ll * cx * M.cw;
    const int npx = M.cw * M.ch;
    long long aL = 0, aA = 0, aB = 0;
    unsigned sr = 0, sg = 0, sb = 0;
    int x = lane % M.cw, y = lane / M.cw;
    const int dx = 32 % M.cw, dy = 32 / M.cw;
    for (int i = lane; i < npx; i += 32) {
      const uint8_t* px = base + (int64_t)y * M.stride + 3 * x;
      const uint32_t r8 = px[0], g8 = px[1], b8 = px[2];
      sr += r8;
      sg += g8;
      sb += b8;
      float L, A, B;
      lab_pixel(s_lut, s_ms, eps, k1, k2, r8, g8, b8, L, A, B);
      aL += lab_quant(L);
      aA += lab_quant(A);
      aB += lab_quant(B);
      x += dx;
      y += dy;
      if (x >= M.cw) {
        x -= M.cw;
        ++y;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      aL += __shfl_xor_sync(0xffffffffu, aL, o);
      aA += __shfl_xor_sync(0xffffffffu, aA, o);
      aB += __shfl_xor_sync(0xffffffffu, aB, o);
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      sg += __shfl_xor_sync(0xffffffffu, sg, o);
      sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    if (lane == 0) {
      lab_out[cell] = make_float4(lab_mean(aL, npx), lab_mean(aA, npx), lab_mean(aB, npx), 0.0f);
      rgb_out[cell] = make_uchar4((unsigned char)(sr / (unsigned)npx), (unsigned char)(sg / (unsigned)npx),
                                  (unsigned char)(sb / (unsigned)npx), 0);
    }
  }
}

__global__ void batch_adjust_kernel(const BatchMosaic* __restrict__ mos, int nm, int total_cells,
                                    const uchar4* __restrict__ thumb_rgb, const uchar4* __restrict__ cell_rgb,
                                    float4* __restrict__ adj) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= total_cells) return;
  const int m = find_mosaic(mos, nm, cell);
  const BatchMosaic& M = mos[m];
  const int local = cell - M.cell_base;
  float4 r = make_float4(0.0f, 1.0f, 0.0f, 1.0f);
  if (local < M.n && M.strength > 0.0f) {
    const int g = M.final_grid[local];
    if (g >= 0) {
      const uchar4 t = thumb_rgb[g], c = cell_rgb[cell];
      const Adjust a = optimal_adjustment(t.x, t.y, t.z, c.x, c.y, c.z, M.strength);
      r = make_float4(a.brightness, a.contrast, a.hue_shift, a.saturation);
    }
  }
  adj[cell] = r;
}

// blockIdx.y = mosaic; a grid-stride loop over its output pixels, four per
// thread when the tile width allows (composite.cuh).
__global__ void __launch_bounds__(256) batch_composite_kernel(const BatchMosaic* __restrict__ mos,
                                                              const uint8_t* __restrict__ thumbs, int tw, int th,
                                                              const float4* __restrict__ adj) {
  __shared__ float s_unit[256];
  s_unit[threadIdx.x] = u8_unit(threadIdx.x);
  __syncthreads();
  const BatchMosaic& M = mos[blockIdx.y];
  const int ow = M.gw * tw, oh = M.gh * th;
  const bool do_adj = M.strength > 0.0f;
  if ((tw & 3) == 0) {
    const int gpr = ow >> 2, total = gpr * oh;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
      const int oy = q / gpr, ox = (q - oy * gpr) << 2;
      const int cy = oy / th, cx = ox / tw;
      const int local = cy * M.gw + cx;
      const int g = M.final_grid[local];
      uint8_t* d = M.out + ((size_t)oy * ow + ox) * 3;
      if (g < 0) {
        uint32_t* dw = reinterpret_cast<uint32_t*>(d);
        dw[0] = dw[1] = dw[2] = 0u;
        continue;
      }
      const uint8_t* src = thumbs + (((size_t)g * th + (oy - cy * th)) * tw + (ox - cx * tw)) * 3;
      Adjust a{0.0f, 1.0f, 0.0f, 1.0f};
      if (do_adj) {
        const float4 a4 = adj[M.cell_base + local];
        a = Adjust{a4.x, a4.y, a4.z, a4.w};
      }
      composite_group4(src, d, do_adj, a, s_unit);
    }
    return;
  }
  const int64_t total = (int64_t)ow * oh;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int oy = (int)(t / ow), ox = (int)(t - (int64_t)oy * ow);
    const int cy = oy / th, cx = ox / tw;
    const int local = cy * M.gw + cx;
    const int g = M.final_grid[local];
    uint8_t o0 = 0, o1 = 0, o2 = 0;
    if (g >= 0) {
      const uint8_t* s = thumbs + ((size_t)g * th * tw + (size_t)(oy - cy * th) * tw + (ox - cx * tw)) * 3;
      o0 = s[0];
      o1 = s[1];
      o2 = s[2];
      if (do_adj) {
        const float4 a4 = adj[M.cell_base + local];
        const Adjust a{a4.x, a4.y, a4.z, a4.w};
        adjust_pixel(a, s_unit[o0], s_unit[o1], s_unit[o2], o0, o1, o2);
      }
    }
    uint8_t* d = M.out + t * 3;
    d[0] = o0;
    d[1] = o1;
    d[2] = o2;
  }
}

}  // namespace

int launch_batch_cells(const BatchMosaic* mos, int nm, int total_cells, const LabConsts* consts, float4* lab,
                       uchar4* rgb, int warps, cudaStream_t stream) {
  if (total_cells <= 0) return MG_OK;
  const int grid = std::min((total_cells + 7) / 8, 152 * 64);
  if (warps == 4)
    batch_cells_kernel<4><<<std::min((total_cells + 3) / 4, 152 * 64), 128, 0, stream>>>(mos, nm, total_cells, consts, lab, rgb);
  else
    batch_cells_kernel<8><<<grid, 256, 0, stream>>>(mos, nm, total_cells, consts, lab, rgb);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_batch_finish(const BatchMosaic* mos, int nm, int total_cells, const uchar4* thumb_rgb,
                        const uchar4* cell_rgb, float4* adj, const uint8_t* thumbs, int tw, int th, int max_out_px,
                        cudaStream_t stream) {
  if (nm <= 0) return MG_OK;
  batch_adjust_kernel<<<(total_cells + 255) / 256, 256, 0, stream>>>(mos, nm, total_cells, thumb_rgb, cell_rgb, adj);
  const int bx = std::max(1, std::min(((tw & 3) == 0 ? max_out_px / 4 : max_out_px) / 256 + 1, 256));
  batch_composite_kernel<<<dim3(bx, nm), 256, 0, stream>>>(mos, thumbs, tw, th, adj);
  g_launches += 2;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
