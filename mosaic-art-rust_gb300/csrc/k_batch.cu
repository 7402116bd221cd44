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
#include "composite.cuh"
#include "lab_reduce.cuh"

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

constexpr int kCellBaseSmem = 1024;  // mosaics whose first cells the cell kernel keeps in shared memory

// One warp per (padded) cell of any mosaic: the cell's rows through
// lab_reduce.cuh (exact fixed-point Lab and integer RGB sums, reduced by
// shuffles), means written by lane 0.  Padding cells get 0.  Each CTA loads the
// transfer table and (for batches of up to 1024 mosaics) the mosaics' first
// cell indices into shared memory once, so finding a cell's mosaic is a
// binary search on chip.
template <int kWarps>
__global__ void __launch_bounds__(32 * kWarps) batch_cells_kernel(const BatchMosaic* __restrict__ mos, int nm,
                                                                  int total_cells, const LabConsts* __restrict__ C,
                                                                  float4* __restrict__ lab_out,
                                                                  uchar4* __restrict__ rgb_out) {
  __shared__ float s_lut[256];
  __shared__ int s_base[kCellBaseSmem];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s_lut[i] = C->lut[i];
  const bool base_in_smem = nm <= kCellBaseSmem;
  if (base_in_smem)
    for (int i = threadIdx.x; i < nm; i += blockDim.x) s_base[i] = mos[i].cell_base;
  __syncthreads();
  const LabK K = make_lab_k(C->ms, C->eps, C->k1, C->k2);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int cell = blockIdx.x * kWarps + warp; cell < total_cells; cell += gridDim.x * kWarps) {
    int m;
    if (base_in_smem) {
      int lo = 0, hi = nm - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_base[mid] <= cell) lo = mid;
        else hi = mid - 1;
      }
      m = lo;
    } else {
      m = find_mosaic(mos, nm, cell);
    }
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
    LabAcc acc;
    reduce_rows<true>(base, M.cw, M.stride, 0, M.ch, lane, s_lut, K, acc);
    const LabSums t = warp_sums<true>(acc);
    if (lane == 0) {
      const long long npx = (long long)M.cw * M.ch;
      const unsigned long long n = (unsigned long long)npx;
      lab_out[cell] = make_float4(lab_mean(t.L, npx), lab_mean(t.A, npx), lab_mean(t.B, npx), 0.0f);
      rgb_out[cell] = make_uchar4((unsigned char)(t.R / n), (unsigned char)(t.G / n), (unsigned char)(t.Bc / n), 0);
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

// One CTA per tile (cell) of any mosaic; CTA b takes a contiguous run of the
// flat cell index, so its mosaic is found once and then advanced.  Tables of
// tiles alternate between two shared buffers (one barrier per tile, taken by
// every CTA thread on every pass, padding cells included).
__global__ void __launch_bounds__(256) batch_composite_kernel(const BatchMosaic* __restrict__ mos, int nm,
                                                              int total_cells, const uint8_t* __restrict__ thumbs,
                                                              int tw, int th, const float4* __restrict__ adj) {
  __shared__ float s_bc[2][256];
  __shared__ uint32_t s_perm[8];
  sector_perm_table(s_perm);
  const int per = (total_cells + gridDim.x - 1) / gridDim.x;
  const int c0 = blockIdx.x * per, c1 = min(total_cells, c0 + per);
  int mi = c0 < c1 ? find_mosaic(mos, nm, c0) : 0;
  int it = 0;
  for (int c = c0; c < c1; ++c, ++it) {
    while (mi + 1 < nm && mos[mi + 1].cell_base <= c) ++mi;
    const BatchMosaic& M = mos[mi];
    const int local = c - M.cell_base;
    const bool real = local < M.n;  // else a padding cell
    const int g = real ? M.final_grid[local] : -1;
    const bool adjust = M.strength > 0.0f;
    float* bc = s_bc[it & 1];
    Adjust a{0.0f, 1.0f, 0.0f, 1.0f};
    if (adjust && g >= 0) {
      const float4 a4 = adj[c];
      a = Adjust{a4.x, a4.y, a4.z, a4.w};
      tile_bc_table(bc, a);
    }
    __syncthreads();
    if (!real) continue;
    const size_t pitch = (size_t)M.gw * tw * 3;
    const int cy = local / M.gw, cx = local - cy * M.gw;
    uint8_t* dst = M.out + (size_t)cy * th * pitch + (size_t)cx * tw * 3;
    const uint8_t* src = g >= 0 ? thumbs + (size_t)g * tw * th * 3 : nullptr;
    composite_tile(src, dst, tw, th, pitch, adjust, a, bc, s_perm);
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
                        const uchar4* cell_rgb, float4* adj, const uint8_t* thumbs, int tw, int th, cudaStream_t stream) {
  if (nm <= 0) return MG_OK;
  batch_adjust_kernel<<<(total_cells + 255) / 256, 256, 0, stream>>>(mos, nm, total_cells, thumb_rgb, cell_rgb, adj);
  int dev = 0, sms = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = std::max(1, std::min(total_cells, sms * 8));
  batch_composite_kernel<<<blocks, tile_threads(tw, th), 0, stream>>>(mos, nm, total_cells, thumbs, tw, th, adj);
  g_launches += 2;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
