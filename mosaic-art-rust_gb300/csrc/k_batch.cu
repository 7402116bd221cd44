// k_batch.cu -- many mosaics of uneven size over one resident palette.
//
// The per-mosaic path (main.rs:477-685 once per target) is sequential inside a
// mosaic -- the greedy walk and each annealing chain -- so a single mosaic
// cannot fill the GPU.  The batch runs the data-parallel stages once over the
// cells of every mosaic (cell statistics, k-nearest, adjustment, composite) and
// runs the sequential stages in one persistent launch whose warps pull work
// items from a device queue:
//   item (walk, m)      the greedy walk of mosaic m; on completion it publishes
//                       the mosaic's K chain items (or its final grid when the
//                       optimiser is off);
//   item (chain, m, c)  annealing chain c of mosaic m; the last chain of a
//                       mosaic to finish picks the lowest final cost (ties: the
//                       lowest chain) and writes the final grid.
// Walk items are queued largest mosaic first, so the longest walks start
// first and short mosaics' chains fill the SMs while they run.  Every wait on
// the queue is bounded (it sets an error word and the warp leaves).  Each item
// is the same code as the single-mosaic kernels (greedy_walk.cuh,
// anneal_chain.cuh), so batched results equal the one-mosaic-per-launch
// results bit for bit.
#include "anneal_chain.cuh"
#include "composite.cuh"
#include "greedy_walk.cuh"

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

__device__ __forceinline__ unsigned long long make_item(unsigned type, unsigned chain, unsigned m) {
  return ((unsigned long long)type << 48) | ((unsigned long long)chain << 32) | m;
}

constexpr unsigned kMaxQueueSpins = 20u * 1000u * 1000u;  // with <= 1 us naps: ~20 s at most

// Persistent walk + chain workers, kWorkers warps per CTA, each with its own
// shared-memory slice of worker_smem bytes.
template <bool kLabSmem, int kWorkers>
__global__ void __launch_bounds__(32 * kWorkers) batch_place_kernel(const float4* __restrict__ pal, int p,
                                                                    const BatchMosaic* __restrict__ mos, BatchQueue q,
                                                                    int k, size_t worker_smem, uint32_t* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint8_t* my = smem + (size_t)w * worker_smem;
  for (;;) {
    unsigned slot = 0;
    if (lane == 0) slot = atomicAdd(q.head, 1u);
    slot = __shfl_sync(0xffffffffu, slot, 0);
    if (slot >= q.total) break;
    unsigned long long item = 0;
    int ok = 1;
    if (lane == 0) {
      unsigned spins = 0, nap = 32;
      while (((volatile unsigned*)q.ready)[slot] == 0u) {
        __nanosleep(nap);
        nap = nap < 1024 ? nap * 2 : 1024;
        if (++spins > kMaxQueueSpins) {
          ok = 0;
          break;
        }
      }
      __threadfence();
      item = ((volatile unsigned long long*)q.items)[slot];
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) {
      if (lane == 0) atomicOr(err, kErrTimeout);
      break;
    }
    item = __shfl_sync(0xffffffffu, item, 0);
    const unsigned type = (unsigned)(item >> 48);
    const int chain = (int)((item >> 32) & 0xFFFFu);
    const int m = (int)(item & 0xFFFFFFFFu);
    const BatchMosaic& M = mos[m];
    if (type == 0) {
      GreedyJob J{q.cand_idx + (size_t)M.cell_base * k, q.cand_dist + (size_t)M.cell_base * k, M.grid, M.gw, M.gh, k,
                  M.max_usage, M.weight, M.n_resets, M.init_cost};
      greedy_detail::greedy_walk<kLabSmem, true>(pal, p, J, my, nullptr, err);
      __syncwarp();
      if (M.run_sa && M.chains > 0) {
        if (lane == 0) {
          __threadfence();  // the grid and initial cost before the chain items
          const unsigned base = atomicAdd(q.tail, (unsigned)M.chains);
          for (int c = 0; c < M.chains; ++c) q.items[base + c] = make_item(1u, (unsigned)c, (unsigned)m);
          __threadfence();
          for (int c = 0; c < M.chains; ++c) atomicExch(q.ready + base + c, 1u);
        }
      } else {
        for (int i = lane; i < M.n; i += 32) M.final_grid[i] = M.grid[i];
        if (lane == 0) *M.best_chain = -1;
      }
    } else {
      AnnealJob J{};
      J.grid_in = M.grid;
      J.chain_grids = M.chain_grids;
      J.results = M.results;
      J.initial_cost = M.init_cost;
      J.gw = M.gw;
      J.gh = M.gh;
      J.chains = M.chains;
      J.iters = M.iters;
      J.t0 = M.t0;
      J.decay = M.decay;
      J.key0 = M.key0;
      J.key1 = M.key1;
      J.stream = M.stream;
      J.greedy_only = 0;
      anneal_detail::anneal_chain<kLabSmem>(pal, p, J, chain, my);
      __syncwarp();
      unsigned left = 0;
      if (lane == 0) {
        __threadfence();
        left = atomicSub(q.chains_left + m, 1u);
      }
      left = __shfl_sync(0xffffffffu, left, 0);
      if (left == 1u) {  // last chain of the mosaic: pick the best
        __threadfence();
        int b = 0;
        if (lane == 0) {
          float bf = __ldcg(&M.results[0].final_cost);
          for (int c = 1; c < M.chains; ++c) {
            const float f = __ldcg(&M.results[c].final_cost);
            if (f < bf) {
              bf = f;
              b = c;
            }
          }
          *M.best_chain = b;
        }
        b = __shfl_sync(0xffffffffu, b, 0);
        const int32_t* src = M.chain_grids + (size_t)b * M.n;
        for (int i = lane; i < M.n; i += 32) M.final_grid[i] = __ldcg(src + i);
      }
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

namespace {
__global__ void fill_u32_kernel(unsigned* p, unsigned n, unsigned v) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = v;
}
}  // namespace

int launch_fill_u32(unsigned* p, unsigned n, unsigned v, cudaStream_t stream) {
  if (n == 0) return MG_OK;
  fill_u32_kernel<<<std::min((n + 255) / 256, 1024u), 256, 0, stream>>>(p, n, v);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

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

size_t batch_worker_smem(int k, int max_gw, int max_cells, int p, bool lab_smem) {
  const size_t g = greedy_detail::greedy_smem_bytes(k, max_gw, p, lab_smem, true);
  const size_t a = anneal_detail::anneal_smem_bytes(max_cells, p, lab_smem);
  return ((g > a ? g : a) + 127) & ~(size_t)127;
}

int launch_batch_place(const float4* pal, int p, const BatchMosaic* mos, const BatchQueue& q, int k, int max_gw,
                       int max_cells, int workers, uint32_t* err, cudaStream_t stream) {
  constexpr size_t kMaxSmem = 227 * 1024;
  bool lab_smem = true;
  size_t ws = batch_worker_smem(k, max_gw, max_cells, p, true);
  if (ws * workers > kMaxSmem) {
    lab_smem = false;
    ws = batch_worker_smem(k, max_gw, max_cells, p, false);
  }
  while (workers > 1 && ws * workers > kMaxSmem) workers >>= 1;
  if (ws * workers > kMaxSmem) return fail(MG_ERR_ARG, "a mosaic of this batch is too large for one worker");
  const size_t bytes = ws * workers;
  int dev = 0, sms = 0, per_sm = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  auto go = [&](auto kernel) -> int {
    MG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * workers, bytes));
    if (per_sm < 1) return fail(MG_ERR_ARG, "batch worker does not fit on an SM");
    const int grid = (int)std::min<long long>((long long)sms * per_sm, ((long long)q.total + workers - 1) / workers);
    kernel<<<std::max(grid, 1), 32 * workers, bytes, stream>>>(pal, p, mos, q, k, ws, err);
    g_launches += 1;
    MG_CUDA(cudaGetLastError());
    return MG_OK;
  };
  if (lab_smem) {
    if (workers == 4) return go(batch_place_kernel<true, 4>);
    if (workers == 2) return go(batch_place_kernel<true, 2>);
    return go(batch_place_kernel<true, 1>);
  }
  if (workers == 4) return go(batch_place_kernel<false, 4>);
  if (workers == 2) return go(batch_place_kernel<false, 2>);
  return go(batch_place_kernel<false, 1>);
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
