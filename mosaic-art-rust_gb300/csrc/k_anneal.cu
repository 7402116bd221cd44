// k_anneal.cu -- (e) the standalone annealing kernels (one CTA per chain,
// anneal_cta.cuh; or one warp per chain, anneal_chain.cuh, for grids whose
// state does not fit beside the CTA's round buffers) and the batched adjacency evaluators of the
// C ABI (adjacency.rs:63-214), one thread per item, the reference's loops
// verbatim.
#include "anneal_cta.cuh"

namespace mg {
namespace {
using namespace anneal_detail;

template <bool kLabSmem, int kRound>
__global__ void __launch_bounds__(anneal_cta_detail::kThreads)
    anneal_cta_kernel(const float4* __restrict__ pal, int p, const AnnealJob* __restrict__ jobs,
                      const int* __restrict__ chain_job, const int* __restrict__ chain_id) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int jid = chain_job ? chain_job[blockIdx.x] : 0;
  const int chain = chain_id ? chain_id[blockIdx.x] : (int)blockIdx.x;
  const AnnealJob J = jobs[jid];
  anneal_cta_detail::anneal_chain_cta<kLabSmem, kRound>(pal, p, J, chain, smem);
}

// Grids of at least this many cells take 32 proposals a round.
constexpr int kWideRoundCells = 12000;

template <bool kLabSmem>
__global__ void __launch_bounds__(32) anneal_kernel(const float4* __restrict__ pal, int p,
                                                    const AnnealJob* __restrict__ jobs,
                                                    const int* __restrict__ chain_job,
                                                    const int* __restrict__ chain_id) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int jid = chain_job ? chain_job[blockIdx.x] : 0;
  const int chain = chain_id ? chain_id[blockIdx.x] : (int)blockIdx.x;
  const AnnealJob J = jobs[jid];
  anneal_chain<kLabSmem>(pal, p, J, chain, smem);
}

// Lowest final cost wins (ties: lowest chain); copy its grid.
__global__ void select_best_kernel(const AnnealJob* __restrict__ jobs, int32_t* const* __restrict__ finals,
                                   int* __restrict__ best_chain) {
  __shared__ int s_best;
  const AnnealJob J = jobs[blockIdx.x];
  if (threadIdx.x == 0) {
    int b = J.chains > 0 ? 0 : -1;
    for (int c = 1; c < J.chains; ++c)
      if (J.results[c].final_cost < J.results[b].final_cost) b = c;
    s_best = b;
    if (best_chain) best_chain[blockIdx.x] = b;
  }
  __syncthreads();
  const int n = J.gw * J.gh;
  const int32_t* src = s_best < 0 ? J.grid_in : J.chain_grids + (size_t)s_best * n;
  int32_t* dst = finals[blockIdx.x];
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// ---- batched evaluators (one thread per item, the reference's loops verbatim) ----
__device__ __forceinline__ float wgt_idx(const float4* pal, int a, int b) { return wgt(__ldg(pal + a), __ldg(pal + b)); }

__device__ int adjacent_positions(int x, int y, int gw, int gh, int* nx, int* ny) {
  int n = 0;
  if (y > 0) { nx[n] = x; ny[n] = y - 1; ++n; }
  if (y < gh - 1) { nx[n] = x; ny[n] = y + 1; ++n; }
  if (x > 0) { nx[n] = x - 1; ny[n] = y; ++n; }
  if (x < gw - 1) { nx[n] = x + 1; ny[n] = y; ++n; }
  return n;
}

__global__ void swap_delta_kernel(const float4* __restrict__ pal, const int32_t* __restrict__ grid, int gw, int gh,
                                  const int4* __restrict__ pairs, int n, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 q = pairs[i];
  const int x1 = q.x, y1 = q.y, x2 = q.z, y2 = q.w;
  const int a1 = grid[y1 * gw + x1], a2 = grid[y2 * gw + x2];
  if (a1 < 0 || a2 < 0 || a1 == a2) { out[i] = 0.0f; return; }
  float old_cost = 0.0f, new_cost = 0.0f;
  int nx[4], ny[4];
  bool adj = false;
  int m = adjacent_positions(x1, y1, gw, gh, nx, ny);
  for (int t = 0; t < m; ++t) {
    if (nx[t] == x2 && ny[t] == y2) { adj = true; continue; }
    const int a = grid[ny[t] * gw + nx[t]];
    if (a >= 0) {
      old_cost = __fadd_rn(old_cost, wgt_idx(pal, a1, a));
      new_cost = __fadd_rn(new_cost, wgt_idx(pal, a2, a));
    }
  }
  m = adjacent_positions(x2, y2, gw, gh, nx, ny);
  for (int t = 0; t < m; ++t) {
    if (nx[t] == x1 && ny[t] == y1) continue;
    const int a = grid[ny[t] * gw + nx[t]];
    if (a >= 0) {
      old_cost = __fadd_rn(old_cost, wgt_idx(pal, a2, a));
      new_cost = __fadd_rn(new_cost, wgt_idx(pal, a1, a));
    }
  }
  if (adj) {
    const float c = wgt_idx(pal, a1, a2);
    old_cost = __fadd_rn(old_cost, c);
    new_cost = __fadd_rn(new_cost, c);
  }
  out[i] = __fsub_rn(new_cost, old_cost);
}

__global__ void penalty_kernel(const float4* __restrict__ pal, const int32_t* __restrict__ grid, int gw, int gh,
                               float weight, const int4* __restrict__ cxy, int n, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 q = cxy[i];
  int nx[4], ny[4];
  const int m = adjacent_positions(q.y, q.z, gw, gh, nx, ny);
  float pen = 0.0f;
  for (int t = 0; t < m; ++t) {
    const int a = grid[ny[t] * gw + nx[t]];
    if (a >= 0) pen = __fadd_rn(pen, wgt_idx(pal, q.x, a));
  }
  out[i] = __fmul_rn(pen, weight);
}

__global__ void total_cost_kernel(const float4* __restrict__ pal, const int32_t* __restrict__ grid, int gw, int gh,
                                  float* __restrict__ out) {
  const int lane = threadIdx.x;
  float total = 0.0f;
  const int n = gw * gh;
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int c = c0 + lane;
    float tr = 0.0f, td = 0.0f;
    if (c < n) {
      const int x = c % gw, y = c / gw;
      const int cur = grid[c];
      if (cur >= 0) {
        if (x < gw - 1 && grid[c + 1] >= 0) tr = wgt_idx(pal, cur, grid[c + 1]);
        if (y < gh - 1 && grid[c + gw] >= 0) td = wgt_idx(pal, cur, grid[c + gw]);
      }
    }
    const int cnt = min(32, n - c0);
    for (int s = 0; s < cnt; ++s) {
      total = __fadd_rn(total, __shfl_sync(0xffffffffu, tr, s));
      total = __fadd_rn(total, __shfl_sync(0xffffffffu, td, s));
    }
  }
  if (lane == 0) *out = total;
}

}  // namespace

int launch_anneal(const float4* pal, int p, const AnnealJob* jobs_dev, const int* chain_job_dev,
                  const int* chain_id_dev, int total_chains, int max_cells, cudaStream_t stream, int min_cells) {
  if (total_chains <= 0) return MG_OK;
  if (p >= 65535) return fail(MG_ERR_ARG, "annealing supports palettes below 65535 materials");
  const size_t grid_bytes = kRing * sizeof(int4) + (((size_t)max_cells * 2 + 15) & ~(size_t)15);
  const size_t lab_bytes = (size_t)p * sizeof(float4);
  const size_t kMaxSmem = 200 * 1024;
  if (grid_bytes > kMaxSmem) return fail(MG_ERR_ARG, "grid too large for the annealer (max 102400 cells)");
  static int configured_device = -1;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    MG_CUDA(cudaFuncSetAttribute(anneal_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(anneal_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(anneal_cta_kernel<true, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(anneal_cta_kernel<false, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(anneal_cta_kernel<true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(anneal_cta_kernel<false, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    configured_device = dev;
  }
  // A CTA of several warps per chain (more proposals per round) when it fits.
  {
    using anneal_cta_detail::anneal_cta_smem_bytes;
    const size_t with_lab = anneal_cta_smem_bytes(max_cells, p, true), no_lab = anneal_cta_smem_bytes(max_cells, p, false);
    if (with_lab <= kMaxSmem || no_lab <= kMaxSmem) {
      const bool wide = (min_cells < 0 ? max_cells : min_cells) >= kWideRoundCells;
      const unsigned nt = anneal_cta_detail::kThreads;
      if (with_lab <= kMaxSmem) {
        if (wide)
          anneal_cta_kernel<true, 32><<<total_chains, nt, with_lab, stream>>>(pal, p, jobs_dev, chain_job_dev, chain_id_dev);
        else
          anneal_cta_kernel<true, 16><<<total_chains, nt, with_lab, stream>>>(pal, p, jobs_dev, chain_job_dev, chain_id_dev);
      } else {
        if (wide)
          anneal_cta_kernel<false, 32><<<total_chains, nt, no_lab, stream>>>(pal, p, jobs_dev, chain_job_dev, chain_id_dev);
        else
          anneal_cta_kernel<false, 16><<<total_chains, nt, no_lab, stream>>>(pal, p, jobs_dev, chain_job_dev, chain_id_dev);
      }
      g_launches += 1;
      MG_CUDA(cudaGetLastError());
      return MG_OK;
    }
  }
  if (grid_bytes + lab_bytes <= kMaxSmem)
    anneal_kernel<true><<<total_chains, 32, grid_bytes + lab_bytes, stream>>>(pal, p, jobs_dev, chain_job_dev, chain_id_dev);
  else
    anneal_kernel<false><<<total_chains, 32, grid_bytes, stream>>>(pal, p, jobs_dev, chain_job_dev, chain_id_dev);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_select_best(const AnnealJob* jobs_dev, int n_jobs, int32_t* const* final_grids_dev, int* best_chain_dev,
                       cudaStream_t stream) {
  if (n_jobs <= 0) return MG_OK;
  select_best_kernel<<<n_jobs, 256, 0, stream>>>(jobs_dev, final_grids_dev, best_chain_dev);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_total_cost(const float4* pal, const int32_t* grid, int gw, int gh, float* out, cudaStream_t stream) {
  total_cost_kernel<<<1, 32, 0, stream>>>(pal, grid, gw, gh, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_swap_delta(const float4* pal, const int32_t* grid, int gw, int gh, const int4* pairs, int n, float* out,
                      cudaStream_t stream) {
  if (n <= 0) return MG_OK;
  swap_delta_kernel<<<(n + 127) / 128, 128, 0, stream>>>(pal, grid, gw, gh, pairs, n, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_penalty(const float4* pal, const int32_t* grid, int gw, int gh, float weight, const int4* cxy, int n,
                   float* out, cudaStream_t stream) {
  if (n <= 0) return MG_OK;
  penalty_kernel<<<(n + 127) / 128, 128, 0, stream>>>(pal, grid, gw, gh, weight, cxy, n, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
