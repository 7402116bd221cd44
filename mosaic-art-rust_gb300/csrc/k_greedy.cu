// k_greedy.cu -- (d) greedy usage-limited, adjacency-penalised placement.
//
// Reference: main.rs:529-545 (row-major walk over the grid), main.rs:335-418
// find_and_use_best_tile_with_position, main.rs:420-475 fallback_tile_selection,
// main.rs:309-333 can_place_at_position, lib.rs:57-89 UsageTracker,
// adjacency.rs:63-88 calculate_penalty.
//
// The walk is sequential within a mosaic (each choice changes the usage counts
// and the left neighbour of the next cell), so one warp walks one mosaic and
// the 32 lanes evaluate the candidate list of a cell in parallel:
//   score = squared Lab distance + weight * (w(up) + w(left)),  w = 1/(sim+1)
// in the reference's order (penalty accumulated up, down, left, right from
// zero, then scaled; down and right are never placed yet in a row-major walk).
// A warp minimum over the 64-bit key (score bits, list position) reproduces the
// reference's strict "<" scan: the first of equal scores wins.  Candidates are
// sorted by distance and the penalty is non-negative, so once the next
// unevaluated distance is >= the best score, no later candidate can win and
// the scan of that cell stops.  Usage counters live in shared memory when the
// palette fits.  The fallback resets every counter (the reference's global
// UsageTracker::reset), then takes the first candidate that passes the
// same-neighbour ban, else the nearest one.
//
// After the walk the same warp evaluates calculate_total_cost of the placed
// grid (adjacency.rs:91-130) as one sequential FP32 sum in the reference's
// order; it is the annealer's initial cost.
#include "mg_internal.h"

namespace mg {
namespace {

__device__ __forceinline__ float wgt(const float4& a, const float4& b) {
  return adj_weight_from_sim(lab_distance(a.x, a.y, a.z, b.x, b.y, b.z));
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t < v ? t : v;
  }
  return v;
}

constexpr unsigned long long kMaxKey = ~0ull;

// Sequential calculate_total_cost of a complete grid by one warp: lanes compute
// the right and down terms of 32 cells, lane order then feeds one FP32
// accumulator (terms of absent neighbours are +0, which leaves the sum as is).
__device__ float warp_total_cost(const float4* __restrict__ pal, const int32_t* grid, int gw, int gh, int lane) {
  float total = 0.0f;
  const int n = gw * gh;
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int c = c0 + lane;
    float tr = 0.0f, td = 0.0f;
    if (c < n) {
      const int x = c % gw, y = c / gw;
      const int cur = grid[c];
      if (cur >= 0) {
        const float4 lc = __ldg(pal + cur);
        if (x < gw - 1) {
          const int r = grid[c + 1];
          if (r >= 0) tr = wgt(lc, __ldg(pal + r));
        }
        if (y < gh - 1) {
          const int d = grid[c + gw];
          if (d >= 0) td = wgt(lc, __ldg(pal + d));
        }
      }
    }
    const int cnt = min(32, n - c0);
    for (int s = 0; s < cnt; ++s) {
      total = __fadd_rn(total, __shfl_sync(0xffffffffu, tr, s));
      total = __fadd_rn(total, __shfl_sync(0xffffffffu, td, s));
    }
  }
  return total;
}

__global__ void __launch_bounds__(32) greedy_kernel(const float4* __restrict__ pal, int p,
                                                    const GreedyJob* __restrict__ jobs, uint32_t* usage_global,
                                                    int smem_usage) {
  extern __shared__ __align__(16) uint8_t smem[];
  const GreedyJob J = jobs[blockIdx.x];
  const int lane = threadIdx.x;
  const int gw = J.gw, gh = J.gh, k = J.k;
  int32_t* s_row = reinterpret_cast<int32_t*>(smem);
  uint32_t* usage = smem_usage ? reinterpret_cast<uint32_t*>(smem + ((gw * 4 + 15) & ~15))
                               : usage_global + (size_t)blockIdx.x * p;
  for (int i = lane; i < p; i += 32) usage[i] = 0;
  __syncwarp();

  int resets = 0;
  int last = -1;
  const float weight = J.weight;
  const bool use_pen = weight > 0.0f;
  for (int y = 0; y < gh; ++y) {
    for (int x = 0; x < gw; ++x) {
      const int c = y * gw + x;
      const int up = y > 0 ? s_row[x] : -1;
      const int left = x > 0 ? last : -1;
      float4 lab_up = make_float4(0.f, 0.f, 0.f, 0.f), lab_left = lab_up;
      if (use_pen) {
        if (up >= 0) lab_up = __ldg(pal + up);
        if (left >= 0) lab_left = __ldg(pal + left);
      }
      const uint32_t* cidx = J.cand_idx + (size_t)c * k;
      const float* cdist = J.cand_dist + (size_t)c * k;
      unsigned long long best = kMaxKey;
      for (int r = 0; r * 32 < k; ++r) {
        const int j = r * 32 + lane;
        unsigned long long key = kMaxKey;
        if (j < k) {
          const int t = (int)cidx[j];
          const float d = cdist[j];
          if (t != up && t != left && usage[t] < J.max_usage) {
            float score;
            if (use_pen) {
              const float4 lt = __ldg(pal + t);
              float pen = 0.0f;
              if (up >= 0) pen = __fadd_rn(pen, wgt(lt, lab_up));
              if (left >= 0) pen = __fadd_rn(pen, wgt(lt, lab_left));
              score = __fadd_rn(d, __fmul_rn(pen, weight));
            } else {
              score = __fadd_rn(d, 0.0f);
            }
            key = ((unsigned long long)__float_as_uint(score) << 32) | (unsigned)j;
          }
        }
        const unsigned long long m = warp_min_u64(key);
        best = m < best ? m : best;
        const int nxt = (r + 1) * 32;
        if (best != kMaxKey && nxt < k && cdist[nxt] >= __uint_as_float((uint32_t)(best >> 32))) break;
      }
      int t;
      if (best != kMaxKey) {
        t = (int)cidx[(uint32_t)best];
        if (lane == 0) usage[t] += 1u;
      } else {
        // main.rs:420-475: global reset, first candidate passing can_place, else nearest.
        ++resets;
        for (int i = lane; i < p; i += 32) usage[i] = 0;
        t = -1;
        for (int r = 0; r * 32 < k && t < 0; ++r) {
          const int j = r * 32 + lane;
          bool ok = false;
          int tj = -1;
          if (j < k) {
            tj = (int)cidx[j];
            ok = tj != up && tj != left;
          }
          const unsigned mask = __ballot_sync(0xffffffffu, ok);
          if (mask) t = __shfl_sync(0xffffffffu, tj, __ffs(mask) - 1);
        }
        if (t < 0) t = (int)cidx[0];
        __syncwarp();
        if (lane == 0) usage[t] = 1u;
      }
      if (lane == 0) {
        J.grid[c] = t;
        s_row[x] = t;
      }
      last = t;
      __syncwarp();
    }
  }
  const float total = warp_total_cost(pal, J.grid, gw, gh, lane);
  if (lane == 0) {
    if (J.n_resets) *J.n_resets = resets;
    if (J.total_cost) *J.total_cost = total;
  }
}

}  // namespace

int launch_greedy(const float4* pal, int p, const GreedyJob* jobs_dev, int n_jobs, uint32_t* usage_scratch,
                  int smem_usage_bytes, cudaStream_t stream) {
  if (n_jobs <= 0) return MG_OK;
  // smem_usage_bytes: bytes of shared memory for the row buffer (+ counters
  // when usage_scratch is null).
  static int configured_device = -1;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    configured_device = dev;
  }
  greedy_kernel<<<n_jobs, 32, smem_usage_bytes, stream>>>(pal, p, jobs_dev, usage_scratch, usage_scratch ? 0 : 1);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
