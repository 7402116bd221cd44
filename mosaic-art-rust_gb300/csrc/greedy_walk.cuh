// greedy_walk.cuh -- the greedy placement walk of one mosaic by one warp
// (greedy_kernel in k_greedy.cu: palettes above 65535, grids narrower than 8
// cells, walks whose scouted form does not fit in shared memory).
//
// k_greedy.cu -- (d) greedy usage-limited, adjacency-penalised placement.
//
// Reference: main.rs:529-545 (row-major walk over the grid), main.rs:335-418
// find_and_use_best_tile_with_position, main.rs:420-475 fallback_tile_selection,
// main.rs:309-333 can_place_at_position, lib.rs:57-89 UsageTracker,
// adjacency.rs:63-88 calculate_penalty.
//
// The reference scores every candidate of a cell (the min(P,100) nearest, in
// ascending squared distance) that passes the usage cap and the same-neighbour
// ban as
//   score = distance + weight * penalty,  penalty = w(up) + w(left) accumulated
//   from zero in up, down, left, right order (down and right are never placed
//   yet in a row-major walk), w = 1/(sim+1),
// and keeps the first strict minimum.  The walk is sequential within a mosaic,
// so one warp walks one mosaic and its lanes hold one candidate each per round
// of 32 list positions.  Two exact observations make most cells cheap:
//  - every w is in (0, 1], so the penalty is in [0, 2] and
//    score(e0) <= d(e0) + 2*weight for the first eligible candidate e0, while
//    score(t) >= d(t) for every t: only eligible candidates after e0 with
//    d < fl(d(e0) + fl(2*weight)) can beat e0.  When there is none (more than
//    99% of cells on the measured workloads) e0 wins and no penalty is
//    evaluated; otherwise the exact scores of e0 and that window are compared
//    (key: score bits, then list position).
//  - rounds after the first are loaded only when no eligible candidate was
//    found earlier in the list.
// Nothing on a cell's path touches global memory: candidate rows are streamed
// into shared memory 16 cells per TMA bulk copy, four stages ahead; usage
// counters and the palette Lab sit in shared memory; the first round of the
// next cell is loaded before the current cell's decision (its commit changes
// one usage counter, that of its choice, which the next decision re-checks).
// The fallback resets every counter (the reference's global
// UsageTracker::reset), then takes the first candidate that passes the
// same-neighbour ban, else the nearest one.
//
// After the walk the same warp evaluates calculate_total_cost of the placed
// grid (adjacency.rs:91-130) as one sequential FP32 sum in the reference's
// order; it is the annealer's initial cost.
#pragma once
#include "mg_internal.h"
#include "mg_ptx.cuh"

namespace mg {
namespace greedy_detail {

constexpr int kStageCells = 16;  // cells per TMA stage (candidate rows are k entries each)
constexpr int kStageBufs = 4;    // stages in flight
constexpr uint32_t kNoCand = 0xFFFFFFFFu;

__device__ __forceinline__ float wgt(const float4& a, const float4& b) {
  return __frcp_rn(__fadd_rn(lab_distance(a.x, a.y, a.z, b.x, b.y, b.z), 1.0f));
}

// Sequential calculate_total_cost of a complete grid by one warp: lanes compute
// the right and down terms of 32 cells, lane order then feeds one FP32
// accumulator (terms of absent neighbours are +0, which leaves the sum as is).
template <class LabFn>
__device__ float warp_total_cost(LabFn lab, const int32_t* grid, int gw, int gh, int lane) {
  float total = 0.0f;
  const int n = gw * gh;
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int c = c0 + lane;
    float tr = 0.0f, td = 0.0f;
    if (c < n) {
      const int x = c % gw, y = c / gw;
      const int cur = grid[c];
      if (cur >= 0) {
        const float4 lc = lab(cur);
        if (x < gw - 1) {
          const int r = grid[c + 1];
          if (r >= 0) tr = wgt(lc, lab(r));
        }
        if (y < gh - 1) {
          const int d = grid[c + gw];
          if (d >= 0) td = wgt(lc, lab(d));
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

__host__ __device__ inline size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

__host__ __device__ inline size_t greedy_smem_bytes(int k, int gw, int p, bool lab_smem, bool usage_smem) {
  size_t b = 8 * kStageBufs;
  b += 2 * align16((size_t)kStageCells * k * 4) * kStageBufs;
  b += align16((size_t)gw * 4);
  if (lab_smem) b += (size_t)p * 16;
  if (usage_smem) b += align16((size_t)p * 4);
  return b;
}

// One mosaic's walk by one warp.  smem: greedy_smem_bytes(k, gw, p, kLabSmem,
// kUsageSmem) bytes, 128-byte aligned; usage_slot: p counters in global memory
// (used when kUsageSmem is false).
template <bool kLabSmem, bool kUsageSmem>
__device__ __forceinline__ void greedy_walk(const float4* __restrict__ pal, int p, const GreedyJob& J, uint8_t* smem,
                                            uint32_t* usage_slot, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const int gw = J.gw, gh = J.gh, k = J.k, n = gw * gh;
  const size_t stage_elems = align16((size_t)kStageCells * k * 4) / 4;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  uint32_t* cidx_buf = reinterpret_cast<uint32_t*>(smem + 8 * kStageBufs);
  float* cdist_buf = reinterpret_cast<float*>(cidx_buf + kStageBufs * stage_elems);
  int32_t* row = reinterpret_cast<int32_t*>(cdist_buf + kStageBufs * stage_elems);
  float4* s_lab = reinterpret_cast<float4*>(reinterpret_cast<uint8_t*>(row) + align16((size_t)gw * 4));
  uint32_t* s_usage = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(s_lab) + (kLabSmem ? (size_t)p * 16 : 0));
  uint32_t* usage = kUsageSmem ? s_usage : usage_slot;
  if (kLabSmem)
    for (int i = lane; i < p; i += 32) s_lab[i] = pal[i];
  for (int i = lane; i < p; i += 32) usage[i] = 0;
  auto lab = [=](int i) -> float4 { return kLabSmem ? s_lab[i] : __ldg(pal + i); };

  // Candidate rows of cells [s*16, s*16+16) live in buffer s%4 (its s/4-th use,
  // hence barrier parity (s/4)&1).  The arrays are padded to a multiple of 16
  // rows, so a stage is one bulk copy of 16*k*4 bytes per array.
  const int nstages = (n + kStageCells - 1) / kStageCells;
  const uint32_t stage_copy = (uint32_t)(kStageCells * k * 4);
  auto issue = [=](int s) {
    const int b = s % kStageBufs;
    mbar_arrive_expect_tx(&bars[b], 2 * stage_copy);
    tma_load_1d(cidx_buf + b * stage_elems, J.cand_idx + (size_t)s * kStageCells * k, stage_copy, &bars[b]);
    tma_load_1d(cdist_buf + b * stage_elems, J.cand_dist + (size_t)s * kStageCells * k, stage_copy, &bars[b]);
  };
  if (lane == 0) {
    for (int b = 0; b < kStageBufs; ++b) mbar_init(&bars[b], 1);
    mbar_fence_init();
  }
  __syncwarp();
  if (lane == 0)
    for (int s = 0; s < kStageBufs && s < nstages; ++s) issue(s);
  int waited = -1;
  bool aborted = false;
  auto row_ptr = [&](int c, const uint32_t*& ci, const float*& cd) {
    const int s = c / kStageCells;
    if (s > waited) {
      if (!aborted && !mbar_spin_bounded(&bars[s % kStageBufs], (uint32_t)((s / kStageBufs) & 1))) {
        if (lane == 0) atomicOr(err, kErrTimeout);
        aborted = true;
      }
      waited = s;
    }
    const size_t off = (size_t)(s % kStageBufs) * stage_elems + (size_t)(c - s * kStageCells) * k;
    ci = cidx_buf + off;
    cd = cdist_buf + off;
  };

  const uint32_t max_usage = J.max_usage;
  const float weight = J.weight;
  const bool use_pen = weight > 0.0f;
  const float two_w = __fmul_rn(2.0f, weight);
  int resets = 0, last = -1;
  // Round 0 of the current cell: candidate t0, distance d0, eligibility ignoring left.
  uint32_t t0 = kNoCand;
  float d0 = 0.0f;
  bool ok0 = false;
  auto load_round0 = [&](int c, int up) {
    const uint32_t* ci;
    const float* cd;
    row_ptr(c, ci, cd);
    t0 = kNoCand;
    d0 = __int_as_float(0x7f800000);
    ok0 = false;
    if (lane < k) {
      t0 = ci[lane];
      d0 = cd[lane];
      ok0 = (int)t0 != up && usage[t0] < max_usage;
    }
  };
  if (n > 0) load_round0(0, -1);
  int x = 0, y = 0;
  for (int c = 0; c < n && !aborted; ++c) {
    const int left = x > 0 ? last : -1;
    const int up = y > 0 ? row[x] : -1;
    const int xn = x + 1 == gw ? 0 : x + 1, yn = x + 1 == gw ? y + 1 : y;
    const bool has_next = c + 1 < n;
    const int up_next = (has_next && yn > 0) ? row[xn] : -1;  // committed unless gw == 1
    // The previous choice is this cell's left neighbour except at a row start;
    // its usage may have reached the cap after this cell's round 0 was loaded.
    const bool prev_full = last >= 0 && usage[last] >= max_usage;
    auto elig = [&](uint32_t t, bool ok) { return ok && (int)t != left && !(prev_full && (int)t == last); };

    // ---- first eligible candidate, lazily round by round
    uint32_t tr = t0;
    float dr = d0;
    unsigned m = __ballot_sync(0xffffffffu, elig(t0, ok0));
    int r = 0;
    const uint32_t* ci;
    const float* cd;
    row_ptr(c, ci, cd);
    while (!m && (r + 1) * 32 < k) {
      ++r;
      const int j = r * 32 + lane;
      tr = kNoCand;
      dr = __int_as_float(0x7f800000);
      bool ok = false;
      if (j < k) {
        tr = ci[j];
        dr = cd[j];
        ok = (int)tr != up && usage[tr] < max_usage;
      }
      m = __ballot_sync(0xffffffffu, elig(tr, ok));
    }
    // The next cell's round 0 goes out before this cell's commit.
    if (has_next && gw > 1) load_round0(c + 1, up_next);

    int t;
    if (m) {
      const int e0l = __ffs(m) - 1;
      const int e0 = r * 32 + e0l;
      int win = e0;
      if (use_pen) {
        const float b0 = __fadd_rn(__shfl_sync(0xffffffffu, dr, e0l), two_w);
        const unsigned wm = m & __ballot_sync(0xffffffffu, dr < b0) & ~((2u << e0l) - 1u);
        const bool spill = (r + 1) * 32 < k && __shfl_sync(0xffffffffu, dr, 31) < b0;
        if (wm || spill) {
          // Exact scores of e0 and every eligible candidate after it with d < b0.
          const float4 lab_up = up >= 0 ? lab(up) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float4 lab_left = left >= 0 ? lab(left) : make_float4(0.f, 0.f, 0.f, 0.f);
          uint32_t best_s = 0xFFFFFFFFu;
          for (int rr = r; rr * 32 < k; ++rr) {
            const int j = rr * 32 + lane;
            uint32_t tj = kNoCand;
            float dj = __int_as_float(0x7f800000);
            if (j < k) {
              tj = ci[j];
              dj = cd[j];
            }
            const bool okj = j < k && (int)tj != up && usage[tj] < max_usage;
            const bool in = j >= e0 && dj < b0 && elig(tj, okj);
            uint32_t sb = 0xFFFFFFFFu;
            if (in) {
              const float4 lt = lab((int)tj);
              float pen = 0.0f;
              if (up >= 0) pen = __fadd_rn(pen, wgt(lt, lab_up));
              if (left >= 0) pen = __fadd_rn(pen, wgt(lt, lab_left));
              sb = __float_as_uint(__fadd_rn(dj, __fmul_rn(pen, weight)));
            }
            const uint32_t mn = __reduce_min_sync(0xffffffffu, sb);
            if (mn < best_s) {
              best_s = mn;
              win = rr * 32 + __ffs(__ballot_sync(0xffffffffu, sb == mn)) - 1;
            }
            if (!__any_sync(0xffffffffu, dj < b0)) break;  // later rounds have larger d
          }
        }
      }
      t = (int)ci[win];
      if (lane == 0) usage[t] += 1u;
    } else {
      // main.rs:420-475: global reset, first candidate passing can_place, else nearest.
      ++resets;
      for (int i = lane; i < p; i += 32) usage[i] = 0;
      t = -1;
      for (int rr = 0; rr * 32 < k && t < 0; ++rr) {
        const int j = rr * 32 + lane;
        int tj = -1;
        if (j < k) tj = (int)ci[j];
        const unsigned mask = __ballot_sync(0xffffffffu, j < k && tj != up && tj != left);
        if (mask) t = __shfl_sync(0xffffffffu, tj, __ffs(mask) - 1);
      }
      if (t < 0) t = (int)ci[0];
      __syncwarp();
      if (lane == 0) usage[t] = 1u;
    }
    if (lane == 0) {
      J.grid[c] = t;
      row[x] = t;
    }
    last = t;
    __syncwarp();
    if (has_next && (gw == 1 || !m)) load_round0(c + 1, gw == 1 ? t : up_next);
    // After the last cell of a stage its buffer is free for stage s+4.
    if ((c + 1) % kStageCells == 0 || c + 1 == n) {
      const int s = c / kStageCells;
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0 && s + kStageBufs < nstages) issue(s + kStageBufs);
    }
    x = xn;
    y = yn;
  }
  if (aborted) {
    // Give in-flight copies a bounded chance to land before the CTA exits, and
    // leave every cell empty so the stages after the walk read no stale index.
    for (int b = 0; b < kStageBufs; ++b) mbar_wait_bounded(&bars[b], 0, 1u << 16);
    for (int i = lane; i < n; i += 32) J.grid[i] = -1;
    if (lane == 0 && J.n_resets) *J.n_resets = 0;
    return;
  }
  __syncwarp();
  const float total = warp_total_cost(lab, J.grid, gw, gh, lane);
  if (lane == 0) {
    if (J.n_resets) *J.n_resets = resets;
    if (J.total_cost) *J.total_cost = total;
  }
}

}  // namespace greedy_detail
}  // namespace mg
