// anneal_chain.cuh -- one simulated-annealing chain by one warp (anneal_kernel
// in k_anneal.cu, the fallback of the CTA form of anneal_cta.cuh).
//
// k_anneal.cu -- (e) simulated annealing, K independent chains per mosaic,
// plus the batched adjacency evaluators of the C ABI.
//
// Reference: optimizer.rs:41-129 MosaicOptimizer::optimize (and
// optimizer.rs:132-198 optimize_greedy), adjacency.rs:91-130
// calculate_total_cost, adjacency.rs:133-214 calculate_swap_delta,
// adjacency.rs:63-88 calculate_penalty.
//
// One CTA (one warp) per chain.  The chain's grid lives in shared memory as
// 16-bit palette indices, and the palette Lab too when it fits, so a proposal
// touches no global memory.  Random numbers are counter-based: at iteration t
// of chain c, Philox4x32-10 with key (seed lo, seed hi) and counter
// (t, c, stream, 2*(t>>32)) gives x1, y1, x2, y2 (multiply-high range
// reduction) and counter (t, c, stream, 2*(t>>32)+1) gives the acceptance
// uniform, so a CPU replay of the same stream makes the same decisions.  The
// lanes fill a 64-entry ring of decoded proposals 32 at a time.
//
// A chain is sequential, and one proposal alone is a long dependent chain of
// instructions, so the warp evaluates kGroups = 4 consecutive proposals at once
// (8 lanes each: lanes 0-3 the up/down/left/right neighbours of pos1, 4-7 those
// of pos2; the lane whose pos1 neighbour is pos2 supplies the mutual term) on
// the same grid, and then commits them in order.  This is exact:
//  - a proposal reads only pos1, pos2 and their neighbours, so its delta equals
//    the sequential one unless an earlier proposal of the same round swapped one
//    of those cells; the commit stops at the first proposal whose read cells lie
//    within Manhattan distance 1 of an earlier accepted swap, and the next round
//    re-evaluates it on the updated grid;
//  - whether an iteration is skipped (pos1 == pos2 or an empty cell) does not
//    depend on the grid's state (swaps never move empty cells), so the
//    temperature of each proposal in the round -- T multiplied by the decay once
//    per earlier non-skipped iteration, as in the reference -- is known before
//    the commit, and so is the acceptance decision;
//  - the costs are accumulated in the reference's order (old and new sums over
//    the neighbour slots in order, the mutual term last; delta = new - old; the
//    running cost += delta per accepted swap, in iteration order).
// The acceptance test uses this library's own exp, identical on host and
// device.
#pragma once
#include "mg_internal.h"

namespace mg {
namespace anneal_detail {

constexpr uint16_t kNone16 = 0xFFFFu;
constexpr int kGroups = 4;     // proposals evaluated per round
constexpr int kRing = 64;      // decoded proposals kept in shared memory

__device__ __forceinline__ float wgt(const float4& a, const float4& b) {
  // 1/(sim+1): the correctly rounded reciprocal equals the correctly rounded 1.0/x.
  return __frcp_rn(__fadd_rn(lab_distance(a.x, a.y, a.z, b.x, b.y, b.z), 1.0f));
}


__host__ __device__ inline size_t anneal_smem_bytes(int max_cells, int p, bool lab_smem) {
  return kRing * 16 + (lab_smem ? (size_t)p * 16 : 0) + (((size_t)max_cells * 2 + 15) & ~(size_t)15);
}

// One chain by one warp.  smem: anneal_smem_bytes(n, p, kLabSmem) bytes,
// 16-byte aligned.
template <bool kLabSmem>
__device__ __forceinline__ void anneal_chain(const float4* __restrict__ pal, int p, const AnnealJob& J, int chain,
                                             uint8_t* smem) {
  const int lane = threadIdx.x & 31;
  const int gw = J.gw, gh = J.gh, n = gw * gh;
  int4* s_ring = reinterpret_cast<int4*>(smem);
  float4* s_lab = reinterpret_cast<float4*>(smem + kRing * sizeof(int4));
  uint16_t* s_grid =
      reinterpret_cast<uint16_t*>(smem + kRing * sizeof(int4) + (kLabSmem ? (size_t)p * sizeof(float4) : 0));
  if (kLabSmem)
    for (int i = lane; i < p; i += 32) s_lab[i] = pal[i];
  for (int i = lane; i < n; i += 32) {
    const int g = __ldcg(J.grid_in + i);  // may come from another SM in the same launch
    s_grid[i] = g < 0 ? kNone16 : (uint16_t)g;
  }
  __syncwarp();
  auto lab = [&](int i) -> float4 { return kLabSmem ? s_lab[i] : __ldg(pal + i); };

  // Initial cost: calculate_total_cost of the start grid (sequential FP32 sum).
  float current;
  if (J.initial_cost) {
    current = __ldcg(J.initial_cost);
  } else {
    current = 0.0f;
    for (int c0 = 0; c0 < n; c0 += 32) {
      const int c = c0 + lane;
      float tr = 0.0f, td = 0.0f;
      if (c < n) {
        const int x = c % gw, y = c / gw;
        const uint16_t cur = s_grid[c];
        if (cur != kNone16) {
          const float4 lc = lab(cur);
          if (x < gw - 1 && s_grid[c + 1] != kNone16) tr = wgt(lc, lab(s_grid[c + 1]));
          if (y < gh - 1 && s_grid[c + gw] != kNone16) td = wgt(lc, lab(s_grid[c + gw]));
        }
      }
      const int cnt = min(32, n - c0);
      for (int s = 0; s < cnt; ++s) {
        current = __fadd_rn(current, __shfl_sync(0xffffffffu, tr, s));
        current = __fadd_rn(current, __shfl_sync(0xffffffffu, td, s));
      }
    }
  }
  const float initial = current;
  float best = current;
  long long accepted = 0, improved = 0, cooled = 0;
  float temp = J.t0;
  const float decay = J.decay;
  const bool greedy_only = J.greedy_only != 0;
  const uint32_t k0 = J.key0, k1 = J.key1, strm = J.stream;
  const long long iters = J.iters;
  const int grp = lane >> 3, slot = lane & 7;
  const int leader = grp << 3;

  long long it = 0, filled = 0;
  while (it < iters) {
    if (filled < iters && filled - it < kGroups) {
      const long long my = filled + lane;
      if (my < iters) {
        const uint32_t hi = (uint32_t)((unsigned long long)my >> 32);
        const u32x4 a = philox((uint32_t)my, (uint32_t)chain, strm, 2u * hi, k0, k1);
        const u32x4 b = philox((uint32_t)my, (uint32_t)chain, strm, 2u * hi + 1u, k0, k1);
        const uint32_t x1 = range_u32(a.x, (uint32_t)gw), y1 = range_u32(a.y, (uint32_t)gh);
        const uint32_t x2 = range_u32(a.z, (uint32_t)gw), y2 = range_u32(a.w, (uint32_t)gh);
        s_ring[my & (kRing - 1)] = make_int4((int)(x1 | (y1 << 16)), (int)(x2 | (y2 << 16)),
                                             __float_as_int(unit_f32(b.x)), 0);
      }
      filled += 32;
      __syncwarp();
    }
    // ---- evaluate proposal it + grp --------------------------------------------------
    const long long i = it + grp;
    const bool live = i < iters;
    int4 e = make_int4(0, 0, 0, 0);
    if (live) e = s_ring[i & (kRing - 1)];
    const int x1 = e.x & 0xFFFF, y1 = (e.x >> 16) & 0xFFFF, x2 = e.y & 0xFFFF, y2 = (e.y >> 16) & 0xFFFF;
    const float u = __int_as_float(e.z);
    const int p1 = y1 * gw + x1, p2 = y2 * gw + x2;
    bool skip = !live || p1 == p2;
    uint16_t g1 = 0, g2 = 0;
    if (!skip) {
      g1 = s_grid[p1];
      g2 = s_grid[p2];
      skip = g1 == kNone16 || g2 == kNone16;
    }
    const bool same = g1 == g2;
    float o = 0.0f, nw = 0.0f, m = 0.0f;
    if (!skip && !same) {
      const bool first = slot < 4;
      const int bx = first ? x1 : x2, by = first ? y1 : y2;
      const int other = first ? p2 : p1;
      const int dir = slot & 3;
      int nx = bx, ny = by;
      bool inb;
      if (dir == 0) { ny = by - 1; inb = by > 0; }
      else if (dir == 1) { ny = by + 1; inb = by < gh - 1; }
      else if (dir == 2) { nx = bx - 1; inb = bx > 0; }
      else { nx = bx + 1; inb = bx < gw - 1; }
      if (inb) {
        const int nb = ny * gw + nx;
        if (nb == other) {
          if (first) m = wgt(lab(g1), lab(g2));
        } else {
          const uint16_t a = s_grid[nb];
          if (a != kNone16) {
            const float4 la = lab(a);
            const float w1 = wgt(lab(g1), la), w2 = wgt(lab(g2), la);
            o = first ? w1 : w2;
            nw = first ? w2 : w1;
          }
        }
      }
    }
    float old_cost = 0.0f, new_cost = 0.0f;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      old_cost = __fadd_rn(old_cost, __shfl_sync(0xffffffffu, o, leader + t));
      new_cost = __fadd_rn(new_cost, __shfl_sync(0xffffffffu, nw, leader + t));
    }
    const int dx = x2 - x1, dy = y2 - y1;
    const bool adjacent = (dx == 0 && (dy == 1 || dy == -1)) || (dy == 0 && (dx == 1 || dx == -1));
    const int dir12 = dy == -1 ? 0 : (dy == 1 ? 1 : (dx == -1 ? 2 : 3));
    const float mm = __shfl_sync(0xffffffffu, m, leader + dir12);
    if (adjacent) {
      old_cost = __fadd_rn(old_cost, mm);
      new_cost = __fadd_rn(new_cost, mm);
    }
    const float delta = same ? 0.0f : __fsub_rn(new_cost, old_cost);
    // temperature of this proposal: one decay per earlier non-skipped proposal of the round
    const unsigned live_mask = __ballot_sync(0xffffffffu, slot == 0 && !skip);
    float t_i = temp;
    if (!greedy_only) {
      const int before = __popc(live_mask & ((1u << leader) - 1u));
      for (int q = 0; q < before; ++q) t_i = __fmul_rn(t_i, decay);
    }
    bool acc = false;
    if (!skip) {
      if (greedy_only) acc = delta < 0.0f;
      else acc = delta < 0.0f || u < exp_spec(__fdiv_rn(-delta, t_i));
    }
    // ---- commit in order, up to the first proposal that reads an earlier accepted swap --------
    const unsigned acc_mask = __ballot_sync(0xffffffffu, slot == 0 && acc);
    bool conflict = false;
#pragma unroll
    for (int h = 0; h < kGroups - 1; ++h) {
      const int hx1 = __shfl_sync(0xffffffffu, x1, h * 8), hy1 = __shfl_sync(0xffffffffu, y1, h * 8);
      const int hx2 = __shfl_sync(0xffffffffu, x2, h * 8), hy2 = __shfl_sync(0xffffffffu, y2, h * 8);
      if (h < grp && ((acc_mask >> (h * 8)) & 1u)) {
        const bool near = abs(hx1 - x1) + abs(hy1 - y1) <= 1 || abs(hx1 - x2) + abs(hy1 - y2) <= 1 ||
                          abs(hx2 - x1) + abs(hy2 - y1) <= 1 || abs(hx2 - x2) + abs(hy2 - y2) <= 1;
        conflict = conflict || near;
      }
    }
    const unsigned cmask = __ballot_sync(0xffffffffu, slot == 0 && live && !skip && conflict);
    const int gc = cmask ? ((__ffs(cmask) - 1) >> 3) : kGroups;  // >= 1: group 0 never conflicts
    const long long remaining = iters - it;
    const int ncommit = (int)min((long long)gc, remaining);
    for (int h = 0; h < ncommit; ++h) {
      const float dh = __shfl_sync(0xffffffffu, delta, h * 8);
      if (!((live_mask >> (h * 8)) & 1u)) continue;  // skipped: no cooling
      if ((acc_mask >> (h * 8)) & 1u) {
        current = __fadd_rn(current, dh);
        ++accepted;
        if (current < best) {
          best = current;
          ++improved;
        }
      }
      if (!greedy_only) temp = __fmul_rn(temp, decay);
      ++cooled;
    }
    if (slot == 0 && grp < ncommit && acc) {
      s_grid[p1] = g2;
      s_grid[p2] = g1;
    }
    it += ncommit;
    __syncwarp();
  }
  int32_t* out = J.chain_grids + (size_t)chain * n;
  for (int i = lane; i < n; i += 32) {
    const uint16_t g = s_grid[i];
    out[i] = g == kNone16 ? -1 : (int32_t)g;
  }
  if (lane == 0) {
    ChainResult r;
    r.initial_cost = initial;
    r.final_cost = current;
    r.best_cost = greedy_only ? current : best;
    r.pad = 0.0f;
    r.accepted = accepted;
    r.improved = greedy_only ? accepted : improved;
    r.cooled = cooled;
    r.pad2 = 0;
    J.results[chain] = r;
  }
}

}  // namespace anneal_detail
}  // namespace mg
