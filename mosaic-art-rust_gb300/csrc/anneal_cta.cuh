// anneal_cta.cuh -- one simulated-annealing chain by one CTA of kChainWarps
// warps (anneal_cta_kernel, for single mosaics and for every chain of a batch;
// the one-warp chain of anneal_chain.cuh, whose rules this follows exactly, is
// the fallback when the CTA form does not fit in shared memory).
//
// Reference: optimizer.rs:41-129 MosaicOptimizer::optimize, optimizer.rs:132-198
// optimize_greedy, adjacency.rs:133-214 calculate_swap_delta.
//
// A chain is a sequence of dependent swaps, and a single proposal is a long
// dependent chain of instructions, so a round evaluates kRound consecutive
// proposals at once (eight lanes each, as in anneal_chain.cuh) on the same grid
// and commits them in order, up to the first proposal that reads a cell within
// Manhattan distance 1 of an earlier accepted swap of the round; the next round
// re-evaluates that one on the updated grid.  Per round:
//  1. every group evaluates its proposal: skip flag, delta (the reference's
//     summation order), and publishes them with its positions;
//  2. after one barrier every warp derives the same round outcome redundantly:
//     lanes 0..kRound-1 take one proposal each -- its temperature (the chain's T
//     times the decay once per earlier non-skipped proposal of the round,
//     multiplied step by step), its acceptance (this library's exp), then the
//     earlier-accepted-neighbour test over all pairs (lanes split the pairs,
//     one OR reduction) -- and every thread runs the in-order commit
//     bookkeeping (running cost, best, counters, temperature);
//  3. the groups of committed accepted proposals swap their two cells; a
//     second barrier ends the round.
// Whether a proposal is skipped does not depend on the grid (swaps never move
// empty cells), so step 2 needs nothing from the commit itself.  Random
// numbers: the same counter-based Philox stream as anneal_chain.cuh (a CPU
// replay of the stream makes the same decisions); every thread of the CTA
// decodes one proposal per refill of a shared ring.
#pragma once
#include "anneal_chain.cuh"

namespace mg {
namespace anneal_cta_detail {
using anneal_detail::kNone16;
using anneal_detail::wgt;

constexpr int kChainWarps = 4;
constexpr int kThreads = kChainWarps * 32;
// Proposals per round: 16 (eight lanes each, one neighbour term a lane) or,
// on large grids, where two proposals of a round rarely touch, 32 (four lanes
// each, two terms a lane): about as long a round, nearly twice the swaps.
constexpr int kRoundMax = 32;
constexpr int kCtaRing = 4 * kThreads;   // decoded proposals in shared memory

struct RoundSlot {  // one proposal's outcome of step 1
  float delta;
  float u;              // acceptance uniform
  uint32_t flags;       // bit 0: skipped
  uint32_t pos1, pos2;  // x | y << 16
  uint32_t pad[3];
};

__host__ __device__ inline size_t anneal_cta_smem_bytes(int max_cells, int p, bool lab_smem) {
  return (size_t)kCtaRing * 16 + (size_t)kRoundMax * sizeof(RoundSlot) + (lab_smem ? (size_t)p * 16 : 0) +
         (((size_t)max_cells * 2 + 15) & ~(size_t)15);
}

template <bool kLabSmem, int kRound>
__device__ __forceinline__ void anneal_chain_cta(const float4* __restrict__ pal, int p, const AnnealJob& J, int chain,
                                                 uint8_t* smem) {
  static_assert(kRound == 16 || kRound == 32, "16 or 32 proposals a round");
  constexpr int kL = kThreads / kRound;  // lanes per proposal: 8 or 4
  constexpr int kT = 8 / kL;             // neighbour terms per lane: 1 or 2
  constexpr int kConfPerWarp = (kRound - 1 + kChainWarps - 1) / kChainWarps;  // conflict tests per warp
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gw = J.gw, gh = J.gh, n = gw * gh;
  __shared__ unsigned s_conf[kChainWarps];  // written after the round's first barrier, read after the second
  int4* s_ring = reinterpret_cast<int4*>(smem);
  RoundSlot* s_round = reinterpret_cast<RoundSlot*>(smem + (size_t)kCtaRing * 16);
  float4* s_lab = reinterpret_cast<float4*>(smem + (size_t)kCtaRing * 16 + (size_t)kRoundMax * sizeof(RoundSlot));
  uint16_t* s_grid = reinterpret_cast<uint16_t*>(reinterpret_cast<uint8_t*>(s_lab) +
                                                 (kLabSmem ? (size_t)p * sizeof(float4) : 0));
  if (kLabSmem)
    for (int i = tid; i < p; i += kThreads) s_lab[i] = pal[i];
  for (int i = tid; i < n; i += kThreads) {
    const int g = __ldcg(J.grid_in + i);
    s_grid[i] = g < 0 ? kNone16 : (uint16_t)g;
  }
  __syncthreads();
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
  const int grp = lane / kL, slot = lane % kL, leader = grp * kL;
  const int q_mine = warp * (32 / kL) + grp;  // this group's proposal within the round

  long long it = 0, filled = 0;
  while (it < iters) {
    // ---- refill the ring (uniform condition) ---------------------------------------
    if (filled < iters && filled - it < kRound) {
      const long long my = filled + tid;
      if (my < iters) {
        const uint32_t hi = (uint32_t)((unsigned long long)my >> 32);
        const u32x4 a = philox((uint32_t)my, (uint32_t)chain, strm, 2u * hi, k0, k1);
        const u32x4 b = philox((uint32_t)my, (uint32_t)chain, strm, 2u * hi + 1u, k0, k1);
        const uint32_t x1 = range_u32(a.x, (uint32_t)gw), y1 = range_u32(a.y, (uint32_t)gh);
        const uint32_t x2 = range_u32(a.z, (uint32_t)gw), y2 = range_u32(a.w, (uint32_t)gh);
        s_ring[my & (kCtaRing - 1)] = make_int4((int)(x1 | (y1 << 16)), (int)(x2 | (y2 << 16)),
                                                __float_as_int(unit_f32(b.x)), 0);
      }
      filled += kThreads;
      __syncthreads();
    }
    // ---- 1. evaluate proposal it + q_mine ------------------------------------------------
    // Branch-free: every lane of a group computes two weights on clamped
    // operands and keeps what its slot needs (lanes 0-3: neighbours of pos1 in
    // up, down, left, right order; 4-7: those of pos2).
    const long long i = it + q_mine;
    const bool live = i < iters;
    const int4 e = s_ring[(live ? i : it) & (kCtaRing - 1)];
    const int x1 = e.x & 0xFFFF, y1 = (e.x >> 16) & 0xFFFF, x2 = e.y & 0xFFFF, y2 = (e.y >> 16) & 0xFFFF;
    const int p1 = y1 * gw + x1, p2 = y2 * gw + x2;
    const uint16_t g1 = s_grid[p1], g2 = s_grid[p2];
    const bool skip = !live || p1 == p2 || g1 == kNone16 || g2 == kNone16;
    const bool same = g1 == g2;
    float old_cost = 0.0f, new_cost = 0.0f, m0 = 0.0f;
    if constexpr (kT == 1) {
      const bool first = slot < 4;
      const int dir = slot & 3;
      const int bx = first ? x1 : x2, by = first ? y1 : y2;
      const int nx = bx + (dir == 2 ? -1 : (dir == 3 ? 1 : 0)), ny = by + (dir == 0 ? -1 : (dir == 1 ? 1 : 0));
      const bool inb = nx >= 0 && nx < gw && ny >= 0 && ny < gh;
      const int nb = inb ? ny * gw + nx : p1;
      const bool mutual = inb && nb == (first ? p2 : p1);
      const uint16_t an = s_grid[nb];
      const bool work = !skip && !same && inb;
      const bool nbr = work && !mutual && an != kNone16;  // a placed neighbour
      const uint16_t gs1 = skip ? (uint16_t)0 : g1, gs2 = skip ? (uint16_t)0 : g2;
      const uint16_t c_idx = mutual ? gs2 : (an != kNone16 ? an : gs1);
      const float4 la1 = lab(gs1), la2 = lab(gs2), lc = lab(c_idx);
      const float w1 = wgt(la1, lc), w2 = wgt(la2, lc);
      const float o = nbr ? (first ? w1 : w2) : 0.0f;
      const float nw = nbr ? (first ? w2 : w1) : 0.0f;
      m0 = (work && mutual && first) ? w1 : 0.0f;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        old_cost = __fadd_rn(old_cost, __shfl_sync(0xffffffffu, o, leader + t));
        new_cost = __fadd_rn(new_cost, __shfl_sync(0xffffffffu, nw, leader + t));
      }
    } else {
      const uint16_t gs1 = skip ? (uint16_t)0 : g1, gs2 = skip ? (uint16_t)0 : g2;
      const float4 la1 = lab(gs1), la2 = lab(gs2);
      // this lane's terms t = slot + kL * tt (0-3: neighbours of pos1 in up, down,
      // left, right order; 4-7: those of pos2)
      float o[kT], nw[kT], m[kT];
#pragma unroll
      for (int tt = 0; tt < kT; ++tt) {
        const int t = slot + kL * tt;
        const bool first = t < 4;
        const int dir = t & 3;
        const int bx = first ? x1 : x2, by = first ? y1 : y2;
        const int nx = bx + (dir == 2 ? -1 : (dir == 3 ? 1 : 0)), ny = by + (dir == 0 ? -1 : (dir == 1 ? 1 : 0));
        const bool inb = nx >= 0 && nx < gw && ny >= 0 && ny < gh;
        const int nb = inb ? ny * gw + nx : p1;
        const bool mutual = inb && nb == (first ? p2 : p1);
        const uint16_t an = s_grid[nb];
        const bool work = !skip && !same && inb;
        const bool nbr = work && !mutual && an != kNone16;  // a placed neighbour
        const uint16_t c_idx = mutual ? gs2 : (an != kNone16 ? an : gs1);
        const float4 lc = lab(c_idx);
        const float w1 = wgt(la1, lc), w2 = wgt(la2, lc);
        o[tt] = nbr ? (first ? w1 : w2) : 0.0f;
        nw[tt] = nbr ? (first ? w2 : w1) : 0.0f;
        m[tt] = (work && mutual && first) ? w1 : 0.0f;
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        old_cost = __fadd_rn(old_cost, __shfl_sync(0xffffffffu, o[t / kL], leader + t % kL));
        new_cost = __fadd_rn(new_cost, __shfl_sync(0xffffffffu, nw[t / kL], leader + t % kL));
      }
      m0 = m[0];
    }
    const int dx = x2 - x1, dy = y2 - y1;
    const bool adjacent = (dx == 0 && (dy == 1 || dy == -1)) || (dy == 0 && (dx == 1 || dx == -1));
    const int dir12 = dy == -1 ? 0 : (dy == 1 ? 1 : (dx == -1 ? 2 : 3));
    const float mm = __shfl_sync(0xffffffffu, m0, leader + dir12);  // term dir12 < 4 sits in lane dir12's first term
    if (adjacent) {
      old_cost = __fadd_rn(old_cost, mm);
      new_cost = __fadd_rn(new_cost, mm);
    }
    const float delta = same ? 0.0f : __fsub_rn(new_cost, old_cost);
    if (slot == 0) {
      RoundSlot& r = s_round[q_mine];
      r.delta = delta;
      r.u = __int_as_float(e.z);
      r.flags = skip ? 1u : 0u;
      r.pos1 = (uint32_t)e.x;
      r.pos2 = (uint32_t)e.y;
    }
    __syncthreads();

    // ---- 2. the round's outcome, derived identically by every warp -------------------------
    // lane q < kRound holds proposal q (lanes kRound.. duplicate lane q - kRound)
    const int q = lane & (kRound - 1);
    const RoundSlot rq = s_round[q];
    const bool skip_q = rq.flags & 1u;
    const unsigned live_mask = __ballot_sync(0xffffffffu, lane < kRound && !skip_q);  // bit q: not skipped
    // The temperatures T_k (the chain's T after k more coolings, multiplied step
    // by step); lane k keeps T_k.
    // (T_kRound, wanted when every proposal of a 32-proposal round cools, is
    // held by every lane as t_last: there is no lane 32)
    float t_lane = temp, t_last = temp;
    if (!greedy_only) {
      float tk = temp;
#pragma unroll
      for (int kk = 1; kk <= kRound; ++kk) {
        tk = __fmul_rn(tk, decay);
        if (kk == lane) t_lane = tk;
      }
      t_last = tk;
    }
    bool acc_q = false;
    {
      const int before = __popc(live_mask & ((1u << q) - 1u));
      const float t_q = __shfl_sync(0xffffffffu, t_lane, before);
      if (!skip_q) {
        if (greedy_only) acc_q = rq.delta < 0.0f;
        else acc_q = rq.delta < 0.0f || rq.u < exp_spec(__fdiv_rn(-rq.delta, t_q));
      }
    }
    const unsigned acc_mask = __ballot_sync(0xffffffffu, lane < kRound && acc_q);
    // proposal q reads a cell within distance 1 of an earlier accepted swap?
    // (branch-free: Manhattan distances of the four position pairs).  The
    // earlier proposals h are split over the warps -- warp w tests
    // h in [w * kConfPerWarp, (w + 1) * kConfPerWarp) for every q -- and the
    // warps' conflict masks are ORed through shared memory.
    const int qx1 = (int)(rq.pos1 & 0xFFFFu), qy1 = (int)(rq.pos1 >> 16);
    const int qx2 = (int)(rq.pos2 & 0xFFFFu), qy2 = (int)(rq.pos2 >> 16);
    unsigned conf_bits = 0u;
#pragma unroll
    for (int j = 0; j < kConfPerWarp; ++j) {
      const int h = warp * kConfPerWarp + j;
      const uint32_t hp1 = __shfl_sync(0xffffffffu, rq.pos1, h & 31), hp2 = __shfl_sync(0xffffffffu, rq.pos2, h & 31);
      const int hx1 = (int)(hp1 & 0xFFFFu), hy1 = (int)(hp1 >> 16), hx2 = (int)(hp2 & 0xFFFFu), hy2 = (int)(hp2 >> 16);
      const unsigned hit = (unsigned)(abs(hx1 - qx1) + abs(hy1 - qy1) <= 1) | (unsigned)(abs(hx1 - qx2) + abs(hy1 - qy2) <= 1) |
                           (unsigned)(abs(hx2 - qx1) + abs(hy2 - qy1) <= 1) | (unsigned)(abs(hx2 - qx2) + abs(hy2 - qy2) <= 1);
      conf_bits |= hit & (acc_mask >> (h & 31)) & (unsigned)(h < q);
    }
    const unsigned part = __ballot_sync(0xffffffffu, lane < kRound && (conf_bits & 1u) != 0u);
    if (lane == 0) s_conf[warp] = part;
    __syncthreads();
    unsigned conf_mask = 0u;
#pragma unroll
    for (int w = 0; w < kChainWarps; ++w) conf_mask |= s_conf[w];
    const unsigned cmask = conf_mask & live_mask;
    const int gc = cmask ? __ffs(cmask) - 1 : kRound;  // >= 1: proposal 0 never conflicts
    const int ncommit = (int)min((long long)gc, iters - it);
    const unsigned commit = ncommit >= 32 ? 0xFFFFFFFFu : (1u << ncommit) - 1u;
    // in-order bookkeeping (every thread, identical values)
#pragma unroll
    for (int h = 0; h < kRound; ++h) {
      const float dh = __shfl_sync(0xffffffffu, rq.delta, h);
      const bool a = ((acc_mask & commit) >> h) & 1u;
      const float nc = __fadd_rn(current, dh);
      current = a ? nc : current;
      const bool imp = a && current < best;
      best = imp ? current : best;
      improved += imp ? 1 : 0;
    }
    accepted += __popc(acc_mask & commit);
    const int ncool = __popc(live_mask & commit);  // skipped proposals do not cool
    cooled += ncool;
    if (!greedy_only) {
      const float t_n = __shfl_sync(0xffffffffu, t_lane, ncool & 31);
      temp = ncool == 32 ? t_last : t_n;
    }
    // ---- 3. committed accepted swaps -------------------------------------------------------
    if (slot == 0 && q_mine < ncommit && ((acc_mask >> q_mine) & 1u)) {
      s_grid[p1] = g2;
      s_grid[p2] = g1;
    }
    it += ncommit;
    __syncthreads();
  }
  int32_t* out = J.chain_grids + (size_t)chain * n;
  for (int i = tid; i < n; i += kThreads) {
    const uint16_t g = s_grid[i];
    out[i] = g == kNone16 ? -1 : (int32_t)g;
  }
  if (tid == 0) {
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

}  // namespace anneal_cta_detail
}  // namespace mg
