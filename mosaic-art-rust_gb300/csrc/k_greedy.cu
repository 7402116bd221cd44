// k_greedy.cu -- (d) the standalone greedy placement kernels.
//
// Reference: main.rs:529-545 (row-major walk), main.rs:335-418
// find_and_use_best_tile_with_position, main.rs:420-475 fallback_tile_selection,
// main.rs:309-333 can_place_at_position, lib.rs:57-89 UsageTracker,
// adjacency.rs:63-88 calculate_penalty.  The decision rule and its exact
// shortcuts are described in greedy_walk.cuh.
//
// Two kernels:
//  - greedy_kernel: one warp walks one mosaic (greedy_walk.cuh).  Used for
//    palettes whose counters do not fit in shared memory and for grids narrower
//    than 8 cells.
//  - greedy_scout_kernel: one 16-warp CTA per mosaic.  The walk is a chain of
//    dependent decisions, so its speed is the latency of one decision.  Warp 0
//    (the walker) makes the decisions; twelve scout warps, on the other three
//    SM sub-partitions, prepare each cell's decision ahead of the walker from a
//    snapshot of the usage counters:
//      e0', e1'  the first two candidates (list order) that pass the usage cap
//                and differ from the cell above, in the snapshot;
//      clear     whether no later such candidate lies inside the 2*weight
//                window of e0' (resp. e1'), i.e. whether the penalty cannot
//                change the decision.
//    Counters only grow between resets, so a candidate that fails the cap in
//    the snapshot still fails it when the walker arrives, and the walker's
//    first eligible candidate is e0' if e0' still passes (fresh counter, left
//    neighbour), else e1' if that passes.  With `clear` set that candidate is
//    the reference's choice, bit for bit; in every other case (window not
//    clear, both fail, no candidate, a reset since the snapshot) the walker
//    evaluates the cell in full, exactly as greedy_walk does.  A scout reads
//    the cell above only after the walker has committed it (acquire/release
//    on a progress counter) and a reset bumps an epoch that invalidates older
//    snapshots.  The walker's fast path is a few shared-memory loads per cell.
#include "greedy_walk.cuh"

namespace mg {
namespace {
using namespace greedy_detail;

template <bool kLabSmem, bool kUsageSmem>
__global__ void __launch_bounds__(32) greedy_kernel(const float4* __restrict__ pal, int p,
                                                    const GreedyJob* __restrict__ jobs, uint32_t* usage_global,
                                                    uint32_t* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  const GreedyJob J = jobs[blockIdx.x];
  greedy_walk<kLabSmem, kUsageSmem>(pal, p, J, smem, usage_global ? usage_global + (size_t)blockIdx.x * p : nullptr,
                                    err);
}

// ---- the scouted walk -------------------------------------------------------------------
constexpr int kScoutWarps = 16;  // warp 0 walks; warps w with w % 4 != 0 scout
constexpr int kScouts = 12;
constexpr uint32_t kInvalidEpoch = 0xFFFFFFFFu;
constexpr uint32_t kWalkPolls = 1u << 24;
constexpr uint32_t kScoutPolls = 1u << 24;
enum Ctrl { kProgress = 0, kEpoch = 1, kAbort = 2 };

// A cell's prepared decision: two candidate lists of up to 32 entries in list
// (= ascending distance) order, entry i for walker lane i, both without the
// cell above:
//  f: the candidates under the usage cap in the scout's snapshot (valid while
//     the epoch is unchanged);
//  r: all candidates (valid in any epoch, used after a reset).
// Entry i is the key (i << 16 | palette index), ~0 where the list is
// shorter; the lowest key among eligible entries is the first eligible one.
// clear_*: bit i set when no later entry of the list (nor anything beyond it)
// lies inside the 2*weight window of entry i -- then, if entry i is the first
// eligible one, the penalty cannot change the decision.  Palette indices are
// 16-bit (palettes of at most 65535).
struct __align__(16) CellRecord {
  uint32_t kf[32];
  uint32_t kr[32];
  float df[32];
  float dr[32];
  uint32_t clear_f, clear_r, epoch, pad;
};

// Records live in a ring.  A scout writes cell c's record once the walker has
// committed the cell above (c - gw), so the walker is done with every record
// up to c - gw + 1; a ring of more than gw + 1 slots keeps that slot free.
__host__ __device__ inline int ring_size(int gw) {
  int r = 32;
  while (r < gw + kScouts + 4) r <<= 1;
  return r;
}

__host__ __device__ inline size_t scout_smem_bytes(int gw, int p, bool lab_smem) {
  const int R = ring_size(gw);
  size_t b = 16;                                    // control words
  b += (size_t)R * sizeof(CellRecord) + (size_t)R * 4;  // records + sequence words
  b += align16((size_t)gw * 4);                        // the row above
  b += align16((size_t)p * 4);                         // usage counters
  if (lab_smem) b += (size_t)p * 16;
  return b;
}

// The exact decision for one cell (greedy_walk's per-cell rule, candidate rows
// read from global memory).  Updates the counters; a fallback resets them and
// bumps the epoch.  Returns the chosen palette index.
template <class LabFn>
__device__ int full_cell(LabFn lab, const uint32_t* __restrict__ ci, const float* __restrict__ cd, int k, int p, int up,
                         int left, uint32_t* usage, uint32_t max_usage, float weight, uint32_t* ctrl,
                         uint32_t& epoch, int& resets, int lane) {
  const bool use_pen = weight > 0.0f;
  const float two_w = __fmul_rn(2.0f, weight);
  auto okf = [&](uint32_t t, int j) {
    return j < k && t < (uint32_t)p && (int)t != up && (int)t != left && usage[t] < max_usage;
  };
  uint32_t tr = kNoCand;
  float dr = __int_as_float(0x7f800000);
  unsigned m = 0;
  int r = -1;
  do {
    ++r;
    const int j = r * 32 + lane;
    tr = kNoCand;
    dr = __int_as_float(0x7f800000);
    if (j < k) {
      tr = __ldg(ci + j);
      dr = __ldg(cd + j);
    }
    m = __ballot_sync(0xffffffffu, okf(tr, j));
  } while (!m && (r + 1) * 32 < k);
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
        const float4 lab_up = up >= 0 ? lab(up) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 lab_left = left >= 0 ? lab(left) : make_float4(0.f, 0.f, 0.f, 0.f);
        uint32_t best_s = 0xFFFFFFFFu;
        for (int rr = r; rr * 32 < k; ++rr) {
          const int j = rr * 32 + lane;
          uint32_t tj = kNoCand;
          float dj = __int_as_float(0x7f800000);
          if (j < k) {
            tj = __ldg(ci + j);
            dj = __ldg(cd + j);
          }
          const bool in = j >= e0 && dj < b0 && okf(tj, j);
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
    t = (int)__ldg(ci + win);
    __syncwarp();
    if (lane == 0) usage[t] += 1u;
  } else {
    // main.rs:420-475: global reset, first candidate passing can_place, else nearest.
    ++resets;
    __syncwarp();
    for (int i = lane; i < p; i += 32) usage[i] = 0;
    t = -1;
    for (int rr = 0; rr * 32 < k && t < 0; ++rr) {
      const int j = rr * 32 + lane;
      int tj = -1;
      if (j < k) tj = (int)__ldg(ci + j);
      const unsigned mask = __ballot_sync(0xffffffffu, j < k && tj >= 0 && tj < p && tj != up && tj != left);
      if (mask) t = __shfl_sync(0xffffffffu, tj, __ffs(mask) - 1);
    }
    if (t < 0) t = (int)__ldg(ci);
    __threadfence_block();
    __syncwarp();
    ++epoch;
    if (lane == 0) {
      usage[t] = 1u;
      st_release_cta(&ctrl[kEpoch], epoch);
    }
  }
  return t;
}

// A scout warp: prepares the records of cells s, s + 12, s + 24, ...
__device__ void scout_cells(int s, const GreedyJob& J, int p, const uint32_t* usage, const int32_t* row,
                            CellRecord* rec, uint32_t* seq, uint32_t* ctrl, int R, uint32_t* err) {
  const int lane = threadIdx.x & 31;
  const int gw = J.gw, k = J.k, n = gw * J.gh;
  const uint32_t max_usage = J.max_usage;
  const bool use_pen = J.weight > 0.0f;
  const float two_w = __fmul_rn(2.0f, J.weight);
  const int nr = (k + 31) >> 5;
  const float inf = __int_as_float(0x7f800000);
  const unsigned lt = (1u << lane) - 1u;
  for (int c = s; c < n; c += kScouts) {
    const int x = c % gw, y = c / gw;
    const uint32_t* ci = J.cand_idx + (size_t)c * k;
    const float* cd = J.cand_dist + (size_t)c * k;
    uint32_t t[4];
    float d[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = r * 32 + lane;
      t[r] = kNoCand;
      d[r] = inf;
      if (r < nr && j < k) {
        t[r] = __ldg(ci + j);
        d[r] = __ldg(cd + j);
      }
    }
    int up = -1;
    if (y > 0) {
      const uint32_t need = (uint32_t)(c - gw + 1);
      uint32_t polls = 0;
      while (ld_acquire_cta(&ctrl[kProgress]) < need) {
        if (ld_volatile_u32(&ctrl[kAbort])) return;
        if (++polls > kScoutPolls) {
          if (lane == 0) {
            atomicOr(err, kErrTimeout);
            *reinterpret_cast<volatile uint32_t*>(&ctrl[kAbort]) = 1u;
          }
          return;
        }
        __nanosleep(32);
      }
      up = row[x];
    }
    CellRecord& Rc = rec[c & (R - 1)];
    const uint32_t ep0 = ld_acquire_cta(&ctrl[kEpoch]);
    int bf = 0, br = 0;
    float af = inf, ar = inf;  // distance of the 33rd entry
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (r < nr && (bf <= 32 || br <= 32)) {
        const bool in = t[r] < (uint32_t)p && (int)t[r] != up;
        const bool okf = in && usage[t[r]] < max_usage;
        const unsigned mf = __ballot_sync(0xffffffffu, okf), mr = __ballot_sync(0xffffffffu, in);
        const int pf = bf + __popc(mf & lt), pr = br + __popc(mr & lt);
        if (okf && pf < 32) {
          Rc.kf[pf] = ((uint32_t)pf << 16) | t[r];
          Rc.df[pf] = d[r];
        }
        if (in && pr < 32) {
          Rc.kr[pr] = ((uint32_t)pr << 16) | t[r];
          Rc.dr[pr] = d[r];
        }
        const unsigned f32 = __ballot_sync(0xffffffffu, okf && pf == 32);
        const unsigned r32 = __ballot_sync(0xffffffffu, in && pr == 32);
        if (f32) af = __shfl_sync(0xffffffffu, d[r], __ffs(f32) - 1);
        if (r32) ar = __shfl_sync(0xffffffffu, d[r], __ffs(r32) - 1);
        bf += __popc(mf);
        br += __popc(mr);
      }
    }
    __threadfence_block();
    const uint32_t ep1 = ld_volatile_u32(&ctrl[kEpoch]);
    __syncwarp();
    const int cf = min(bf, 32), cr = min(br, 32);
    // static window test of entry `lane` against the next entry of its list
    const float dfi = lane < cf ? Rc.df[lane] : inf, dfn = lane + 1 < cf ? Rc.df[lane + 1] : af;
    const float dri = lane < cr ? Rc.dr[lane] : inf, drn = lane + 1 < cr ? Rc.dr[lane + 1] : ar;
    const unsigned clear_f = __ballot_sync(0xffffffffu, lane < cf && (!use_pen || !(dfn < __fadd_rn(dfi, two_w))));
    const unsigned clear_r = __ballot_sync(0xffffffffu, lane < cr && (!use_pen || !(drn < __fadd_rn(dri, two_w))));
    if (lane >= cf) Rc.kf[lane] = 0xFFFFFFFFu;
    if (lane >= cr) Rc.kr[lane] = 0xFFFFFFFFu;
    if (lane == 0) {
      Rc.clear_f = clear_f;
      Rc.clear_r = clear_r;
      Rc.epoch = ep0 == ep1 ? ep0 : kInvalidEpoch;
    }
    __threadfence_block();
    __syncwarp();
    if (lane == 0) st_release_cta(&seq[c & (R - 1)], (uint32_t)(c + 1));
  }
}

template <bool kLabSmem>
__global__ void __launch_bounds__(kScoutWarps * 32) greedy_scout_kernel(const float4* __restrict__ pal, int p,
                                                                        const GreedyJob* __restrict__ jobs,
                                                                        uint32_t* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  const GreedyJob J = jobs[blockIdx.x];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = J.gw, gh = J.gh, k = J.k, n = gw * gh;
  const int R = ring_size(gw);
  uint32_t* ctrl = reinterpret_cast<uint32_t*>(smem);
  CellRecord* rec = reinterpret_cast<CellRecord*>(smem + 16);
  uint32_t* seq = reinterpret_cast<uint32_t*>(rec + R);
  int32_t* row = reinterpret_cast<int32_t*>(seq + R);
  uint32_t* usage = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(row) + align16((size_t)gw * 4));
  float4* s_lab = reinterpret_cast<float4*>(reinterpret_cast<uint8_t*>(usage) + align16((size_t)p * 4));
  for (int i = threadIdx.x; i < p; i += blockDim.x) {
    usage[i] = 0;
    if (kLabSmem) s_lab[i] = pal[i];
  }
  for (int i = threadIdx.x; i < R; i += blockDim.x) seq[i] = 0;
  if (threadIdx.x < 4) ctrl[threadIdx.x] = 0;
  __syncthreads();

  if (warp != 0) {
    if ((warp & 3) == 0) return;  // shares the walker's sub-partition
    scout_cells((warp >> 2) * 3 + (warp & 3) - 1, J, p, usage, row, rec, seq, ctrl, R, err);
    return;
  }

  // ---- warp 0: the walker
  const uint32_t max_usage = J.max_usage;
  const float weight = J.weight;
  auto lab = [=](int i) -> float4 { return kLabSmem ? s_lab[i] : __ldg(pal + i); };
  uint32_t epoch = 0;
  int resets = 0, last = -1, x = 0, y = 0;
  int ready_until = 0;  // records of cells [.., ready_until) are published
  bool aborted = false;
  // Whether the record of cell c is published.  Records [0, ready_until) are
  // known to be; a probe checks the next eight (lane i acquires the sequence
  // word of cell ready_until + i).  With `block` it waits (bounded).
  auto ready = [&](int c, bool block) -> bool {
    if (c < ready_until) return true;
    uint32_t polls = 0;
    for (;;) {
      const int base = ready_until;
      const int cc = base + (lane & 7);
      const bool mine = lane >= 8 || cc >= n || ld_acquire_cta(&seq[cc & (R - 1)]) == (uint32_t)(cc + 1);
      const unsigned pending = __ballot_sync(0xffffffffu, !mine);
      const int nready = pending ? __ffs(pending) - 1 : 8;
      if (nready > 0) {
        ready_until = min(n, base + nready);
        __syncwarp();  // the acquiring lanes' view reaches every lane
      }
      if (c < ready_until) return true;
      if (!block) return false;
      if (++polls > kWalkPolls || ld_volatile_u32(&ctrl[kAbort])) {
        aborted = true;
        return false;
      }
    }
  };
  // The walk is a chain of dependent decisions; per cell the critical path is
  // the eligibility test, one warp minimum and the clear bit.  Record reads are
  // software-pipelined around it: the header of cell c + 2 and the counters of
  // cell c + 1 are read while cell c is decided, and everything uncommon (the
  // full evaluation, row ends, progress releases, records not yet published)
  // sits behind one branch.
  struct Head {
    uint32_t ep, kf, kr, cf, cr;
  };
  struct Cur {
    uint32_t key, ti, ui, clear;
  };
  auto load_head = [&](int c) {
    const CellRecord& Rc = rec[c & (R - 1)];
    Head h;
    h.ep = Rc.epoch;
    h.kf = Rc.kf[lane];
    h.kr = Rc.kr[lane];
    h.cf = Rc.clear_f;
    h.cr = Rc.clear_r;
    return h;
  };
  auto finish = [&](const Head& h) {
    const bool f = h.ep == epoch;
    Cur r;
    r.key = f ? h.kf : h.kr;
    r.clear = f ? h.cf : h.cr;
    r.ti = r.key & 0xFFFFu;
    r.ui = r.key != 0xFFFFFFFFu ? usage[r.ti] : 0xFFFFFFFFu;
    return r;
  };
  Cur cur{0xFFFFFFFFu, 0u, 0xFFFFFFFFu, 0u};
  Head h1{};
  bool h1_ok = false;
  if (n > 0 && ready(0, true)) {
    cur = finish(load_head(0));
    h1_ok = n > 1 && ready(1, false);
    if (h1_ok) h1 = load_head(1);
  }
  for (int c = 0; c < n && !aborted; ++c) {
    // (a) header of cell c + 2, if published (waiting here, before this
    // cell's progress release, could wait on a scout that waits on this cell)
    Head h2{};
    const bool h2_ok = c + 2 < n && ready(c + 2, false);
    if (h2_ok) h2 = load_head(c + 2);
    // (b) counters of cell c + 1, read before this cell's commit: the choice
    // made here is that cell's left neighbour (row starts are re-read below)
    Cur nxt = cur;
    if (h1_ok) nxt = finish(h1);
    // (c) this cell: the lowest key among entries that pass the counters and
    // the left neighbour (the lists already exclude the cell above)
    const int left = x > 0 ? last : -1;
    const bool ok = cur.ui < max_usage && cur.ti != (uint32_t)left;
    const uint32_t best = __reduce_min_sync(0xffffffffu, ok ? cur.key : 0xFFFFFFFFu);
    const int e = (int)(best >> 16);
    const bool fast = best != 0xFFFFFFFFu && ((cur.clear >> (e & 31)) & 1u);
    int t = (int)(best & 0xFFFFu);
    if (fast && lane == e) {
      usage[cur.ti] = cur.ui + 1u;
      row[x] = t;
    }
    const bool row_end = x + 1 == gw;
    const bool rare = !fast || row_end || ((c + 1) & 7) == 0 || c + 1 == n || !h1_ok;
    if (rare) {
      if (!fast) {
        const int up = y > 0 ? row[x] : -1;
        t = full_cell(lab, J.cand_idx + (size_t)c * k, J.cand_dist + (size_t)c * k, k, p, up, left, usage,
                      max_usage, weight, ctrl, epoch, resets, lane);
        if (lane == 0) row[x] = t;
      }
      __syncwarp();
      if (row_end) {
        // the finished row goes to global memory in one coalesced pass
        for (int i = lane; i < gw; i += 32) J.grid[(size_t)y * gw + i] = row[i];
      }
      if (lane == 0 && (((c + 1) & 7) == 0 || c + 1 == n)) st_release_cta(&ctrl[kProgress], (uint32_t)(c + 1));
      if (c + 1 < n) {
        if (!h1_ok) {
          h1_ok = ready(c + 1, true);
          if (h1_ok) h1 = load_head(c + 1);
        }
        // the counters moved (a full evaluation), or the next cell starts a row
        // and may take this cell's choice, or its record came late: read afresh
        if (h1_ok) nxt = finish(h1);
      }
    } else {
      __syncwarp();
    }
    last = t;
    cur = nxt;
    h1 = h2;
    h1_ok = h2_ok;
    if (++x == gw) {
      x = 0;
      ++y;
    }
  }
  if (aborted) {
    if (lane == 0) {
      atomicOr(err, kErrTimeout);
      *reinterpret_cast<volatile uint32_t*>(&ctrl[kAbort]) = 1u;
    }
    return;
  }
  __syncwarp();
  const float total = warp_total_cost(lab, J.grid, gw, gh, lane);
  if (lane == 0) {
    if (J.n_resets) *J.n_resets = resets;
    if (J.total_cost) *J.total_cost = total;
  }
}

}  // namespace

size_t greedy_shared_bytes(int k, int gw, int p, bool lab_smem, bool usage_smem) {
  return greedy_smem_bytes(k, gw, p, lab_smem, usage_smem);
}

int launch_greedy(const float4* pal, int p, const GreedyJob* jobs_dev, int n_jobs, int k, int max_gw,
                  uint32_t* usage_scratch, uint32_t* err, cudaStream_t stream) {
  if (n_jobs <= 0) return MG_OK;
  if (k < 1 || k > 100) return fail(MG_ERR_ARG, "candidate count must be in 1..100");
  constexpr size_t kMaxSmem = 220 * 1024;
  static int configured_device = -1;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(greedy_scout_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(greedy_scout_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    configured_device = dev;
  }
  // The scouted walk: counters in shared memory, 16-bit palette indices, rows
  // of at least 8 cells.
  if (max_gw >= 8 && p <= 65535) {
    bool lab_smem = scout_smem_bytes(max_gw, p, true) <= kMaxSmem;
    const size_t bytes = scout_smem_bytes(max_gw, p, lab_smem);
    if (bytes <= kMaxSmem) {
      if (lab_smem)
        greedy_scout_kernel<true><<<n_jobs, kScoutWarps * 32, bytes, stream>>>(pal, p, jobs_dev, err);
      else
        greedy_scout_kernel<false><<<n_jobs, kScoutWarps * 32, bytes, stream>>>(pal, p, jobs_dev, err);
      g_launches += 1;
      MG_CUDA(cudaGetLastError());
      return MG_OK;
    }
  }
  bool lab_smem = true, usage_smem = true;
  size_t bytes = greedy_smem_bytes(k, max_gw, p, lab_smem, usage_smem);
  if (bytes > kMaxSmem) {
    lab_smem = false;
    bytes = greedy_smem_bytes(k, max_gw, p, lab_smem, usage_smem);
  }
  if (bytes > kMaxSmem) {
    usage_smem = false;
    bytes = greedy_smem_bytes(k, max_gw, p, lab_smem, usage_smem);
  }
  if (bytes > kMaxSmem) return fail(MG_ERR_ARG, "grid row too wide for the greedy walk");
  if (!usage_smem && !usage_scratch) return fail(MG_ERR_ARG, "usage scratch required for this palette size");
  if (lab_smem)
    greedy_kernel<true, true><<<n_jobs, 32, bytes, stream>>>(pal, p, jobs_dev, usage_scratch, err);
  else if (usage_smem)
    greedy_kernel<false, true><<<n_jobs, 32, bytes, stream>>>(pal, p, jobs_dev, usage_scratch, err);
  else
    greedy_kernel<false, false><<<n_jobs, 32, bytes, stream>>>(pal, p, jobs_dev, usage_scratch, err);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
