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
//    palettes above 65535 materials, grids narrower than 8 cells and walks
//    whose three-CTA form does not fit in shared memory.
//  - greedy_pair_kernel: a cluster of three CTAs per mosaic.  The walk is a
//    chain of dependent decisions, so its speed is the latency of one decision.
//    One warp of CTA 0 (the walker) makes the decisions; 64 scout warps in
//    CTAs 1 and 2, on other SMs, prepare each cell's decision ahead of the walker
//    from a snapshot of the usage counters, reading the walk's state and
//    writing their records through distributed shared memory:
//      the first 32 candidates (list order) that differ from the cell above
//      and were under the usage cap in the snapshot, and for each whether the
//      next such candidate lies outside its 2*weight window (`clear`: then the
//      penalty cannot change the decision if that candidate is the first
//      eligible one); also the first 32 candidates regardless of the counters,
//      for use after a reset.
//    Counters only grow between resets, so a candidate that failed the cap in
//    the snapshot still fails it when the walker arrives: the walker's first
//    eligible candidate is the first record entry that passes the fresh
//    counter and differs from the left neighbour -- one warp minimum -- and
//    with its `clear` bit set it is the reference's choice, bit for bit.  In
//    every other case (window not clear, no entry passes, a reset since the
//    snapshot for the filtered list) the walker evaluates the cell in full,
//    exactly as greedy_walk does -- except that with the palette Lab in global
//    memory a window that closes inside the filtered list is settled from the
//    record (window_cell).  A scout builds a record once the walker has placed
//    the cell kLead cells (or a row) back, polling the walker's ring of
//    placed cells, and a reset bumps an epoch that invalidates older snapshots.
//    The walker's shared memory holds rings (records, placed cells), not the
//    grid, so a mosaic of any cell count walks in this form.  After the walk
//    the scout CTA computes calculate_total_cost: terms in parallel, one
//    sequential FP32 sum in the reference's order.
#include <cstddef>

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
// A cluster of 1 + kScoutCtas CTAs per mosaic.  CTA 0 walks (warp 0; the
// state of the walk lives in its shared memory); the other CTAs, on other
// SMs, hold the scouts, which read the walk's state and write their records
// through distributed shared memory, so the walker's SM runs nothing but the
// walk.  Two cluster shapes hold the same 64 scouts: four scout CTAs of 16
// warps (128 registers a thread, which the walker's loop uses: a launch of a
// few mosaics), or two of 32 warps (64 registers; a batch, whose clusters
// then take three SMs each instead of five).
constexpr int kScouts = 64;                 // every warp of the scout CTAs
constexpr int kScoutWarpsMax = 32;          // per CTA, the larger shape
constexpr uint32_t kInvalidEpoch = 0xFFFFFFFFu;
constexpr uint32_t kWalkPolls = 1u << 24;      // the walker's bounded wait for a record
constexpr uint32_t kInjectedWalkPolls = 1u << 12;  // ... when a timeout is injected (well under a millisecond)
constexpr uint32_t kScoutPolls = 1u << 22;  // polls of about 1 us each
// Records are built at most kLead cells ahead of the walker: 124 in the
// five-CTA shape (a ring of 128 holds them; fewer late records), 80 in the
// three-CTA shape of batches (fresher snapshots: fewer cells whose whole list
// was capped since, which matters with their dense palettes).  The rings are
// sized for the larger.
constexpr int kScoutLead = 124;
constexpr int kScoutLeadBatch = 80;
constexpr int kCostChunk = 2048;  // cells per pass of the final cost sum
constexpr uint32_t kFollowPolls = 1u << 26;  // the cost warp's bounded wait for a placement (seconds)
enum Ctrl { kProgress = 0, kEpoch = 1, kAbort = 2 };

// A cell's prepared decision: two candidate lists of up to 32 entries in list
// (= ascending distance) order, entry i for walker lane i, both without the
// cell above:
//  f: the candidates under the usage cap in the scout's snapshot (valid while
//     the epoch is unchanged);
//  r: all candidates (valid in any epoch, used after a reset).
// Entry i is the key (i << 17 | blocked << 16 | palette index), ~0 where the
// list is shorter, so the lowest key among eligible entries is the first
// eligible one.  `blocked` is clear when no later entry of the list (nor
// anything beyond it) lies inside the 2*weight window of entry i -- then, if
// entry i is the first eligible one, the penalty cannot change the decision.
// Palette indices are 16-bit (palettes of at most 65535).
// The record also carries, for each f entry, its distance, its weight against
// the cell above (0 in the first row) and its Lab, and `f_next`, the distance
// of the first entry after the list (+inf when the list holds every entry
// under the cap): the walker then settles a cell whose penalty window holds
// several entries from shared memory (window_cell).
struct __align__(16) CellRecord {
  uint32_t kf[32];
  uint32_t kr[32];
  uint32_t epoch;
  float f_next;
  uint32_t pad[2];
  float wd[32];
  float wu[32];
  float4 wl[32];
};
// A scout's working copy of one record (in its own CTA).
struct ScoutStage {
  uint32_t kf[32], kr[32];
  float df[32], dr[32];
};

// Records live in a ring.  A scout writes cell c's record once the walker has
// placed cell c - lead (lead = min(gw, kScoutLead)), so the walker is past
// every record up to c - lead and reads at most two ahead of its cell; a ring
// of more than lead + 3 slots keeps the slot of record c - R free.
__host__ __device__ inline int ring_size(int gw) {
  const int lead = gw < kScoutLead ? gw : kScoutLead;
  int r = 32;
  while (r < lead + 4) r <<= 1;
  return r;
}

// The placed cells live in the walker CTA's shared memory in one of two forms:
//  - the grid, 16-bit, kUnplaced until placed (copied to global memory after
//    the walk);
//  - when the grid does not fit: a ring of words (cell index & 0xFFFF) << 16 |
//    material, one 32-bit store publishing a placement and naming its cell.
//    The walker reads the cell above its own; a scout reads its lead cell and
//    the cell above its cell.  The walker never passes a cell whose record is
//    missing, so no cell read is more than gw + kScoutLead + 64 behind the
//    newest placement, and a ring of more slots than that keeps every cell
//    until it is read.  The global grid receives each placement as it is made.
constexpr uint16_t kUnplaced = 0xFFFFu;
constexpr uint32_t kNoCell = 0xFFFFFFFFu;  // a ring slot no placement has written yet
__host__ __device__ inline int cell_ring_size(int gw) {
  int r = 64;
  while (r < gw + kScoutLead + 72) r <<= 1;
  return r;
}
__device__ __forceinline__ uint32_t cell_word(int c, int t) { return ((uint32_t)c << 16) | ((uint32_t)t & 0xFFFFu); }

// Shared memory of the walker CTA: control words, record ring, sequence
// words, the placed cells (grid or ring), usage counters, optionally the
// palette Lab.
__host__ __device__ inline size_t cells_bytes(int gw, int n, bool ring) {
  return ring ? (size_t)cell_ring_size(gw) * 4 : align16((size_t)n * 2);
}
__host__ __device__ inline size_t walker_smem_bytes(int gw, int n, int p, bool lab_smem, bool ring) {
  const int R = ring_size(gw);
  size_t b = 16 + (size_t)R * sizeof(CellRecord) + (size_t)R * 4;
  b += cells_bytes(gw, n, ring);
  b += align16((size_t)p * 4);
  if (lab_smem) b += (size_t)p * 16;
  return b;
}
// Shared memory of the scout CTA: staging per warp, then the cost terms.
__host__ __device__ inline size_t scout_cta_smem_bytes() {
  return (size_t)kScoutWarpsMax * sizeof(ScoutStage) + (size_t)kCostChunk * 8;
}
__host__ __device__ inline size_t pair_smem_bytes(int gw, int n, int p, bool lab_smem, bool ring) {
  const size_t a = walker_smem_bytes(gw, n, p, lab_smem, ring), b = scout_cta_smem_bytes();
  return a > b ? a : b;
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
    fence_cluster();
    __syncwarp();
    ++epoch;
    if (lane == 0) {
      usage[t] = 1u;
      st_release_cluster(smem_u32(&ctrl[kEpoch]), epoch);
    }
  }
  return t;
}

// full_cell with the whole candidate row (k <= 100: four entries per lane)
// and the neighbours' Lab read at once, then the Lab of the candidates inside
// the penalty window: two dependent memory round trips whatever the depth of
// the first eligible entry.  Taken when the palette's Lab is read from global
// memory, where a round trip costs most; the same decision as full_cell.
template <class LabFn>
__device__ int full_cell_rows(LabFn lab, const uint32_t* __restrict__ ci, const float* __restrict__ cd, int k, int p,
                              int up, int left, uint32_t* usage, uint32_t max_usage, float weight, uint32_t* ctrl,
                              uint32_t& epoch, int& resets, int lane) {
  constexpr int kRounds = 4;  // ceil(100 / 32)
  const bool use_pen = weight > 0.0f;
  const float two_w = __fmul_rn(2.0f, weight);
  const float kInf = __int_as_float(0x7f800000);
  uint32_t tr[kRounds];
  float dr[kRounds];
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    const int j = r * 32 + lane;
    tr[r] = j < k ? __ldg(ci + j) : kNoCand;
    dr[r] = j < k ? __ldg(cd + j) : kInf;
  }
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 lab_up = use_pen && up >= 0 ? lab(up) : zero;
  const float4 lab_left = use_pen && left >= 0 ? lab(left) : zero;
  auto okf = [&](uint32_t t) { return t < (uint32_t)p && (int)t != up && (int)t != left && usage[t] < max_usage; };
  int r0 = -1;
  unsigned m = 0;
#pragma unroll
  for (int r = 0; r < kRounds; ++r) {
    const unsigned mr = __ballot_sync(0xffffffffu, okf(tr[r]));
    if (r0 < 0 && mr) {
      r0 = r;
      m = mr;
    }
  }
  int t;
  if (r0 >= 0) {
    const int e0l = __ffs(m) - 1;
    int win = r0 * 32 + e0l;
    uint32_t t_win = 0;
#pragma unroll
    for (int r = 0; r < kRounds; ++r)
      if (r == r0) t_win = __shfl_sync(0xffffffffu, tr[r], e0l);
    if (use_pen) {
      float d0 = 0.0f;
#pragma unroll
      for (int r = 0; r < kRounds; ++r)
        if (r == r0) d0 = __shfl_sync(0xffffffffu, dr[r], e0l);
      const float b0 = __fadd_rn(d0, two_w);
      // another eligible entry after e0 inside [d0, d0 + 2w): penalties decide
      bool any_in = false;
#pragma unroll
      for (int r = 0; r < kRounds; ++r) any_in |= r * 32 + lane > win && dr[r] < b0 && okf(tr[r]);
      if (__any_sync(0xffffffffu, any_in)) {
        float4 lt[kRounds];
        bool in[kRounds];
#pragma unroll
        for (int r = 0; r < kRounds; ++r) {
          in[r] = r * 32 + lane >= win && dr[r] < b0 && okf(tr[r]);
          lt[r] = in[r] ? lab((int)tr[r]) : zero;
        }
        uint32_t best_s = 0xFFFFFFFFu;
#pragma unroll
        for (int r = 0; r < kRounds; ++r) {
          uint32_t sb = 0xFFFFFFFFu;
          if (in[r]) {
            float pen = 0.0f;
            if (up >= 0) pen = __fadd_rn(pen, wgt(lt[r], lab_up));
            if (left >= 0) pen = __fadd_rn(pen, wgt(lt[r], lab_left));
            sb = __float_as_uint(__fadd_rn(dr[r], __fmul_rn(pen, weight)));
          }
          const uint32_t mn = __reduce_min_sync(0xffffffffu, sb);
          if (mn < best_s) {  // strict: the earliest entry keeps a tie
            best_s = mn;
            const int l = __ffs(__ballot_sync(0xffffffffu, sb == mn)) - 1;
            win = r * 32 + l;
            t_win = __shfl_sync(0xffffffffu, tr[r], l);
          }
        }
      }
    }
    t = (int)t_win;
    __syncwarp();
    if (lane == 0) usage[t] += 1u;
  } else {
    // main.rs:420-475: global reset, first candidate passing can_place, else nearest.
    ++resets;
    __syncwarp();
    for (int i = lane; i < p; i += 32) usage[i] = 0;
    t = -1;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
      const int tj = (int)tr[r];
      const unsigned mask = __ballot_sync(0xffffffffu, tr[r] != kNoCand && tj >= 0 && tj < p && tj != up && tj != left);
      if (t < 0 && mask) t = __shfl_sync(0xffffffffu, tj, __ffs(mask) - 1);
    }
    if (t < 0) t = (int)__shfl_sync(0xffffffffu, tr[0], 0);
    fence_cluster();
    __syncwarp();
    ++epoch;
    if (lane == 0) {
      usage[t] = 1u;
      st_release_cluster(smem_u32(&ctrl[kEpoch]), epoch);
    }
  }
  return t;
}

// The walker CTA's shared-memory layout (both CTAs compute it; the scouts map
// it into the walker CTA's window).
struct WalkerLayout {
  uint32_t* ctrl;
  CellRecord* rec;
  uint32_t* seq;
  uint32_t* ring;    // the placed cells as a ring (kRing) ...
  uint16_t* grid16;  // ... or as the 16-bit grid; the same address
  uint32_t* usage;
  float4* lab;
};
__device__ inline WalkerLayout walker_layout(uint8_t* smem, int gw, int n, int p, int R, bool ring) {
  WalkerLayout L;
  L.ctrl = reinterpret_cast<uint32_t*>(smem);
  L.rec = reinterpret_cast<CellRecord*>(smem + 16);
  L.seq = reinterpret_cast<uint32_t*>(L.rec + R);
  L.ring = L.seq + R;
  L.grid16 = reinterpret_cast<uint16_t*>(L.ring);
  L.usage = reinterpret_cast<uint32_t*>(reinterpret_cast<uint8_t*>(L.ring) + cells_bytes(gw, n, ring));
  L.lab = reinterpret_cast<float4*>(reinterpret_cast<uint8_t*>(L.usage) + align16((size_t)p * 4));
  return L;
}

// A scout warp: prepares the records of cells s, s + kScouts, s + 2 kScouts, ...
// Returns false when the walk was aborted.
// (The layout is recomputed here rather than passed by reference: a struct
// whose address escapes would turn the walker's shared-memory pointers into
// generic ones.)
// withhold: build the records but never publish them (an injected fault: the
// walker's wait for the first record then runs out).
template <bool kRing, int kLead>
__device__ bool scout_cells(int s, const GreedyJob& J, const float4* __restrict__ pal, int p, uint8_t* smem,
                            ScoutStage& S, int R, uint32_t* err, bool withhold) {
  const int lane = threadIdx.x & 31;
  const int gw = J.gw, k = J.k, n = gw * J.gh;
  const WalkerLayout L = walker_layout(smem, gw, n, p, R, kRing);
  const uint32_t max_usage = J.max_usage;
  const bool use_pen = J.weight > 0.0f;
  const float two_w = __fmul_rn(2.0f, J.weight);
  const int nr = (k + 31) >> 5;
  const float inf = __int_as_float(0x7f800000);
  const unsigned lt = (1u << lane) - 1u;
  // the walker CTA's words, in the cluster window
  const uint32_t r_epoch = cluster_map(&L.ctrl[kEpoch], 0), r_abort = cluster_map(&L.ctrl[kAbort], 0);
  const uint32_t r_usage = cluster_map(L.usage, 0), r_cells = cluster_map(L.ring, 0);
  const int cmask = cell_ring_size(gw) - 1;
  const uint32_t r_rec = cluster_map(L.rec, 0), r_seq = cluster_map(L.seq, 0);
  for (int c = s; c < n; c += kScouts) {
    const int y = c / gw;
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
    // Wait until the walker has placed cell c - min(gw, kLead): the
    // cell above is then placed, and the counters this record is filtered by
    // are at most kLead placements old (in a region of one colour a
    // row's placements cap dozens of the nearest materials; a record built a
    // whole row ahead would list none left).  Each cell is written once, by a
    // single 16-bit store, so a scout that sees a value sees the final one; and
    // the walker read that cell's record before placing it (the placement
    // depends on it), so the walker is done with the ring slot this record
    // reuses (the ring holds more than gw records).
    const int lead = c - min(gw, kLead);
    uint32_t v_lead = kNoCell;  // the lead cell's material in the low 16 bits
    if (lead >= 0) {
      const uint32_t a_lead = kRing ? r_cells + 4u * (uint32_t)(lead & cmask) : r_cells + 2u * (uint32_t)lead;
      const uint32_t tag = (uint32_t)lead & 0xFFFFu;
      uint32_t polls = 0;
      auto placed = [&]() {
        if (kRing) {
          v_lead = ld_cluster_u32(a_lead);
          return (v_lead >> 16) == tag;
        }
        v_lead = ld_cluster_u16(a_lead);
        return v_lead != kUnplaced;
      };
      while (!placed()) {
        if (ld_cluster_u32(r_abort)) return false;
        if (++polls > kScoutPolls) {
          if (lane == 0) {
            atomicOr(err, kErrTimeout);
            st_cluster_u32(r_abort, 1u);
          }
          return false;
        }
        __nanosleep(1000);  // the scouts run far ahead: poll the walker's SM rarely
      }
    }
    const int up = y == 0           ? -1
                   : lead == c - gw ? (int)(v_lead & 0xFFFFu)
                   : kRing          ? (int)(ld_cluster_u32(r_cells + 4u * (uint32_t)((c - gw) & cmask)) & 0xFFFFu)
                                    : (int)ld_cluster_u16(r_cells + 2u * (uint32_t)(c - gw));
    const uint32_t ep0 = ld_acquire_cluster(r_epoch);
    int bf = 0, br = 0;
    float af = inf, ar = inf;  // distance of the 33rd entry
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      if (r < nr && (bf <= 32 || br <= 32)) {
        const bool in = t[r] < (uint32_t)p && (int)t[r] != up;
        // counters are read on demand: each one is a load from the walker's SM
        const bool okf = in && ld_cluster_u32(r_usage + 4u * t[r]) < max_usage;
        const unsigned mf = __ballot_sync(0xffffffffu, okf), mr = __ballot_sync(0xffffffffu, in);
        const int pf = bf + __popc(mf & lt), pr = br + __popc(mr & lt);
        if (okf && pf < 32) {
          S.kf[pf] = ((uint32_t)pf << 17) | t[r];
          S.df[pf] = d[r];
        }
        if (in && pr < 32) {
          S.kr[pr] = ((uint32_t)pr << 17) | t[r];
          S.dr[pr] = d[r];
        }
        const unsigned f32 = __ballot_sync(0xffffffffu, okf && pf == 32);
        const unsigned r32 = __ballot_sync(0xffffffffu, in && pr == 32);
        if (f32) af = __shfl_sync(0xffffffffu, d[r], __ffs(f32) - 1);
        if (r32) ar = __shfl_sync(0xffffffffu, d[r], __ffs(r32) - 1);
        bf += __popc(mf);
        br += __popc(mr);
      }
    }
    fence_cluster();
    const uint32_t ep1 = ld_acquire_cluster(r_epoch);
    __syncwarp();
    const int cf = min(bf, 32), cr = min(br, 32);
    // static window test of entry `lane` against the next entry of its list
    const float dfi = lane < cf ? S.df[lane] : inf, dfn = lane + 1 < cf ? S.df[lane + 1] : af;
    const float dri = lane < cr ? S.dr[lane] : inf, drn = lane + 1 < cr ? S.dr[lane + 1] : ar;
    const bool blocked_f = use_pen && dfn < __fadd_rn(dfi, two_w);
    const bool blocked_r = use_pen && drn < __fadd_rn(dri, two_w);
    const uint32_t slot = (uint32_t)(c & (R - 1));
    const uint32_t rr = r_rec + slot * (uint32_t)sizeof(CellRecord);
    // final keys into the local copy, then 16-byte stores to the walker's SM
    // (fewer requests on its shared memory)
    const uint32_t kf_final = lane < cf ? S.kf[lane] | (blocked_f ? 0x10000u : 0u) : 0xFFFFFFFFu;
    const uint32_t kr_final = lane < cr ? S.kr[lane] | (blocked_r ? 0x10000u : 0u) : 0xFFFFFFFFu;
    __syncwarp();
    S.kf[lane] = kf_final;
    S.kr[lane] = kr_final;
    __syncwarp();
    if (lane < 16) {
      const uint4 v = reinterpret_cast<const uint4*>(lane < 8 ? S.kf : S.kr)[lane & 7];
      st_cluster_v4(rr + 16u * (uint32_t)lane, v);
    }
    if (lane == 0) st_cluster_u32(rr + 256u, ep0 == ep1 ? ep0 : kInvalidEpoch);
    {
      // distance, weight against the cell above and Lab of each f entry (wgt
      // as full_cell computes it), and the distance after the list
      float d = inf, wu = 0.0f;
      float4 la = make_float4(0.f, 0.f, 0.f, 0.f);
      if (lane < cf) {
        d = S.df[lane];
        la = __ldg(pal + (kf_final & 0xFFFFu));
        if (use_pen && up >= 0) wu = wgt(la, __ldg(pal + up));
      }
      const uint32_t wrec = rr + (uint32_t)offsetof(CellRecord, wd);
      st_cluster_u32(wrec + 4u * (uint32_t)lane, __float_as_uint(d));
      st_cluster_u32(rr + (uint32_t)offsetof(CellRecord, wu) + 4u * (uint32_t)lane, __float_as_uint(wu));
      st_cluster_v4(rr + (uint32_t)offsetof(CellRecord, wl) + 16u * (uint32_t)lane,
                    make_uint4(__float_as_uint(la.x), __float_as_uint(la.y), __float_as_uint(la.z), 0u));
      if (lane == 0) st_cluster_u32(rr + (uint32_t)offsetof(CellRecord, f_next), __float_as_uint(cf < 32 ? inf : af));
    }
    fence_cluster();
    __syncwarp();
    if (lane == 0 && !withhold) st_release_cluster(r_seq + 4u * slot, (uint32_t)(c + 1));
  }
  return true;
}

template <bool kLabSmem, bool kRing, int kScoutCtas, int kWarps>
__global__ void __cluster_dims__(1 + kScoutCtas, 1, 1) __maxnreg__(65536 / (kWarps * 32))
    greedy_pair_kernel(const float4* __restrict__ pal, int p, const GreedyJob* __restrict__ jobs, uint32_t* err,
                       uint32_t walk_polls, uint32_t withhold) {
  extern __shared__ __align__(128) uint8_t smem[];
  const GreedyJob J = jobs[blockIdx.x / (1 + kScoutCtas)];
  const uint32_t rank = cluster_ctarank();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gw = J.gw, gh = J.gh, k = J.k, n = gw * gh;
  const int R = ring_size(gw);
  const WalkerLayout L = walker_layout(smem, gw, n, p, R, kRing);
  if (rank == 0) {
    for (int i = threadIdx.x; i < p; i += blockDim.x) {
      L.usage[i] = 0;
      if (kLabSmem) L.lab[i] = pal[i];
    }
    for (int i = threadIdx.x; i < R; i += blockDim.x) L.seq[i] = 0;
    if (kRing)
      for (int i = threadIdx.x; i < cell_ring_size(gw); i += blockDim.x) L.ring[i] = kNoCell;
    else
      for (int i = threadIdx.x; i < n; i += blockDim.x) L.grid16[i] = kUnplaced;
    if (threadIdx.x < 4) L.ctrl[threadIdx.x] = 0;
  }
  cluster_sync_all();  // the walker CTA's state exists before any scout reads it

  if (rank >= 1) {
    // ---- the scouts, then (CTA 1) the final cost of the walk
    ScoutStage* stage = reinterpret_cast<ScoutStage*>(smem);
    float* terms = reinterpret_cast<float*>(smem + (size_t)kWarps * sizeof(ScoutStage));
    static_assert(kScoutCtas * kWarps == kScouts, "64 scouts");
    bool ok = scout_cells<kRing, kScoutCtas == 4 ? kScoutLead : kScoutLeadBatch>((int)(rank - 1) * kWarps + warp, J, pal, p, smem, stage[warp], R, err,
                                       withhold != 0u);
    if (rank > 1) {
      cluster_sync_all();
      return;
    }
    if (!kRing) {  // the walker CTA's cost warp follows the walk instead
      cluster_sync_all();
      return;
    }
    // calculate_total_cost (adjacency.rs:91-130) of the placed grid once the
    // walk is complete: terms in parallel, one sequential FP32 sum in the
    // reference's order (right then down, row-major).
    __shared__ uint32_t s_ok;
    if (threadIdx.x == 0) s_ok = 1u;
    __syncthreads();
    if (!ok) s_ok = 0u;
    __syncthreads();
    if (threadIdx.x == 0 && s_ok) {
      const uint32_t r_progress = cluster_map(&L.ctrl[kProgress], 0), r_abort = cluster_map(&L.ctrl[kAbort], 0);
      uint32_t polls = 0;
      while (ld_acquire_cluster(r_progress) < (uint32_t)n) {
        if (ld_cluster_u32(r_abort) || ++polls > kScoutPolls) {
          s_ok = 0u;
          break;
        }
        __nanosleep(256);
      }
    }
    __syncthreads();
    if (s_ok) {
      float total = 0.0f;
      for (int c0 = 0; c0 < n; c0 += kCostChunk) {
        const int m = min(kCostChunk, n - c0);
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
          const int c = c0 + i, x = c % gw, y = c / gw;
          const int cur = J.grid[c];
          float tr = 0.0f, td = 0.0f;
          if (cur >= 0) {
            const float4 lc = __ldg(pal + cur);
            if (x < gw - 1) {
              const int r = J.grid[c + 1];
              if (r >= 0) tr = wgt(lc, __ldg(pal + r));
            }
            if (y < gh - 1) {
              const int d = J.grid[c + gw];
              if (d >= 0) td = wgt(lc, __ldg(pal + d));
            }
          }
          terms[2 * i] = tr;
          terms[2 * i + 1] = td;
        }
        __syncthreads();
        if (threadIdx.x == 0)
          for (int i = 0; i < 2 * m; ++i) total = __fadd_rn(total, terms[i]);
        __syncthreads();
      }
      if (threadIdx.x == 0 && J.total_cost) *J.total_cost = total;
    }
    cluster_sync_all();
    return;
  }
  if (!kRing && warp == 1) {
    // ---- CTA 0, warp 1: calculate_total_cost (adjacency.rs:91-130) following
    // the walk, and the placed grid into global memory.  Cell c's terms (right,
    // then down) are final once cells c, c + 1 and c + gw are placed (each is
    // written once, so a value seen is the final one); one FP32 sum in the
    // reference's order, 32 cells behind a row of the walker at most, so the
    // total is ready when the walk ends.  On another SMSP than the walker.
    auto lab_of = [&](int i) -> float4 { return kLabSmem ? L.lab[i] : __ldg(pal + i); };
    const volatile uint16_t* g16 = L.grid16;
    float total = 0.0f;
    bool ok = true;
    for (int c0 = 0; c0 < n && ok; c0 += 32) {
      const int c = c0 + lane, x = c % gw, y = c / gw;
      int cur = 0, rt = 0, dn = 0;
      bool lane_ok = true;
      if (c < n) {
        uint32_t polls = 0;
        for (;;) {
          cur = g16[c];
          rt = x < gw - 1 ? g16[c + 1] : 0;
          dn = y < gh - 1 ? g16[c + gw] : 0;
          if (cur != kUnplaced && rt != kUnplaced && dn != kUnplaced) break;
          if (ld_volatile_u32(&L.ctrl[kAbort]) || ++polls > kFollowPolls) {
            lane_ok = false;
            break;
          }
          __nanosleep(128);
        }
      }
      ok = __all_sync(0xffffffffu, lane_ok);
      if (!ok) break;
      float tr = 0.0f, td = 0.0f;
      if (c < n) {
        const float4 lc = lab_of(cur);
        if (x < gw - 1) tr = wgt(lc, lab_of(rt));
        if (y < gh - 1) td = wgt(lc, lab_of(dn));
        J.grid[c] = cur;
      }
      const int m = min(32, n - c0);
      for (int i = 0; i < m; ++i) {
        const float a = __shfl_sync(0xffffffffu, tr, i), b = __shfl_sync(0xffffffffu, td, i);
        total = __fadd_rn(__fadd_rn(total, a), b);
      }
    }
    if (ok) {
      if (lane == 0 && J.total_cost) *J.total_cost = total;
    } else {
      // the walk gave up: every cell empty (this warp is the grid's only writer)
      for (int i = lane; i < n; i += 32) J.grid[i] = -1;
      if (lane == 0) atomicOr(err, kErrTimeout);
    }
    cluster_sync_all();
    return;
  }
  if (warp != 0) {
    cluster_sync_all();
    return;
  }

  // ---- CTA 0, warp 0: the walker
  // Windows that are not clear are settled inside the common loop in the
  // batch shape (dense palettes: a fifth of a batch's cells had one, each
  // leaving the loop), and on the uncommon path in the five-CTA shape, whose
  // loop the larger body slowed.
  constexpr bool kInlineWindows = kScoutCtas == 2;
  uint32_t* ctrl = L.ctrl;
  CellRecord* rec = L.rec;
  uint32_t* seq = L.seq;
  uint32_t* ring = L.ring;
  uint16_t* grid16 = L.grid16;
  const int cmask = cell_ring_size(gw) - 1;
  // a placement: the 16-bit grid, or the ring word and the global grid
  auto place = [&](int cc, int tt) {
    if (kRing) {
      ring[cc & cmask] = cell_word(cc, tt);
      J.grid[cc] = tt;
    } else {
      grid16[cc] = (uint16_t)tt;
    }
  };
  uint32_t* usage = L.usage;
  const float4* s_lab = L.lab;
  const uint32_t max_usage = J.max_usage;
  const float weight = J.weight;
  auto lab = [=](int i) -> float4 { return kLabSmem ? s_lab[i] : __ldg(pal + i); };
  uint32_t epoch = 0;
  int resets = 0, last = -1, x = 0, y = 0;
  int ready_until = 0;  // records of cells [.., ready_until) are published
  bool aborted = false;
  // Whether the record of cell c is published.  Records [0, ready_until) are
  // known to be; a probe checks the next 32 (lane i acquires the sequence word
  // of cell ready_until + i).  With `block` it waits (bounded).
  auto ready = [&](int c, bool block) -> bool {
    if (c < ready_until) return true;
    uint32_t polls = 0;
    for (;;) {
      const int base = ready_until;
      const int cc = base + lane;
      const bool mine = cc >= n || ld_acquire_cluster(smem_u32(&seq[cc & (R - 1)])) == (uint32_t)(cc + 1);
      const unsigned pending = __ballot_sync(0xffffffffu, !mine);
      const int nready = pending ? __ffs(pending) - 1 : 32;
      if (nready > 0) {
        ready_until = min(n, base + nready);
        __syncwarp();  // the acquiring lanes' view reaches every lane
      }
      if (c < ready_until) return true;
      if (!block) return false;
      if (++polls > walk_polls || ld_volatile_u32(&ctrl[kAbort])) {
        aborted = true;
        return false;
      }
    }
  };
  // The walk is a chain of dependent decisions, so its speed is the latency
  // of one decision in one warp: every warp collective and every memory wait
  // on the path from one cell's choice to the next counts in full.  Per cell,
  // one warp minimum over the record's entries under the usage cap, the left
  // neighbour's material removed, gives the reference's choice.  A record's
  // counters are read before the previous commit; the only counter that
  // commit changed is the left neighbour's, which is removed anyway -- except
  // at a row start (no left neighbour), where that entry counts with its
  // counter + 1.  Record reads are software-pipelined: the counters of cell
  // c + 1 and the header of cell c + 2 are read first while cell c is
  // decided, unconditionally (a record not yet published is read again once
  // it is).  Everything uncommon (the full evaluation, windows that are not
  // clear, late records and the probes for new ones) sits behind one branch.
  // Placements go to the shared-memory grid, which the scouts poll; the grid
  // reaches global memory once, after the walk.
  struct Head {
    uint32_t ep, kf, kr;
  };
  struct Cur {
    uint32_t key, ti, ui;
    bool f;  // the key is the record's f entry (its epoch is the walk's)
  };
  auto load_head = [&](int c) {
    const CellRecord& Rc = rec[c & (R - 1)];
    return Head{Rc.epoch, Rc.kf[lane], Rc.kr[lane]};
  };
  auto finish = [&](const Head& h) {
    Cur r;
    r.f = h.ep == epoch;
    r.key = r.f ? h.kf : h.kr;
    r.ti = r.key & 0xFFFFu;
    r.ui = (r.key != 0xFFFFFFFFu && r.ti < (uint32_t)p) ? usage[r.ti] : 0xFFFFFFFFu;
    return r;
  };
  // A cell (not a row start) whose first eligible f entry has later entries
  // inside its penalty window, settled from the record when the palette's Lab
  // is in global memory: the window's entries are the list's entries under the
  // cap now, other than the left neighbour's material, with distance below
  // d(first) + 2*weight (f_next >= that bound closes the window inside the
  // list); each scores d + (w_up + w_left) * weight in full_cell's arithmetic
  // and the lowest score, then the lowest position, wins -- full_cell's
  // decision.  Commits it and returns the material; -1 when the window may
  // reach past the list (then full_cell decides).  e0: the position of the
  // first eligible entry (the loop's minimum).  Positions and materials come
  // out of warp minimums over packed words (no bit scans or shuffles).
  auto window_cell = [&](int cc, const Cur& cu, int left, bool has_up, int e0) -> int {
    const CellRecord& Rc = rec[cc & (R - 1)];
    const bool elig = cu.key != 0xFFFFFFFFu && cu.ui < max_usage && (int)cu.ti != left;
    const float dl = Rc.wd[lane];
    const float b0 = __fadd_rn(Rc.wd[e0], __fmul_rn(2.0f, weight));
    if (!(Rc.f_next >= b0)) return -1;
    const bool in = elig && lane >= e0 && dl < b0;
    // the left neighbour's Lab: its entry in the previous cell's list, else the palette
    const CellRecord& Rp = rec[(cc - 1) & (R - 1)];
    const uint32_t pk = Rp.kf[lane];
    const uint32_t pl =
        __reduce_min_sync(0xffffffffu, (pk != 0xFFFFFFFFu && (pk & 0xFFFFu) == (uint32_t)left) ? (uint32_t)lane : 32u);
    const float4 lab_left = pl < 32u ? Rp.wl[pl] : lab(left);
    float pen = has_up ? Rc.wu[lane] : 0.0f;  // 0 + w_up, exactly
    pen = __fadd_rn(pen, wgt(Rc.wl[lane], lab_left));
    const uint32_t sb = in ? __float_as_uint(__fadd_rn(dl, __fmul_rn(pen, weight))) : 0xFFFFFFFFu;
    const uint32_t mn = __reduce_min_sync(0xffffffffu, sb);
    const bool wins = mn == 0xFFFFFFFFu ? lane == e0 : (in && sb == mn);
    const uint32_t wn = __reduce_min_sync(0xffffffffu, wins ? ((uint32_t)lane << 16) | cu.ti : 0xFFFFFFFFu);
    const int win = (int)(wn >> 16), tw = (int)(wn & 0xFFFFu);
    if (lane == win) {
      usage[cu.ti] = cu.ui + 1u;
      place(cc, tw);
    }
    return tw;
  };
  Cur cur{0xFFFFFFFFu, 0u, 0xFFFFFFFFu, false};
  bool cur_fresh = true;  // cur's counters include the previous commit
  Head h1{0u, 0xFFFFFFFFu, 0xFFFFFFFFu};
  bool h1_ok = false;
  if (n > 0 && ready(0, true)) {
    cur = finish(load_head(0));
    h1_ok = n > 1 && ready(1, false);
    h1 = load_head(1 < n ? 1 : 0);
  }
  // The common case runs in a tight inner loop of its own; a cell that needs
  // anything else leaves it, is finished below, and the inner loop resumes.
  // Each entry's packed word (position << 27 | blocked << 26 | counter << 16 |
  // material, ~0 unless present and under the cap) is formed when its
  // counter arrives, with the counter as read (wb) and with one more (wp: the
  // entry of a row start whose material the previous cell took, read before
  // that commit).  The decision is then one warp minimum over the words with
  // the left neighbour's material removed, and its commit is made by every
  // lane (the same stores), so no lane waits on another before the next
  // cell's counters are read.  The counter packs to 10 bits: an entry under
  // the cap whose counter does not fit (caps above 1023) is marked as not
  // clear, so a cell that would take it goes the uncommon way.
  struct Words {
    uint32_t ti, wb, wp;
  };
  auto words = [&](const Cur& r) -> Words {
    const uint32_t base = ((r.key >> 17) << 27) | (((r.key >> 16) & 1u) << 26) | (r.key & 0xFFFFu);
    const bool pres = r.key != 0xFFFFFFFFu;
    Words o;
    o.ti = r.ti;
    o.wb = pres & (r.ui < max_usage) ? base | (min(r.ui, 1023u) << 16) | (r.ui < 1023u ? 0u : 1u << 26) : 0xFFFFFFFFu;
    o.wp = pres & (r.ui + 1u < max_usage) ? base | (min(r.ui + 1u, 1023u) << 16) | (r.ui + 1u < 1023u ? 0u : 1u << 26)
                                         : 0xFFFFFFFFu;
    return o;
  };
  const float two_w = __fmul_rn(2.0f, weight);
  int last_pos = -1;  // position of the previous cell's choice in its record's f list, -1 unknown
  bool win_tried = false;
  int c = 0;
  while (c < n && !aborted) {
    win_tried = false;
    Head h2{};
    bool h2_ok = false;
    Cur nxt = cur;
    uint32_t chosen = 0xFFFFFFFFu;
    bool fast = false;
    Words wc = words(cur);
    for (;;) {
      // (a) counters of cell c + 1, read before this cell's commit; header of
      // cell c + 2 -- whether it is published is known from the last probe
      // (probes happen on the uncommon path; waiting here, before this cell's
      // commit, could wait on a scout that waits on this cell)
      nxt = finish(h1);
      h2_ok = c + 2 < ready_until;
      h2 = load_head(c + 2);
      // (b) this cell: the first entry under the cap that is not the left
      // neighbour's material (at a row start, that material's counter + 1)
      const bool same = wc.ti == (uint32_t)last;
      const uint32_t w = !same ? wc.wb : (x != 0 ? 0xFFFFFFFFu : (cur_fresh ? wc.wb : wc.wp));
      uint32_t b = __reduce_min_sync(0xffffffffu, w);
      if (kInlineWindows && (b != 0xFFFFFFFFu) & ((b & (1u << 26)) != 0u) & (x != 0) & cur.f) {
        // (c) a window that is not clear, settled here (window_cell's
        // decision) when the record closes it; the left neighbour's Lab comes
        // from the previous record's entry it was chosen as, else the palette
        win_tried = true;
        const CellRecord& Rc = rec[c & (R - 1)];
        const int e0 = (int)(b >> 27);
        const float b0 = __fadd_rn(Rc.wd[e0], two_w);
        if (Rc.f_next >= b0) {
          const float dl = Rc.wd[lane];
          const bool in = (w != 0xFFFFFFFFu) & (lane >= e0) & (dl < b0);
          const float4 lab_left = last_pos >= 0 ? rec[(c - 1) & (R - 1)].wl[last_pos] : lab(last);
          const float pen = __fadd_rn(Rc.wu[lane], wgt(Rc.wl[lane], lab_left));  // 0 + w_up, then + w_left
          const uint32_t sb = in ? __float_as_uint(__fadd_rn(dl, __fmul_rn(pen, weight))) : 0xFFFFFFFFu;
          const uint32_t mn = __reduce_min_sync(0xffffffffu, sb);
          const uint32_t wn = __reduce_min_sync(0xffffffffu, (in & (sb == mn)) ? w : 0xFFFFFFFFu);
          const uint32_t pk = (mn == 0xFFFFFFFFu ? b : wn) & ~(1u << 26);
          if (((pk >> 16) & 1023u) != 1023u) b = pk;  // a counter that fits its field
        }
      }
      fast = (b != 0xFFFFFFFFu) & !(b & (1u << 26));
      if (!fast || !h1_ok) {
        // the record's key form for the uncommon path; a row start is redone there
        chosen = b != 0xFFFFFFFFu ? (((b >> 27) << 17) | (((b >> 26) & 1u) << 16) | (b & 0xFFFFu)) : b;
        fast = fast && x != 0;
        break;
      }
      const int t = (int)(b & 0xFFFFu);
      usage[t] = ((b >> 16) & 1023u) + 1u;
      place(c, t);
      if (kInlineWindows) {
        last_pos = cur.f ? (int)(b >> 27) : -1;
        win_tried = false;
      }
      last = t;
      cur = nxt;
      wc = words(nxt);
      cur_fresh = false;
      h1 = h2;
      h1_ok = h2_ok;
      const bool wrap = x + 1 == gw;
      x = wrap ? 0 : x + 1;
      y += wrap ? 1 : 0;
      if (++c == n) break;
    }
    if (c == n) break;
    // ---- the uncommon path for cell c
    int t = (int)(chosen & 0xFFFFu);
    if (fast) {
      // only the next record was late
      if (lane == (int)(chosen >> 17)) {
        usage[cur.ti] = cur.ui + 1u;
        place(c, t);
      }
    } else {
      const bool row_start = x == 0;
      bool done = false;
      if (row_start) {
        // no left neighbour: the previous commit's counter counts
        const uint32_t ui = cur.ui + ((!cur_fresh && cur.ti == (uint32_t)last && cur.key != 0xFFFFFFFFu) ? 1u : 0u);
        const uint32_t b = __reduce_min_sync(0xffffffffu, ui < max_usage ? cur.key : 0xFFFFFFFFu);
        if (b != 0xFFFFFFFFu && !(b & 0x10000u)) {
          t = (int)(b & 0xFFFFu);
          if (lane == (int)(b >> 17)) {
            usage[cur.ti] = ui + 1u;
            place(c, t);
          }
          done = true;
        }
      }
      if (!done && !win_tried && !row_start && chosen != 0xFFFFFFFFu && (chosen & 0x10000u) &&
          rec[c & (R - 1)].epoch == epoch) {
        const int tw = window_cell(c, cur, last, y > 0, (int)(chosen >> 17));
        if (tw >= 0) {
          t = tw;
          done = true;
        }
      }
      if (!done) {
        const int up = y == 0 ? -1 : kRing ? (int)(ring[(c - gw) & cmask] & 0xFFFFu) : (int)grid16[c - gw];
        if (kLabSmem)
          t = full_cell(lab, J.cand_idx + (size_t)c * k, J.cand_dist + (size_t)c * k, k, p, up,
                        row_start ? -1 : last, usage, max_usage, weight, ctrl, epoch, resets, lane);
        else
          t = full_cell_rows(lab, J.cand_idx + (size_t)c * k, J.cand_dist + (size_t)c * k, k, p, up,
                             row_start ? -1 : last, usage, max_usage, weight, ctrl, epoch, resets, lane);
        if (lane == 0) place(c, t);
      }
    }
    __syncwarp();
    bool nxt_fresh = false;
    if (c + 1 < n) {
      if (!h1_ok) {
        h1_ok = ready(c + 1, true);
        h1 = load_head(c + 1);
      }
      // the counters moved (a full evaluation), or the record came late: read afresh
      nxt = finish(h1);
      nxt_fresh = true;
      // look ahead for the records of the coming cells (one probe covers 32)
      if (ready_until < n && ready_until <= c + 32) (void)ready(ready_until, false);
      if (!h2_ok && c + 2 < ready_until) {
        h2_ok = true;
        h2 = load_head(c + 2);
      }
    }
    last = t;
    last_pos = -1;
    cur = nxt;
    cur_fresh = nxt_fresh;
    h1 = h2;
    h1_ok = h2_ok;
    const bool wrap = x + 1 == gw;
    x = wrap ? 0 : x + 1;
    y += wrap ? 1 : 0;
    ++c;
  }
  if (aborted) {
    if (lane == 0) {
      atomicOr(err, kErrTimeout);
      *reinterpret_cast<volatile uint32_t*>(&ctrl[kAbort]) = 1u;
    }
    // every cell empty, so the stages after the walk read no stale index (in
    // the 16-bit grid form the cost warp writes the global grid)
    if (kRing)
      for (int i = lane; i < n; i += 32) J.grid[i] = -1;
    if (lane == 0 && J.n_resets) *J.n_resets = 0;
  } else {
    // the placed grid in global memory (every lane's stores visible) before the
    // completion the scout CTA waits for; in the 16-bit grid form the cost warp
    // writes it
    if (kRing) __threadfence();
    if (lane == 0 && J.n_resets) *J.n_resets = resets;
    __syncwarp();
    if (lane == 0) st_release_cluster(smem_u32(&ctrl[kProgress]), (uint32_t)n);
  }
  cluster_sync_all();  // the scouts are done with this CTA's shared memory
}

}  // namespace

size_t greedy_shared_bytes(int k, int gw, int p, bool lab_smem, bool usage_smem) {
  return greedy_smem_bytes(k, gw, p, lab_smem, usage_smem);
}

bool greedy_scouted_fits(int gw, int n, int p) {
  constexpr size_t kMaxSmem = 220 * 1024;
  // the largest ring any row width uses, the palette Lab outside shared memory
  return gw >= 8 && p <= 65535 &&
         (pair_smem_bytes(gw, n, p, false, false) <= kMaxSmem || pair_smem_bytes(gw, n, p, false, true) <= kMaxSmem);
}

int launch_greedy(const float4* pal, int p, const GreedyJob* jobs_dev, int n_jobs, int k, int max_gw,
                  int max_cells, uint32_t* usage_scratch, uint32_t* err, cudaStream_t stream, bool one_warp,
                  bool inject_timeout) {
  if (n_jobs <= 0) return MG_OK;
  if (k < 1 || k > 100) return fail(MG_ERR_ARG, "candidate count must be in 1..100");
  constexpr size_t kMaxSmem = 220 * 1024;
  static int configured_device = -1, sms = 0;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    const int m = (int)kMaxSmem;
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<true, true>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<false, true>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<false, false>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<true, false, 4, 16>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<false, false, 4, 16>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<true, true, 4, 16>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<false, true, 4, 16>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<true, false, 2, 32>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<false, false, 2, 32>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<true, true, 2, 32>, a, m));
    MG_CUDA(cudaFuncSetAttribute(greedy_pair_kernel<false, true, 2, 32>, a, m));
    MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    configured_device = dev;
  }
  // The scouted walk: counters in shared memory, 16-bit palette indices, rows
  // of at least 8 cells.
  if (!one_warp && max_gw >= 8 && p <= 65535) {
    // the grid before the ring (a shorter walker loop), the palette Lab in shared memory before global
    const bool fit[4] = {pair_smem_bytes(max_gw, max_cells, p, true, false) <= kMaxSmem,
                         pair_smem_bytes(max_gw, max_cells, p, false, false) <= kMaxSmem,
                         pair_smem_bytes(max_gw, max_cells, p, true, true) <= kMaxSmem,
                         pair_smem_bytes(max_gw, max_cells, p, false, true) <= kMaxSmem};
    const int form = fit[0] ? 0 : fit[1] ? 1 : fit[2] ? 2 : fit[3] ? 3 : -1;
    if (form >= 0) {
      const bool lab_smem = form == 0 || form == 2, ring = form >= 2;
      const size_t bytes = pair_smem_bytes(max_gw, max_cells, p, lab_smem, ring);
      const uint32_t polls = inject_timeout ? kInjectedWalkPolls : kWalkPolls, hold = inject_timeout ? 1u : 0u;
      // five SMs a mosaic while every cluster finds room at once, else three
      const bool wide = 5 * n_jobs <= sms;
      auto go = [&](auto kernel, int ctas, int threads) {
        kernel<<<(unsigned)(ctas * n_jobs), threads, bytes, stream>>>(pal, p, jobs_dev, err, polls, hold);
      };
      if (wide) {
        if (form == 0) go(greedy_pair_kernel<true, false, 4, 16>, 5, 512);
        else if (form == 1) go(greedy_pair_kernel<false, false, 4, 16>, 5, 512);
        else if (form == 2) go(greedy_pair_kernel<true, true, 4, 16>, 5, 512);
        else go(greedy_pair_kernel<false, true, 4, 16>, 5, 512);
      } else {
        if (form == 0) go(greedy_pair_kernel<true, false, 2, 32>, 3, 1024);
        else if (form == 1) go(greedy_pair_kernel<false, false, 2, 32>, 3, 1024);
        else if (form == 2) go(greedy_pair_kernel<true, true, 2, 32>, 3, 1024);
        else go(greedy_pair_kernel<false, true, 2, 32>, 3, 1024);
      }
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
