// k_nearest_grid.cu -- (b) the k-nearest palette search of main.rs:145-151 /
// 348-352 (kiddo nearest_n::<SquaredEuclidean>, k = min(P, 100)) through a
// bucket grid over the palette's Lab colours, for palettes much larger than k.
//
// The result is the scan's (k_scan.cu) bit for bit: the k smallest 64-bit keys
// (distance bits, palette index) over the whole palette.  The grid only decides
// which entries are looked at, and every entry it skips provably has a distance
// above the k-th:
//  - Index (one CTA, lab_grid_build_kernel): the palette's bounding box split
//    into g x g x g buckets; entries counting-sorted by bucket into `sorted`
//    (x, y, z, palette index as bits); `start[b]` the first entry of bucket b
//    (b = (z * g + y) * g + x), so a row of buckets along x is one contiguous
//    run of entries.
//  - Query (one warp per query): first the smallest cube of buckets around the
//    query's bucket that holds at least k entries, which fixes a k-th distance
//    t; then every bucket of the box [q - R, q + R] (R = sqrt(t) widened by a
//    relative 1e-3 and an absolute 1e-3) not already scanned.  An entry outside
//    that box differs from q by more than R on some axis, so its rounded
//    squared distance exceeds t (the rounding of one subtraction, one square
//    and two sums is below 1e-6 relative) and it cannot be among the k nearest.
//    The box edges fl(q -+ R) carry an absolute error of |q| * 2^-24, which the
//    1e-3 widening covers while |q| * 6e-8 < 1e-3 * (sqrt(t) + 1), i.e. for
//    colour components below 1.6e4 in magnitude (Lab's are within +-130).
//  - Each batch of 32 row segments (two per row: the box row minus the part of
//    it inside the cube already scanned) is prefix-summed across the warp, and
//    the warp walks the concatenated entries 32 at a time, each lane finding
//    its segment by a five-step shuffle search.  Keys go through the warp's
//    top-k list (topk_warp.cuh) exactly as in the scan.
#include <cmath>

#include "mg_internal.h"
#include "topk_warp.cuh"

namespace mg {
namespace {

constexpr int kGridWarps = 16;
constexpr int kGridThreads = kGridWarps * 32;
constexpr int kBoxFactor = 1;   // the first cube holds >= kBoxFactor * k entries
constexpr int kMaxGridDim = 24; // start[] of 24^3 + 1 ints stays in shared memory
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int grid_coord(float v, float lo, float inv, int g) {
  const float t = floorf(__fmul_rn(__fsub_rn(v, lo), inv));
  return (int)fminf(fmaxf(t, 0.0f), (float)(g - 1));  // NaN -> 0
}

struct Box {
  int x0, x1, y0, y1, z0, z1;  // inclusive bucket ranges
};

__device__ __forceinline__ bool box_is_all(const Box& b, int g) {
  return b.x0 == 0 && b.y0 == 0 && b.z0 == 0 && b.x1 == g - 1 && b.y1 == g - 1 && b.z1 == g - 1;
}

// ---- index build (one CTA) --------------------------------------------------------
__global__ void __launch_bounds__(1024) lab_grid_build_kernel(const float4* __restrict__ pal, int p, int g,
                                                              LabGrid* __restrict__ hdr, float4* __restrict__ sorted,
                                                              int* __restrict__ start) {
  extern __shared__ int cnt[];  // g^3 counts, then cursors
  __shared__ float red[6][32];
  __shared__ int part[1024];
  __shared__ LabGrid H;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int nb = g * g * g;
  float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int i = tid; i < p; i += blockDim.x) {
    const float4 e = pal[i];
    v[0] = fminf(v[0], e.x), v[1] = fminf(v[1], e.y), v[2] = fminf(v[2], e.z);
    v[3] = fmaxf(v[3], e.x), v[4] = fmaxf(v[4], e.y), v[5] = fmaxf(v[5], e.z);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[c] = fminf(v[c], __shfl_xor_sync(kFull, v[c], o));
      v[c + 3] = fmaxf(v[c + 3], __shfl_xor_sync(kFull, v[c + 3], o));
    }
  }
  if (lane == 0)
    for (int c = 0; c < 6; ++c) red[c][warp] = v[c];
  for (int b = tid; b < nb; b += blockDim.x) cnt[b] = 0;
  __syncthreads();
  if (tid == 0) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int w = 0; w < nw; ++w)
      for (int c = 0; c < 3; ++c) lo[c] = fminf(lo[c], red[c][w]), hi[c] = fmaxf(hi[c], red[c + 3][w]);
    for (int c = 0; c < 3; ++c) {
      const float ext = __fsub_rn(hi[c], lo[c]);
      H.lo[c] = lo[c];
      H.inv[c] = ext > 0.0f ? __fdiv_rn((float)g, ext) : 0.0f;
    }
    H.g = g;
    H.p = p;
    *hdr = H;
  }
  __syncthreads();
  auto bucket = [&](const float4& e) {
    return (grid_coord(e.z, H.lo[2], H.inv[2], g) * g + grid_coord(e.y, H.lo[1], H.inv[1], g)) * g +
           grid_coord(e.x, H.lo[0], H.inv[0], g);
  };
  for (int i = tid; i < p; i += blockDim.x) atomicAdd(&cnt[bucket(pal[i])], 1);
  __syncthreads();
  // exclusive scan: thread t owns buckets [t * per, (t + 1) * per)
  const int per = (nb + blockDim.x - 1) / blockDim.x;
  const int b0 = min(nb, tid * per), b1 = min(nb, b0 + per);
  int sum = 0;
  for (int b = b0; b < b1; ++b) sum += cnt[b];
  part[tid] = sum;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const int add = tid >= o ? part[tid - o] : 0;
    __syncthreads();
    part[tid] += add;
    __syncthreads();
  }
  int run = part[tid] - sum;
  for (int b = b0; b < b1; ++b) {
    const int c = cnt[b];
    start[b] = run;
    cnt[b] = run;
    run += c;
  }
  if (tid == 0) start[nb] = p;
  __syncthreads();
  // scatter; the order inside a bucket is free: keys carry the palette index
  for (int i = tid; i < p; i += blockDim.x) {
    const float4 e = pal[i];
    const int pos = atomicAdd(&cnt[bucket(e)], 1);
    sorted[pos] = make_float4(e.x, e.y, e.z, __int_as_float(i));
  }
}

// ---- query ----------------------------------------------------------------------------
// Entries in box `o` (bucket ranges) minus box `in` (when has_in), into the
// warp's top-k list.
__device__ __forceinline__ void scan_box(const int* start, int g, const Box& o, const Box& in, bool has_in,
                                         const float4* __restrict__ sorted, const float4& q, WarpLists& W,
                                         int& len, int& nbuf, unsigned long long& thr, int k, int lane) {
  const int ny = o.y1 - o.y0 + 1, nz = o.z1 - o.z0 + 1;
  const int nseg = ny * nz * 2;
  for (int sb = 0; sb < nseg; sb += 32) {
    const int si = sb + lane;
    int beg = 0, n = 0;
    if (si < nseg) {
      const int row = si >> 1, partno = si & 1;
      const int z = o.z0 + row / ny, y = o.y0 + row % ny;
      int xa = o.x0, xb = o.x1;
      const bool inner = has_in && y >= in.y0 && y <= in.y1 && z >= in.z0 && z <= in.z1;
      if (!inner) {
        if (partno) xb = xa - 1;
      } else if (partno == 0) {
        xb = min(o.x1, in.x0 - 1);
      } else {
        xa = max(o.x0, in.x1 + 1);
      }
      if (xa <= xb) {
        const int rb = (z * g + y) * g;
        beg = start[rb + xa];
        n = start[rb + xb + 1] - beg;
      }
    }
    int incl = n;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += t;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    const int excl = incl - n;
    const int delta = beg - excl;  // entry index = position in the concatenation + delta of its segment
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      int j = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int e = __shfl_sync(kFull, excl, j + step);
        if (e <= t) j += step;
      }
      const int dj = __shfl_sync(kFull, delta, j);
      unsigned long long key = kMaxKey;
      if (t < total) {
        const float4 e = __ldg(&sorted[t + dj]);
        key = ((unsigned long long)__float_as_uint(sq_dist(q.x, q.y, q.z, e.x, e.y, e.z)) << 32) |
              (unsigned)__float_as_int(e.w);
      }
      const bool pass = key < thr;
      const unsigned mask = __ballot_sync(kFull, pass);
      if (mask) {
        const int pos = nbuf + __popc(mask & ((1u << lane) - 1u));
        if (pass) W.buf[pos] = key;
        nbuf += __popc(mask);
        __syncwarp();
        if (nbuf > kBufCap - 32) warp_merge(W, len, nbuf, thr, k, lane);
      }
    }
  }
}

// ---- the select-then-sort query ------------------------------------------------------------
// Most queries take this form: their candidate keys are gathered into the
// warp's flat buffer (the WarpLists memory, kGatherCap keys), the k-th
// distance among them is found by bisection on the distance bits (a warp
// count per step), the buffer is cut to the keys at or below it, and one
// bitonic sort of what is left gives the k smallest keys -- instead of the
// top-k list's repeated sorts and merges.  A query whose candidates do not fit
// takes the list form (scan_box + warp_merge), which gives the same keys.
constexpr int kGatherCap = 3 * kListCap;  // list, tmp and buf of WarpLists, contiguous

// Appends the keys of box o (minus box in, when has_in) whose distance bits
// are at most dthr to buf[n..); returns the new count (beyond cap: nothing
// past cap was stored, the caller falls back).
__device__ __forceinline__ int gather_box(const int* start, int g, const Box& o, const Box& in, bool has_in,
                                          const float4* __restrict__ sorted, const float4& q,
                                          unsigned long long* buf, int n, int cap, uint32_t dthr, int lane) {
  const int ny = o.y1 - o.y0 + 1, nz = o.z1 - o.z0 + 1;
  const int nseg = ny * nz * 2;
  for (int sb = 0; sb < nseg; sb += 32) {
    const int si = sb + lane;
    int beg = 0, cnt = 0;
    if (si < nseg) {
      const int row = si >> 1, partno = si & 1;
      const int z = o.z0 + row / ny, y = o.y0 + row % ny;
      int xa = o.x0, xb = o.x1;
      const bool inner = has_in && y >= in.y0 && y <= in.y1 && z >= in.z0 && z <= in.z1;
      if (!inner) {
        if (partno) xb = xa - 1;
      } else if (partno == 0) {
        xb = min(o.x1, in.x0 - 1);
      } else {
        xa = max(o.x0, in.x1 + 1);
      }
      if (xa <= xb) {
        const int rb = (z * g + y) * g;
        beg = start[rb + xa];
        cnt = start[rb + xb + 1] - beg;
      }
    }
    int incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int t = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += t;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    const int excl = incl - cnt;
    const int delta = beg - excl;
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      int j = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int e = __shfl_sync(kFull, excl, j + step);
        if (e <= t) j += step;
      }
      const int dj = __shfl_sync(kFull, delta, j);
      unsigned long long key = kMaxKey;
      if (t < total) {
        const float4 e = __ldg(&sorted[t + dj]);
        key = ((unsigned long long)__float_as_uint(sq_dist(q.x, q.y, q.z, e.x, e.y, e.z)) << 32) |
              (unsigned)__float_as_int(e.w);
      }
      const bool pass = t < total && (uint32_t)(key >> 32) <= dthr;
      const unsigned mask = __ballot_sync(kFull, pass);
      const int pos = n + __popc(mask & ((1u << lane) - 1u));
      if (pass && pos < cap) buf[pos] = key;
      n += __popc(mask);
    }
  }
  __syncwarp();
  return n;
}

// The smallest distance D (as bits) with at least k of buf[0..n) at or below
// it (k <= n <= kGatherCap): bisection between the smallest and the largest.
__device__ uint32_t kth_dist_bits(const unsigned long long* buf, int n, int k, int lane) {
  constexpr int kPer = kGatherCap / 32;
  uint32_t d[kPer];
  uint32_t mn = 0xFFFFFFFFu, mx = 0u;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int i = lane + 32 * j;
    d[j] = i < n ? (uint32_t)(buf[i] >> 32) : 0xFFFFFFFFu;
    if (i < n) {
      mn = min(mn, d[j]);
      mx = max(mx, d[j]);
    }
  }
  uint32_t lo = __reduce_min_sync(kFull, mn), hi = __reduce_max_sync(kFull, mx);
  while (lo < hi) {  // warp-uniform
    const uint32_t mid = lo + ((hi - lo) >> 1);
    unsigned c = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) c += d[j] <= mid ? 1u : 0u;
    if ((int)__reduce_add_sync(kFull, c) >= k) hi = mid;
    else lo = mid + 1u;
  }
  return lo;
}

// Keeps the keys of buf[0..n) whose distance bits are at most dthr (in order);
// returns their count.
__device__ __forceinline__ int cut_keys(unsigned long long* buf, int n, uint32_t dthr, int lane) {
  int m = 0;
  for (int b = 0; b < n; b += 32) {
    const int i = b + lane;
    const unsigned long long key = i < n ? buf[i] : kMaxKey;
    const bool keep = i < n && (uint32_t)(key >> 32) <= dthr;
    const unsigned mask = __ballot_sync(kFull, keep);
    __syncwarp();
    if (keep) buf[m + __popc(mask & ((1u << lane) - 1u))] = key;
    m += __popc(mask);
    __syncwarp();
  }
  return m;
}

// Entries in the rows of box b, summed over the warp.
__device__ __forceinline__ int count_box(const int* start, int g, const Box& b, int lane) {
  const int ny = b.y1 - b.y0 + 1, rows = ny * (b.z1 - b.z0 + 1);
  int c = 0;
  for (int r = lane; r < rows; r += 32) {
    const int rb = ((b.z0 + r / ny) * g + b.y0 + r % ny) * g;
    c += start[rb + b.x1 + 1] - start[rb + b.x0];
  }
  return (int)__reduce_add_sync(kFull, (unsigned)c);
}

__global__ void __launch_bounds__(kGridThreads, 2) nearest_grid_kernel(
    const LabGrid* __restrict__ hdr, const float4* __restrict__ sorted, const int* __restrict__ start_g,
    const float4* __restrict__ queries, int nq, int k, int out_stride, uint32_t* __restrict__ out_idx,
    float* __restrict__ out_dist) {
  extern __shared__ __align__(16) uint8_t smem[];
  WarpLists* lists = reinterpret_cast<WarpLists*>(smem);
  int* start = reinterpret_cast<int*>(smem + kGridWarps * sizeof(WarpLists));
  const LabGrid H = *hdr;
  const int g = H.g, nb = g * g * g;
  for (int i = threadIdx.x; i <= nb; i += blockDim.x) start[i] = start_g[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpLists& W = lists[warp];
  const int target = min(H.p, kBoxFactor * k);
  for (int qi = blockIdx.x * kGridWarps + warp; qi < nq; qi += gridDim.x * kGridWarps) {
    const float4 q = queries[qi];
    int len = 0, nbuf = 0;
    unsigned long long thr = kMaxKey;
    const bool finite = isfinite(q.x) && isfinite(q.y) && isfinite(q.z);
    const int cx = grid_coord(q.x, H.lo[0], H.inv[0], g), cy = grid_coord(q.y, H.lo[1], H.inv[1], g),
              cz = grid_coord(q.z, H.lo[2], H.inv[2], g);
    Box c{0, g - 1, 0, g - 1, 0, g - 1};
    int cube_n = H.p;
    if (finite) {
      for (int s = 0;; ++s) {
        c = Box{max(cx - s, 0), min(cx + s, g - 1), max(cy - s, 0), min(cy + s, g - 1), max(cz - s, 0),
                min(cz + s, g - 1)};
        if (box_is_all(c, g)) break;
        cube_n = count_box(start, g, c, lane);
        if (cube_n >= target) break;
      }
      if (box_is_all(c, g)) cube_n = H.p;
    }
    // ---- select, then sort (the common form)
    unsigned long long* fb = W.list;  // kGatherCap keys
    bool done = false;
    if (cube_n <= kGatherCap) {
      int m = gather_box(start, g, c, c, false, sorted, q, fb, 0, kGatherCap, 0xFFFFFFFFu, lane);
      bool fits = m <= kGatherCap;
      if (fits && m > 0 && !box_is_all(c, g)) {
        // the cube holds >= min(P, k) entries: its k-th distance bounds the search
        const uint32_t dk = kth_dist_bits(fb, m, min(k, m), lane);
        m = cut_keys(fb, m, dk, lane);
        if (m >= k) {
          const float r = __fsqrt_rn(__uint_as_float(dk));
          const float R = __fadd_rn(__fmul_rn(r, 1.001f), 1e-3f);
          const Box o{grid_coord(__fsub_rn(q.x, R), H.lo[0], H.inv[0], g), grid_coord(__fadd_rn(q.x, R), H.lo[0], H.inv[0], g),
                      grid_coord(__fsub_rn(q.y, R), H.lo[1], H.inv[1], g), grid_coord(__fadd_rn(q.y, R), H.lo[1], H.inv[1], g),
                      grid_coord(__fsub_rn(q.z, R), H.lo[2], H.inv[2], g), grid_coord(__fadd_rn(q.z, R), H.lo[2], H.inv[2], g)};
          m = gather_box(start, g, o, c, true, sorted, q, fb, m, kGatherCap, dk, lane);
        } else {
          // fewer than k in the cube (palette below k): every entry counts
          const Box all{0, g - 1, 0, g - 1, 0, g - 1};
          m = gather_box(start, g, all, c, true, sorted, q, fb, m, kGatherCap, 0xFFFFFFFFu, lane);
        }
        fits = m <= kGatherCap;
      }
      if (fits && m > 0) {
        const int kk = min(k, m);
        const uint32_t d2 = kth_dist_bits(fb, m, kk, lane);
        m = cut_keys(fb, m, d2, lane);  // the k smallest keys and their ties at the k-th distance
        int mp = 1;
        while (mp < m) mp <<= 1;
        if (mp <= kGatherCap) {
          for (int i = m + lane; i < mp; i += 32) fb[i] = kMaxKey;
          __syncwarp();
          warp_bitonic_sort(fb, mp, lane);
          len = kk;
          done = true;
        }
      } else if (fits) {
        len = 0;
        done = true;
      }
    }
    if (!done) {
      // ---- the top-k list form (candidates beyond the buffer)
      len = 0;
      nbuf = 0;
      thr = kMaxKey;
      scan_box(start, g, c, c, false, sorted, q, W, len, nbuf, thr, k, lane);
      if (!box_is_all(c, g)) {
        __syncwarp();
        warp_merge(W, len, nbuf, thr, k, lane);
        // the cube holds >= min(P, k) entries: len == k unless P < k
        const float r = __fsqrt_rn(__uint_as_float((uint32_t)(thr >> 32)));
        const float R = __fadd_rn(__fmul_rn(r, 1.001f), 1e-3f);
        const Box o = len < k ? Box{0, g - 1, 0, g - 1, 0, g - 1} : Box{grid_coord(__fsub_rn(q.x, R), H.lo[0], H.inv[0], g), grid_coord(__fadd_rn(q.x, R), H.lo[0], H.inv[0], g),
                    grid_coord(__fsub_rn(q.y, R), H.lo[1], H.inv[1], g), grid_coord(__fadd_rn(q.y, R), H.lo[1], H.inv[1], g),
                    grid_coord(__fsub_rn(q.z, R), H.lo[2], H.inv[2], g), grid_coord(__fadd_rn(q.z, R), H.lo[2], H.inv[2], g)};
        scan_box(start, g, o, c, true, sorted, q, W, len, nbuf, thr, k, lane);
      }
      __syncwarp();
      warp_merge(W, len, nbuf, thr, k, lane);
    }
    for (int i = lane; i < out_stride; i += 32) {
      const unsigned long long key = i < len ? W.list[i] : kMaxKey;
      out_idx[(size_t)qi * out_stride + i] = i < len ? (uint32_t)key : 0xFFFFFFFFu;
      out_dist[(size_t)qi * out_stride + i] = i < len ? __uint_as_float((uint32_t)(key >> 32)) : __int_as_float(0x7f800000);
    }
    __syncwarp();
  }
}

size_t grid_query_smem(int g) { return kGridWarps * sizeof(WarpLists) + sizeof(int) * ((size_t)g * g * g + 1); }

}  // namespace

int lab_grid_dim(int method, int p, int k) {
  if (p <= 0 || method == kNearestScan) return 0;
  if (method == kNearestAuto && (p < 2048 || p < 16 * k)) return 0;
  const int g = (int)std::lround(std::cbrt(p / 2.0));
  return std::max(1, std::min(kMaxGridDim, g));
}

int LabIndex::build(const float4* pal, int p, int method, int k, cudaStream_t s) {
  g = lab_grid_dim(method, p, k);
  if (g == 0) return MG_OK;
  const int nb = g * g * g;
  MG_CHECK(hdr.ensure(sizeof(LabGrid)));
  MG_CHECK(sorted.ensure(sizeof(float4) * p));
  MG_CHECK(start.ensure(sizeof(int) * (nb + 1)));
  const size_t smem = sizeof(int) * nb;
  static int configured_device = -1;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    MG_CUDA(cudaFuncSetAttribute(lab_grid_build_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(int) * kMaxGridDim * kMaxGridDim * kMaxGridDim)));
    MG_CUDA(cudaFuncSetAttribute(nearest_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)grid_query_smem(kMaxGridDim)));
    configured_device = dev;
  }
  lab_grid_build_kernel<<<1, 1024, smem, s>>>(pal, p, g, hdr.as<LabGrid>(), sorted.as<float4>(), start.as<int>());
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

void LabIndex::release() {
  hdr.release();
  sorted.release();
  start.release();
  g = 0;
}

int launch_nearest_grid(const LabIndex& index, const float4* queries, int nq, int keff, int k, uint32_t* idx,
                        float* dist, cudaStream_t stream) {
  const size_t smem = grid_query_smem(index.g);
  int dev = 0, sms = 0, per_sm = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nearest_grid_kernel, kGridThreads, smem));
  if (per_sm < 1) per_sm = 1;
  const int groups = (nq + kGridWarps - 1) / kGridWarps;
  const int grid = std::min(groups, sms * per_sm);
  nearest_grid_kernel<<<grid, kGridThreads, smem, stream>>>(index.hdr.as<LabGrid>(), index.sorted.as<float4>(),
                                                            index.start.as<int>(), queries, nq, keff, k, idx, dist);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
