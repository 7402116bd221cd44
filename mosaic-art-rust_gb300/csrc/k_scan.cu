// k_scan.cu -- (b) brute-force k-nearest scan over the material palette,
// replacing the kiddo k-d tree query of main.rs:145-151 / 348-352
// (nearest_n::<SquaredEuclidean>, k = min(P, 100)).
//
// Lab is 3-D, so the scan is SM/L1 work, not a contraction.  Design:
//  - The palette (float4 per material) is streamed into shared memory in
//    chunks of kChunk entries by TMA bulk copies (cp.async.bulk, completion on
//    an mbarrier), double-buffered.  When the palette fits in the two stages it
//    is loaded once and stays resident for every query the CTA handles.
//  - One warp per query.  Each lane computes squared distances with no fused
//    multiply-add (the reference's evaluation order), packs (distance bits,
//    index) into a 64-bit key -- distances are non-negative, so key order is
//    (distance, index) order and ties go to the lowest index -- and appends keys
//    below the current k-th best to a per-warp buffer.  A full buffer is
//    bitonic-sorted and merged into the sorted top-k list (merge-path ranks).
#include <algorithm>

#include "mg_internal.h"
#include "mg_ptx.cuh"
#include "topk_warp.cuh"

namespace mg {
namespace {

constexpr int kWarps = 16;
constexpr int kThreads = kWarps * 32;

template <int kChunk>
constexpr size_t smem_bytes() { return 2 * kChunk * sizeof(float4) + 16 + kWarps * sizeof(WarpLists); }

template <int kChunk>  // palette entries per shared-memory stage
__global__ void __launch_bounds__(kThreads) nearest_kernel(const float4* __restrict__ pal, int p,
                                                           const float4* __restrict__ queries, int nq, int k,
                                                           int out_stride, uint32_t* __restrict__ out_idx,
                                                           float* __restrict__ out_dist, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t smem[];
  float4* stage0 = reinterpret_cast<float4*>(smem);

  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + 2 * kChunk * sizeof(float4));
  WarpLists* lists = reinterpret_cast<WarpLists*>(smem + 2 * kChunk * sizeof(float4) + 16);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nchunks = (p + kChunk - 1) / kChunk;
  const bool resident = nchunks <= 2;
  const int ngroups = (nq + kWarps - 1) / kWarps;
  const int my_groups = blockIdx.x < ngroups ? (ngroups - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const long long total_seq = (long long)my_groups * nchunks;

  auto chunk_len = [=](int c) { return min(kChunk, p - c * kChunk); };
  auto issue = [=](int s, int c) {
    const uint32_t bytes = (uint32_t)chunk_len(c) * sizeof(float4);
    mbar_arrive_expect_tx(&bars[s], bytes);
    tma_load_1d(stage0 + s * kChunk, pal + (size_t)c * kChunk, bytes, &bars[s]);
  };

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && total_seq > 0) {
    if (resident) {
      for (int c = 0; c < nchunks; ++c) issue(c, c);
    } else {
      issue(0, 0);
      if (total_seq > 1) issue(1, 1 % nchunks);
    }
  }
  uint32_t parity = 0u;  // bit s: phase parity of stage s
  if (resident && total_seq > 0) {
    for (int c = 0; c < nchunks; ++c) {
      if (!mbar_wait_bounded(&bars[c], 0)) {
        atomicOr(err, kErrTimeout);
        return;
      }
    }
  }

  WarpLists& W = lists[warp];
  long long seq = 0;
  for (int g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int qi = g * kWarps + warp;
    const bool active = qi < nq;
    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
    if (active) q = queries[qi];
    int len = 0, nbuf = 0;
    unsigned long long thr = kMaxKey;
    for (int c = 0; c < nchunks; ++c, ++seq) {
      const int s = resident ? c : (int)(seq & 1);
      if (!resident) {
        if (!mbar_wait_bounded(&bars[s], (parity >> s) & 1u)) {
          atomicOr(err, kErrTimeout);
          return;
        }
        parity ^= 1u << s;
      }
      const float4* sp = stage0 + s * kChunk;
      const int n = chunk_len(c);
      const int gbase = c * kChunk;
      if (active) {
        // 8 entries per lane per step; in steady state the k-th best is tight and
        // a single warp vote rejects all 256 entries.
        for (int base = 0; base < n; base += 256) {
          uint32_t db[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int j = base + u * 32 + lane;
            db[u] = 0xFFFFFFFFu;
            if (j < n) {
              const float4 e = sp[j];
              db[u] = __float_as_uint(sq_dist(q.x, q.y, q.z, e.x, e.y, e.z));
            }
          }
          const uint32_t thr_d = (uint32_t)(thr >> 32), thr_i = (uint32_t)thr;
          bool anyp = false;
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const uint32_t gi = (uint32_t)(gbase + base + u * 32 + lane);
            anyp = anyp || db[u] < thr_d || (db[u] == thr_d && gi < thr_i);
          }
          if (__any_sync(0xffffffffu, anyp)) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int j = base + u * 32 + lane;
              const unsigned long long key =
                  j < n ? (((unsigned long long)db[u] << 32) | (unsigned)(gbase + j)) : kMaxKey;
              const bool pass = key < thr;
              const unsigned mask = __ballot_sync(0xffffffffu, pass);
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
      }
      if (!resident) {
        fence_proxy_async_smem();
        __syncthreads();  // every warp is done with stage s
        if (threadIdx.x == 0 && seq + 2 < total_seq) issue(s, (int)((seq + 2) % nchunks));
      }
    }
    if (active) {
      __syncwarp();
      warp_merge(W, len, nbuf, thr, k, lane);
      for (int i = lane; i < out_stride; i += 32) {
        unsigned long long key = i < len ? W.list[i] : kMaxKey;
        out_idx[(size_t)qi * out_stride + i] = i < len ? (uint32_t)key : 0xFFFFFFFFu;
        out_dist[(size_t)qi * out_stride + i] = i < len ? __uint_as_float((uint32_t)(key >> 32)) : __int_as_float(0x7f800000);
      }
      __syncwarp();
    }
  }
}

template <int kChunk>
int launch_nearest_t(const float4* pal, int p, const float4* queries, int nq, int keff, int k, uint32_t* idx, float* dist,
                     uint32_t* err, cudaStream_t stream) {
  constexpr size_t kSmem = smem_bytes<kChunk>();
  static int configured_device = -1;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    MG_CUDA(cudaFuncSetAttribute(nearest_kernel<kChunk>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
    configured_device = dev;
  }
  int sms = 0, per_sm = 0;
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  MG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nearest_kernel<kChunk>, kThreads, kSmem));
  if (per_sm < 1) per_sm = 1;
  const int ngroups = (nq + kWarps - 1) / kWarps;
  const int grid = min(ngroups, sms * per_sm);
  // Rows shorter than k (p < k) are padded by the kernel with index ~0 / +inf.
  nearest_kernel<kChunk><<<grid, kThreads, kSmem, stream>>>(pal, p, queries, nq, keff, k, idx, dist, err);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace

namespace {
// The GUI generator's colour term (gui/app_full.rs:1435-1440): the square root
// of each candidate's squared distance, correctly rounded like f32::sqrt.
__global__ void __launch_bounds__(256) sqrt_inplace_kernel(float* __restrict__ v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = __fsqrt_rn(v[i]);
}
}  // namespace

int launch_sqrt_inplace(float* v, size_t n, cudaStream_t stream) {
  if (n == 0) return MG_OK;
  int dev = 0, sms = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const size_t blocks = std::min<size_t>((n + 255) / 256, (size_t)sms * 8);
  sqrt_inplace_kernel<<<(unsigned)blocks, 256, 0, stream>>>(v, n);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

int launch_nearest(const float4* pal, int p, const float4* queries, int nq, int k, uint32_t* idx, float* dist,
                   uint32_t* err, cudaStream_t stream, int chunk, const LabIndex* index) {
  if (nq <= 0) return MG_OK;
  if (k <= 0 || k > 100) return fail(MG_ERR_ARG, "k must be in 1..100");
  const int keff = min(k, p);
  if (p <= 0) {
    MG_CUDA(cudaMemsetAsync(idx, 0xFF, sizeof(uint32_t) * (size_t)nq * k, stream));
    return MG_OK;
  }
  if (index && index->g > 0) return launch_nearest_grid(*index, queries, nq, keff, k, idx, dist, stream);
  if (chunk == 4096) return launch_nearest_t<4096>(pal, p, queries, nq, keff, k, idx, dist, err, stream);
  if (chunk == 1024) return launch_nearest_t<1024>(pal, p, queries, nq, keff, k, idx, dist, err, stream);
  return launch_nearest_t<2048>(pal, p, queries, nq, keff, k, idx, dist, err, stream);
}

}  // namespace mg
