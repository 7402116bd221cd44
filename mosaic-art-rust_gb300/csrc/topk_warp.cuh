// topk_warp.cuh -- one warp's sorted top-k list of 64-bit (distance bits,
// index) keys, shared by the k-nearest kernels (k_scan.cu, k_nearest_grid.cu).
// Keys below the current k-th best are appended to a buffer; a full buffer is
// bitonic-sorted and merged into the list by merge-path ranks.
#pragma once
#include <stdint.h>

namespace mg {
namespace {

constexpr int kListCap = 128;  // k <= 100
constexpr int kBufCap = 128;   // candidate buffer; merged when it could overflow
constexpr unsigned long long kMaxKey = ~0ull;

struct WarpLists {
  unsigned long long list[kListCap];
  unsigned long long tmp[kListCap];
  unsigned long long buf[kBufCap];
};

__device__ __forceinline__ int lower_bound_u64(const unsigned long long* a, int n, unsigned long long key) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Sort buf[0..m) ascending (m a power of two, <= kBufCap) with a bitonic network.
__device__ void warp_bitonic_sort(unsigned long long* buf, int m, int lane) {
  for (int size = 2; size <= m; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < (m >> 1); t += 32) {
        int i = 2 * t - (t & (stride - 1));
        int j = i + stride;
        bool asc = (i & size) == 0;
        unsigned long long a = buf[i], b = buf[j];
        if ((a > b) == asc) {
          buf[i] = b;
          buf[j] = a;
        }
      }
      __syncwarp();
    }
  }
}

// Merge the nbuf buffered keys into the sorted list (first k kept).
__device__ void warp_merge(WarpLists& W, int& len, int& nbuf, unsigned long long& thr, int k, int lane) {
  if (nbuf == 0) return;
  int m = 1;
  while (m < nbuf) m <<= 1;
  for (int i = nbuf + lane; i < m; i += 32) W.buf[i] = kMaxKey;
  __syncwarp();
  warp_bitonic_sort(W.buf, m, lane);
  for (int i = lane; i < len; i += 32) {
    unsigned long long key = W.list[i];
    int r = i + lower_bound_u64(W.buf, nbuf, key);
    if (r < k) W.tmp[r] = key;
  }
  for (int j = lane; j < nbuf; j += 32) {
    unsigned long long key = W.buf[j];
    int r = j + lower_bound_u64(W.list, len, key);
    if (r < k) W.tmp[r] = key;
  }
  __syncwarp();
  len = min(k, len + nbuf);
  for (int i = lane; i < len; i += 32) W.list[i] = W.tmp[i];
  __syncwarp();
  nbuf = 0;
  thr = (len == k) ? W.list[k - 1] : kMaxKey;
}

}  // namespace
}  // namespace mg
