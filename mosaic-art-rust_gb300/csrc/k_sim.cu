// k_sim.cu -- (c) the material x material similarity matrix on the device.
//
// Reference: similarity.rs:69-82 build_similarities (Euclidean Lab distance of
// every pair i < j, stored as the strict upper triangle in row order, position
// i*n - i*(i+1)/2 + j - i - 1) and similarity.rs:85-103 get_similarity
// (symmetric, 0 for the same tile).  The full layout stores the same values as
// a P x P symmetric matrix with a zero diagonal; the triangular layout is the
// reference's own.  The distance (a-b)^2 is exactly symmetric in IEEE
// arithmetic, so row i of the full matrix is computed directly from pal[i].
//
// Bound: HBM writes (4 bytes per stored value).  Full layout: 8 rows x 1024
// columns per CTA, four consecutive floats per thread and row (streaming
// 16-byte stores when P % 4 == 0: the matrix is read much later, by other
// kernels, so it need not stay in L1).
#include "mg_internal.h"

namespace mg {
namespace {

constexpr int kSimRows = 8;  // rows of the full matrix per CTA

// A CTA covers kSimRows rows x 1024 columns: each thread holds the Lab of its
// four columns in registers and writes four consecutive floats of each row
// (one 16-byte store when P % 4 == 0), so a warp writes 512 contiguous bytes
// per row and the column colours are loaded once per kSimRows rows.
template <bool kVec4>
__global__ void __launch_bounds__(256) similarity_full_kernel(const float4* __restrict__ pal, int p,
                                                              float* __restrict__ out) {
  const int i0 = blockIdx.y * kSimRows;
  const int j0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (j0 >= p) return;
  float4 b[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) b[u] = j0 + u < p ? pal[j0 + u] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 2
  for (int r = 0; r < kSimRows; ++r) {
    const int i = i0 + r;
    if (i >= p) break;
    const float4 a = pal[i];
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = lab_distance(a.x, a.y, a.z, b[u].x, b[u].y, b[u].z);
    float* row = out + (size_t)i * p;
    if (kVec4) {
      __stcs(reinterpret_cast<float4*>(row + j0), make_float4(v[0], v[1], v[2], v[3]));
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (j0 + u < p) row[j0 + u] = v[u];
    }
  }
}

__global__ void __launch_bounds__(256) similarity_tri_kernel(const float4* __restrict__ pal, int p,
                                                             float* __restrict__ out) {
  const int i = blockIdx.y;
  const int j = i + 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p) return;
  const float4 a = pal[i], b = pal[j];
  const int64_t pos = (int64_t)i * p - (int64_t)i * (i + 1) / 2 + (j - i - 1);
  out[pos] = lab_distance(a.x, a.y, a.z, b.x, b.y, b.z);
}

}  // namespace

int launch_similarity(const float4* pal, int p, int triangular, float* out, cudaStream_t stream) {
  if (p <= 0) return MG_OK;
  if (p > 65535 * 1) {
    // gridDim.y limit
    return fail(MG_ERR_ARG, "palette too large for the similarity matrix (max 65535)");
  }
  if (triangular) {
    if (p < 2) return MG_OK;
    dim3 grid((unsigned)((p - 1 + 255) / 256), (unsigned)p);
    similarity_tri_kernel<<<grid, 256, 0, stream>>>(pal, p, out);
  } else {
    dim3 grid((unsigned)((p + 1023) / 1024), (unsigned)((p + kSimRows - 1) / kSimRows));
    if (p % 4 == 0) similarity_full_kernel<true><<<grid, 256, 0, stream>>>(pal, p, out);
    else similarity_full_kernel<false><<<grid, 256, 0, stream>>>(pal, p, out);
  }
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
