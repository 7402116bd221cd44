// k_lab.cu -- (a) per-region mean Lab and mean RGB (target cells, materials,
// thumbnails), and the area-average thumbnail resize.
//
// Reference: lib.rs:94-119 calculate_average_lab (per-pixel sRGB8 -> Lab, then
// the mean of Lab), main.rs:687-708 calculate_average_rgb (u64 sums,
// truncating division), main.rs:495-496 / 537-541 (cells of w/gw x h/gh at
// (x*cw, y*ch), remainder ignored).
//
// Design: one warp per (region, chunk of rows); the per-pixel work is
// lab_reduce.cuh (packed FP32x2 Lab of pixel pairs from 48-byte loads,
// fixed-point sums).  A region that fits one unit (a target cell) is reduced
// and divided by its warp; larger ones (materials) add each chunk's sums to
// the region's with 64-bit atomics and a second tiny kernel divides.  Integer
// sums are exact, so the result does not depend on the split.
#include <cmath>
#include <mutex>

#include <algorithm>

#include "lab_reduce.cuh"

namespace mg {

__constant__ LabConsts c_lab;

namespace {

struct HostLabConsts {
  LabConsts c;
  HostLabConsts() {
    const double white[3] = {0.95047, 1.0, 1.08883};
    const double xy[3][2] = {{0.64, 0.33}, {0.30, 0.60}, {0.15, 0.06}};
    double P[3][3];
    for (int k = 0; k < 3; ++k) {
      P[0][k] = xy[k][0] / xy[k][1];
      P[1][k] = 1.0;
      P[2][k] = (1.0 - xy[k][0] - xy[k][1]) / xy[k][1];
    }
    // Solve P * S = white by Cramer's rule.
    auto det3 = [](double a[3][3]) {
      return a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) - a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
             a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    };
    double d = det3(P);
    double S[3];
    for (int k = 0; k < 3; ++k) {
      double A[3][3];
      for (int r = 0; r < 3; ++r)
        for (int cc = 0; cc < 3; ++cc) A[r][cc] = (cc == k) ? white[r] : P[r][cc];
      S[k] = det3(A) / d;
    }
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) c.ms[3 * r + k] = (float)(P[r][k] * S[k] / white[r]);
    for (int v = 0; v < 256; ++v) {
      double x = v / 255.0;
      c.lut[v] = (float)(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4));
    }
    const double eps = 216.0 / 24389.0, kappa = 24389.0 / 27.0;
    c.eps = (float)eps;
    c.k1 = (float)(kappa / 116.0);
    c.k2 = (float)(16.0 / 116.0);
  }
};

constexpr int kStatThreads = 256;
constexpr int kStatWarps = kStatThreads / 32;
constexpr int64_t kUnitPx = 4096;  // pixels per warp unit when a region is split into row chunks

// One warp per unit = (region, chunk of its rows).  With one chunk per region
// the unit's warp writes the region's means itself; with several, it adds its
// sums to the region's (zeroed) RegionSums with six 64-bit atomics and
// region_finalize_kernel divides.  The CTA loads the transfer table once and
// its warps take units round robin.
template <bool kCells, bool kLab>
__global__ void __launch_bounds__(kStatThreads) region_stats_kernel(const uint8_t* __restrict__ base, CellGeom geom,
                                                                    const Region* __restrict__ regions, int n_regions,
                                                                    int chunks, RegionSums* __restrict__ sums,
                                                                    float4* __restrict__ out_lab,
                                                                    uchar4* __restrict__ out_rgb) {
  __shared__ float s_lut[256];
  if (kLab) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_lut[i] = c_lab.lut[i];
    __syncthreads();
  }
  const LabK K = make_lab_k(c_lab.ms, c_lab.eps, c_lab.k1, c_lab.k2);
  const int lane = threadIdx.x & 31;
  const int64_t units = (int64_t)n_regions * chunks;
  for (int64_t u = (int64_t)blockIdx.x * kStatWarps + (threadIdx.x >> 5); u < units;
       u += (int64_t)gridDim.x * kStatWarps) {
    const int r = (int)(u / chunks);
    const int chunk = (int)(u - (int64_t)r * chunks);
    int64_t off, stride;
    int w, h;
    if (kCells) {
      const int cx = r % geom.gw, cy = r / geom.gw;
      w = geom.cw;
      h = geom.ch;
      stride = geom.stride;
      off = (int64_t)cy * geom.ch * stride + 3ll * cx * geom.cw;
    } else {
      const Region reg = regions[r];
      off = reg.offset;
      w = reg.w;
      h = reg.h;
      stride = reg.stride;
    }
    const int y0 = (int)((int64_t)chunk * h / chunks), y1 = (int)((int64_t)(chunk + 1) * h / chunks);
    LabAcc acc;
    reduce_rows<kLab>(base + off, w, stride, y0, y1, lane, s_lut, K, acc);
    const LabSums t = warp_sums<kLab>(acc);
    if (lane == 0) {
      if (chunks == 1) {
        const long long npx = (long long)w * h;
        if (kLab && out_lab)
          out_lab[r] = make_float4(lab_mean(t.L, npx), lab_mean(t.A, npx), lab_mean(t.B, npx), 0.0f);
        if (out_rgb) {
          const unsigned long long n = (unsigned long long)npx;
          out_rgb[r] = make_uchar4((unsigned char)(t.R / n), (unsigned char)(t.G / n), (unsigned char)(t.Bc / n), 0);
        }
      } else {
        if (kLab) {
          atomicAdd(reinterpret_cast<unsigned long long*>(&sums[r].lab[0]), (unsigned long long)t.L);
          atomicAdd(reinterpret_cast<unsigned long long*>(&sums[r].lab[1]), (unsigned long long)t.A);
          atomicAdd(reinterpret_cast<unsigned long long*>(&sums[r].lab[2]), (unsigned long long)t.B);
        }
        atomicAdd(&sums[r].rgb[0], t.R);
        atomicAdd(&sums[r].rgb[1], t.G);
        atomicAdd(&sums[r].rgb[2], t.Bc);
      }
    }
  }
}

template <bool kCells>
__global__ void region_finalize_kernel(CellGeom geom, const Region* __restrict__ regions, int n,
                                       const RegionSums* __restrict__ sums, float4* __restrict__ out_lab,
                                       uchar4* __restrict__ out_rgb) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  long long npx;
  if (kCells) npx = (long long)geom.cw * geom.ch;
  else npx = (long long)regions[r].w * regions[r].h;
  const RegionSums s = sums[r];
  if (out_lab) out_lab[r] = make_float4(lab_mean(s.lab[0], npx), lab_mean(s.lab[1], npx), lab_mean(s.lab[2], npx), 0.0f);
  if (out_rgb) {
    const unsigned long long n = (unsigned long long)npx;
    out_rgb[r] = make_uchar4((unsigned char)(s.rgb[0] / n), (unsigned char)(s.rgb[1] / n), (unsigned char)(s.rgb[2] / n), 0);
  }
}

// Area-average resize (integer box sums, rounded half up); one thread per
// output pixel.  Same rule as the host synthetic-input generator.
__global__ void thumbnail_kernel(const uint8_t* __restrict__ base, const Region* __restrict__ regions, int n, int tw,
                                 int th, uint8_t* __restrict__ out) {
  const int64_t total = (int64_t)n * tw * th;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(t / ((int64_t)tw * th));
    const int rem = (int)(t - (int64_t)m * tw * th);
    const int oy = rem / tw, ox = rem - oy * tw;
    const Region reg = regions[m];
    int y0 = (int)((int64_t)oy * reg.h / th), y1 = (int)((int64_t)(oy + 1) * reg.h / th);
    if (y1 <= y0) y1 = y0 + 1;
    int x0 = (int)((int64_t)ox * reg.w / tw), x1 = (int)((int64_t)(ox + 1) * reg.w / tw);
    if (x1 <= x0) x1 = x0 + 1;
    uint32_t s0 = 0, s1 = 0, s2 = 0;
    for (int y = y0; y < y1; ++y) {
      const uint8_t* row = base + reg.offset + (int64_t)y * reg.stride;
      for (int x = x0; x < x1; ++x) {
        s0 += row[3 * x];
        s1 += row[3 * x + 1];
        s2 += row[3 * x + 2];
      }
    }
    const uint32_t cnt = (uint32_t)((y1 - y0) * (x1 - x0));
    uint8_t* d = out + 3 * t;
    d[0] = (uint8_t)((s0 + cnt / 2) / cnt);
    d[1] = (uint8_t)((s1 + cnt / 2) / cnt);
    d[2] = (uint8_t)((s2 + cnt / 2) / cnt);
  }
}

}  // namespace

const LabConsts& host_lab_consts() {
  static HostLabConsts h;
  return h.c;
}

cudaError_t upload_lab_consts(cudaStream_t stream) {
  static HostLabConsts h;
  return cudaMemcpyToSymbolAsync(c_lab, &h.c, sizeof(LabConsts), 0, cudaMemcpyHostToDevice, stream);
}

int launch_region_stats(const uint8_t* base, const CellGeom* geom, const Region* regions, int n_regions,
                        int64_t max_region_px, float4* out_lab, uchar4* out_rgb, RegionSums* scratch, int want_lab,
                        cudaStream_t stream) {
  if (n_regions <= 0) return MG_OK;
  // Regions above 2 units split into row chunks of about kUnitPx pixels, so
  // that a few large materials still spread over the GPU; smaller ones (target
  // cells) are one warp each and need no scratch.
  const int chunks = (int)std::min<int64_t>(64, std::max<int64_t>(1, max_region_px / kUnitPx));
  const int64_t units = (int64_t)n_regions * chunks;
  if (units > (1ll << 40)) return fail(MG_ERR_ARG, "too many regions");
  if (chunks > 1) MG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(RegionSums) * (size_t)n_regions, stream));
  int dev = 0, sms = 0;
  MG_CUDA(cudaGetDevice(&dev));
  MG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((units + kStatWarps - 1) / kStatWarps,
                                                                         (int64_t)sms * 16));
  CellGeom g{};
  if (geom) g = *geom;
  float4* lab = want_lab ? out_lab : nullptr;
  if (geom) {
    if (want_lab) region_stats_kernel<true, true><<<grid, kStatThreads, 0, stream>>>(base, g, nullptr, n_regions, chunks, scratch, lab, out_rgb);
    else region_stats_kernel<true, false><<<grid, kStatThreads, 0, stream>>>(base, g, nullptr, n_regions, chunks, scratch, lab, out_rgb);
    if (chunks > 1)
      region_finalize_kernel<true><<<(n_regions + 255) / 256, 256, 0, stream>>>(g, nullptr, n_regions, scratch, lab,
                                                                               out_rgb);
  } else {
    if (want_lab) region_stats_kernel<false, true><<<grid, kStatThreads, 0, stream>>>(base, g, regions, n_regions, chunks, scratch, lab, out_rgb);
    else region_stats_kernel<false, false><<<grid, kStatThreads, 0, stream>>>(base, g, regions, n_regions, chunks, scratch, lab, out_rgb);
    if (chunks > 1)
      region_finalize_kernel<false><<<(n_regions + 255) / 256, 256, 0, stream>>>(g, regions, n_regions, scratch, lab,
                                                                                out_rgb);
  }
  g_launches += chunks > 1 ? 2 : 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

// ---- allocation-free cell statistics ------------------------------------------------------
// Some callers of the cell reduction cannot allocate device memory at the
// point where they call it: a serving process whose device memory is owned by
// its own pool allocator under a fixed budget (an extra cudaMalloc there either
// fails or breaks the budget), or code that must not pay cudaMalloc/cudaFree's
// implicit device synchronisation in the middle of a stream of work.  For them
// mg_cells_lab_noalloc takes device pointers and keeps its per-cell sums in the
// file-scope array below, which the library reserves on every GPU that loads it
// (kNoAllocMaxCells * 48 bytes = 1.5 MB) until the process exits.
namespace {
constexpr int kNoAllocMaxCells = 32768;
static __device__ __align__(256) RegionSums g_noalloc_sums[kNoAllocMaxCells];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
RegionSums* g_noalloc_ptr[kMaxDevices] = {};
}  // namespace

}  // namespace mg

extern "C" int mg_cells_lab_noalloc(const uint8_t* d_img, int w, int h, int64_t stride, int gw, int gh,
                                    float* d_lab4, uint8_t* d_rgb4, void* stream) {
  using namespace mg;
  if (!d_img || !d_lab4 || w <= 0 || h <= 0 || stride < 3ll * w) return fail(MG_ERR_ARG, "invalid image");
  if (gw <= 0 || gh <= 0 || w / gw <= 0 || h / gh <= 0) return fail(MG_ERR_ARG, "grid larger than the image");
  if ((int64_t)gw * gh > kNoAllocMaxCells)
    return fail(MG_ERR_ARG, "mg_cells_lab_noalloc handles at most " + std::to_string(kNoAllocMaxCells) +
                                " cells; use mg_cells_lab for larger grids");
  if ((reinterpret_cast<uintptr_t>(d_lab4) & 15) || (reinterpret_cast<uintptr_t>(d_rgb4) & 3))
    return fail(MG_ERR_ARG, "lab output must be 16-byte aligned and rgb output 4-byte aligned");
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(MG_ERR_ARG, "device ordinal out of range");
  RegionSums* sums = nullptr;
  {
    // First call on a device: resolve the array's device address (the host-side
    // symbol is only a stand-in) and upload the Lab constants to that device.
    // The address is kept only once both have succeeded, so a failed first
    // call is retried in full by the next one.
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      MG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_sums));
      MG_CUDA(upload_lab_consts(0));
      MG_CUDA(cudaDeviceSynchronize());
      g_noalloc_ptr[dev] = static_cast<RegionSums*>(p);
    }
    sums = g_noalloc_ptr[dev];
  }
  const int n = gw * gh;
  CellGeom g{gw, gh, w / gw, h / gh, stride};
  return launch_region_stats(d_img, &g, nullptr, n, (int64_t)g.cw * g.ch, reinterpret_cast<float4*>(d_lab4),
                             reinterpret_cast<uchar4*>(d_rgb4), sums, 1, static_cast<cudaStream_t>(stream));
}

namespace mg {

int launch_thumbnails(const uint8_t* base, const Region* regions, int n, int tw, int th, uint8_t* out,
                      cudaStream_t stream) {
  if (n <= 0) return MG_OK;
  const int64_t total = (int64_t)n * tw * th;
  const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16);
  thumbnail_kernel<<<grid, 256, 0, stream>>>(base, regions, n, tw, th, out);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

namespace {
// One CTA per item; 16-byte vector copies when source, destination and size allow.
__global__ void __launch_bounds__(256) gather_kernel(const int64_t* __restrict__ src, size_t bytes,
                                                     uint8_t* __restrict__ dst) {
  const uint8_t* s = reinterpret_cast<const uint8_t*>((uintptr_t)src[blockIdx.x]);
  uint8_t* d = dst + (size_t)blockIdx.x * bytes;
  if ((((uintptr_t)s | (uintptr_t)d | bytes) & 15) == 0) {
    const uint4* s4 = reinterpret_cast<const uint4*>(s);
    uint4* d4 = reinterpret_cast<uint4*>(d);
    for (size_t i = threadIdx.x; i < bytes / 16; i += blockDim.x) d4[i] = s4[i];
  } else {
    for (size_t i = threadIdx.x; i < bytes; i += blockDim.x) d[i] = s[i];
  }
}
}  // namespace

int launch_gather(const int64_t* src, int n, size_t bytes, uint8_t* dst, cudaStream_t stream) {
  if (n <= 0 || bytes == 0) return MG_OK;
  gather_kernel<<<n, 256, 0, stream>>>(src, bytes, dst);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
