// k_lab.cu -- (a) per-region mean Lab and mean RGB (target cells, materials,
// thumbnails), and the area-average thumbnail resize.
//
// Reference: lib.rs:94-119 calculate_average_lab (per-pixel sRGB8 -> Lab, then
// the mean of Lab), main.rs:687-708 calculate_average_rgb (u64 sums,
// truncating division), main.rs:495-496 / 537-541 (cells of w/gw x h/gh at
// (x*cw, y*ch), remainder ignored).
//
// Design: one CTA per (region, row chunk).  Each thread converts pixels to Lab
// with the table-driven FP32 arithmetic of mg_math.h and accumulates the
// fixed-point Lab (int64) and RGB (u32) in registers; warp shuffles and one
// shared-memory pass reduce the CTA, and six 64-bit atomics add it to the
// region's sums.  Integer sums are exact, so the result does not depend on the
// CTA count or order.  A second tiny kernel divides.
#include <cmath>
#include <mutex>

#include <algorithm>

#include "mg_internal.h"

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

template <bool kCells, bool kLab>
__global__ void __launch_bounds__(kStatThreads) region_stats_kernel(const uint8_t* __restrict__ base, CellGeom geom,
                                                                    const Region* __restrict__ regions, int chunks,
                                                                    RegionSums* __restrict__ sums) {
  __shared__ float s_lut[256];
  __shared__ float s_ms[9];
  __shared__ long long s_lab[kStatThreads / 32][3];
  __shared__ unsigned long long s_rgb[kStatThreads / 32][3];

  const int r = blockIdx.x / chunks;
  const int chunk = blockIdx.x - r * chunks;
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
  if (kLab) {
    for (int i = threadIdx.x; i < 256; i += blockDim.x) s_lut[i] = c_lab.lut[i];
    if (threadIdx.x < 9) s_ms[threadIdx.x] = c_lab.ms[threadIdx.x];
    __syncthreads();
  }
  const float eps = c_lab.eps, k1 = c_lab.k1, k2 = c_lab.k2;

  const int y0 = (int)((int64_t)chunk * h / chunks), y1 = (int)((int64_t)(chunk + 1) * h / chunks);
  long long aL = 0, aA = 0, aB = 0;
  unsigned int sr = 0, sg = 0, sb = 0;
  auto pixel = [&](uint32_t r8, uint32_t g8, uint32_t b8) {
    sr += r8;
    sg += g8;
    sb += b8;
    if (kLab) {
      float L, A, B;
      lab_pixel(s_lut, s_ms, eps, k1, k2, r8, g8, b8, L, A, B);
      aL += lab_quant(L);
      aA += lab_quant(A);
      aB += lab_quant(B);
    }
  };
  const uint8_t* img = base + off;
  if ((w & 3) == 0 && (stride & 3) == 0 && ((uintptr_t)img & 3) == 0) {
    // Four pixels of a row as three 32-bit words (fewer, wider loads: the
    // regions may sit in pinned host memory read over the CPU-GPU link).  The
    // sums are exact integers, so the order of the pixels does not matter.
    const int gpr = w >> 2;
    const int64_t ng = (int64_t)(y1 - y0) * gpr;
    int gx = threadIdx.x % gpr, y = y0 + threadIdx.x / gpr;
    const int dgx = kStatThreads % gpr, dgy = kStatThreads / gpr;
    for (int64_t q = threadIdx.x; q < ng; q += kStatThreads) {
      const uint32_t* p = reinterpret_cast<const uint32_t*>(img + (int64_t)y * stride + 12 * gx);
      const uint32_t w0 = p[0], w1 = p[1], w2 = p[2];
      pixel(w0 & 0xFFu, (w0 >> 8) & 0xFFu, (w0 >> 16) & 0xFFu);
      pixel(w0 >> 24, w1 & 0xFFu, (w1 >> 8) & 0xFFu);
      pixel((w1 >> 16) & 0xFFu, w1 >> 24, w2 & 0xFFu);
      pixel((w2 >> 8) & 0xFFu, (w2 >> 16) & 0xFFu, w2 >> 24);
      gx += dgx;
      y += dgy;
      if (gx >= gpr) {
        gx -= gpr;
        ++y;
      }
    }
  } else {
    // Walk pixels i = tid, tid + T, ... of the chunk with incremental (x, y).
    const int64_t npx = (int64_t)(y1 - y0) * w;
    int x = threadIdx.x % w, y = y0 + threadIdx.x / w;
    const int dx = kStatThreads % w, dy = kStatThreads / w;
    for (int64_t i = threadIdx.x; i < npx; i += kStatThreads) {
      const uint8_t* p = img + (int64_t)y * stride + 3 * x;
      pixel(p[0], p[1], p[2]);
      x += dx;
      y += dy;
      if (x >= w) {
        x -= w;
        ++y;
      }
    }
  }
  unsigned long long ur = sr, ug = sg, ub = sb;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    if (kLab) {
      aL += __shfl_xor_sync(0xffffffffu, aL, o);
      aA += __shfl_xor_sync(0xffffffffu, aA, o);
      aB += __shfl_xor_sync(0xffffffffu, aB, o);
    }
    ur += __shfl_xor_sync(0xffffffffu, ur, o);
    ug += __shfl_xor_sync(0xffffffffu, ug, o);
    ub += __shfl_xor_sync(0xffffffffu, ub, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_lab[warp][0] = aL; s_lab[warp][1] = aA; s_lab[warp][2] = aB;
    s_rgb[warp][0] = ur; s_rgb[warp][1] = ug; s_rgb[warp][2] = ub;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int c = threadIdx.x % 3;
    if (threadIdx.x < 3) {
      long long t = 0;
      for (int i = 0; i < kStatThreads / 32; ++i) t += s_lab[i][c];
      if (kLab) atomicAdd(reinterpret_cast<unsigned long long*>(&sums[r].lab[c]), (unsigned long long)t);
    } else {
      unsigned long long t = 0;
      for (int i = 0; i < kStatThreads / 32; ++i) t += s_rgb[i][c];
      atomicAdd(&sums[r].rgb[c], t);
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
  MG_CUDA(cudaMemsetAsync(scratch, 0, sizeof(RegionSums) * (size_t)n_regions, stream));
  // Split large regions over several CTAs so that small palettes still fill the GPU.
  int chunks = (int)std::min<int64_t>(64, std::max<int64_t>(1, max_region_px / 8192));
  if ((int64_t)n_regions * chunks > (1ll << 30)) return fail(MG_ERR_ARG, "too many regions");
  const unsigned grid = (unsigned)(n_regions * chunks);
  CellGeom g{};
  if (geom) g = *geom;
  if (geom) {
    if (want_lab) region_stats_kernel<true, true><<<grid, kStatThreads, 0, stream>>>(base, g, nullptr, chunks, scratch);
    else region_stats_kernel<true, false><<<grid, kStatThreads, 0, stream>>>(base, g, nullptr, chunks, scratch);
    region_finalize_kernel<true><<<(n_regions + 255) / 256, 256, 0, stream>>>(g, nullptr, n_regions, scratch,
                                                                             want_lab ? out_lab : nullptr, out_rgb);
  } else {
    if (want_lab) region_stats_kernel<false, true><<<grid, kStatThreads, 0, stream>>>(base, g, regions, chunks, scratch);
    else region_stats_kernel<false, false><<<grid, kStatThreads, 0, stream>>>(base, g, regions, chunks, scratch);
    region_finalize_kernel<false><<<(n_regions + 255) / 256, 256, 0, stream>>>(g, regions, n_regions, scratch,
                                                                              want_lab ? out_lab : nullptr, out_rgb);
  }
  g_launches += 2;
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
