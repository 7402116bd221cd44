// k_resize.cu -- Lanczos3 resize of the material images into thumbnails.
//
// Reference: main.rs:710-738 resize_image, fast_image_resize 5.1.4 with its
// default ResizeOptions (a Lanczos3 convolution, no cropping) on U8x3 images;
// the GUI asks for Lanczos3 explicitly (gui/app_full.rs:1894-1898).  That
// crate's convolution resampler follows the published one of Pillow
// (ImagingResample), which this restates:
//   * per output coordinate o of a dimension in -> out: scale = in / out,
//     filterscale = max(scale, 1), support = 3 * filterscale, centre =
//     (o + 0.5) * scale; taps i in [int(centre - support + 0.5),
//     int(centre + support + 0.5)) clipped to [0, in), weight
//     lanczos3((i - centre + 0.5) / filterscale), lanczos3(x) = sinc(x)
//     sinc(x / 3) on [-3, 3), the weights divided by their sum, then rounded
//     (half away from zero) to 22-bit fixed point;
//   * a horizontal pass into an 8-bit intermediate, then a vertical pass;
//     each output channel is clip8((2^21 + sum of weight * sample) >> 22); a
//     dimension that keeps its size is copied.
// The weights are computed once per distinct source size on the host in FP64
// and uploaded; the passes are integer arithmetic, so the result is exact and
// the CPU oracle computes the same bytes.  Parity with fast_image_resize's own
// fixed-point choices is not pinned (the crate is not here to run).
//
// Layout: a table for in -> out holds [out, kmax], then out (first tap, tap
// count) pairs, then out rows of kmax weights.  One CTA row of the grid per
// image; threads cover the image's output samples of the pass.
#include <cmath>
#include <map>
#include <vector>

#include "mg_internal.h"

namespace mg {

namespace {

constexpr int kResizeBits = 22;

double sinc(double x) {
  if (x == 0.0) return 1.0;
  x *= M_PI;
  return std::sin(x) / x;
}
double lanczos3(double x) { return (-3.0 <= x && x < 3.0) ? sinc(x) * sinc(x / 3.0) : 0.0; }

// The table of one dimension in -> out (out > 0, in > 0).
void build_table(int in, int out, std::vector<int32_t>& t) {
  const double scale = (double)in / (double)out;
  const double filterscale = scale < 1.0 ? 1.0 : scale;
  const double support = 3.0 * filterscale;
  const int kmax = (int)std::ceil(support) * 2 + 1;
  const size_t base = t.size();
  t.resize(base + 2 + 2 * (size_t)out + (size_t)out * kmax, 0);
  t[base] = out;
  t[base + 1] = kmax;
  std::vector<double> w(kmax);
  for (int o = 0; o < out; ++o) {
    const double centre = (o + 0.5) * scale;
    int lo = (int)(centre - support + 0.5);
    if (lo < 0) lo = 0;
    int hi = (int)(centre + support + 0.5);
    if (hi > in) hi = in;
    const int cnt = hi - lo;
    double sum = 0.0;
    for (int i = 0; i < cnt; ++i) {
      w[i] = lanczos3((i + lo - centre + 0.5) / filterscale);
      sum += w[i];
    }
    t[base + 2 + 2 * (size_t)o] = lo;
    t[base + 3 + 2 * (size_t)o] = cnt;
    int32_t* k = t.data() + base + 2 + 2 * (size_t)out + (size_t)o * kmax;
    for (int i = 0; i < cnt; ++i) {
      const double v = sum != 0.0 ? w[i] / sum : w[i];
      k[i] = (int32_t)(v < 0.0 ? -0.5 + v * (1 << kResizeBits) : 0.5 + v * (1 << kResizeBits));
    }
  }
}

__device__ __forceinline__ uint8_t clip8(int32_t v) {
  v >>= kResizeBits;
  return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v));
}

// Horizontal pass: image b's rows (sw wide) into its intermediate (tw wide),
// or a copy when the width is kept.
__global__ void __launch_bounds__(256) resize_h_kernel(const uint8_t* __restrict__ base, const ResizeImage* __restrict__ imgs,
                                                       const int32_t* __restrict__ tabs, int tw,
                                                       uint8_t* __restrict__ inter, int64_t inter_pitch) {
  const ResizeImage I = imgs[blockIdx.x];
  const uint8_t* src = base + I.offset;
  uint8_t* dst = inter + (int64_t)blockIdx.x * inter_pitch;
  const int total = I.h * tw;
  if (I.htab < 0) {  // same width
    for (int q = blockIdx.y * blockDim.x + threadIdx.x; q < total; q += gridDim.y * blockDim.x) {
      const int y = q / tw, x = q - y * tw;
      const uint8_t* s = src + (int64_t)y * I.stride + 3 * x;
      dst[3 * q] = s[0];
      dst[3 * q + 1] = s[1];
      dst[3 * q + 2] = s[2];
    }
    return;
  }
  const int32_t* T = tabs + I.htab;
  const int kmax = T[1];
  const int32_t* bounds = T + 2;
  const int32_t* coef = bounds + 2 * tw;
  for (int q = blockIdx.y * blockDim.x + threadIdx.x; q < total; q += gridDim.y * blockDim.x) {
    const int y = q / tw, x = q - y * tw;
    const int lo = bounds[2 * x], cnt = bounds[2 * x + 1];
    const uint8_t* s = src + (int64_t)y * I.stride + 3 * lo;
    const int32_t* k = coef + (int64_t)x * kmax;
    int32_t a0 = 1 << (kResizeBits - 1), a1 = a0, a2 = a0;
    for (int i = 0; i < cnt; ++i) {
      const int32_t w = __ldg(k + i);
      a0 += w * (int32_t)s[3 * i];
      a1 += w * (int32_t)s[3 * i + 1];
      a2 += w * (int32_t)s[3 * i + 2];
    }
    dst[3 * q] = clip8(a0);
    dst[3 * q + 1] = clip8(a1);
    dst[3 * q + 2] = clip8(a2);
  }
}

// Vertical pass: image b's intermediate (I.h rows of tw) into its thumbnail
// (th rows of tw), or a copy when the height is kept.
__global__ void __launch_bounds__(256) resize_v_kernel(const ResizeImage* __restrict__ imgs,
                                                       const int32_t* __restrict__ tabs, int tw, int th,
                                                       const uint8_t* __restrict__ inter, int64_t inter_pitch,
                                                       uint8_t* __restrict__ out) {
  const ResizeImage I = imgs[blockIdx.x];
  const uint8_t* src = inter + (int64_t)blockIdx.x * inter_pitch;
  uint8_t* dst = out + (int64_t)blockIdx.x * tw * th * 3;
  const int total = th * tw;
  const int pitch = 3 * tw;
  if (I.vtab < 0) {  // same height
    for (int q = blockIdx.y * blockDim.x + threadIdx.x; q < 3 * total; q += gridDim.y * blockDim.x) dst[q] = src[q];
    return;
  }
  const int32_t* T = tabs + I.vtab;
  const int kmax = T[1];
  const int32_t* bounds = T + 2;
  const int32_t* coef = bounds + 2 * th;
  for (int q = blockIdx.y * blockDim.x + threadIdx.x; q < total; q += gridDim.y * blockDim.x) {
    const int y = q / tw, x = q - y * tw;
    const int lo = bounds[2 * y], cnt = bounds[2 * y + 1];
    const uint8_t* s = src + (int64_t)lo * pitch + 3 * x;
    const int32_t* k = coef + (int64_t)y * kmax;
    int32_t a0 = 1 << (kResizeBits - 1), a1 = a0, a2 = a0;
    for (int i = 0; i < cnt; ++i) {
      const int32_t w = __ldg(k + i);
      const uint8_t* p = s + (int64_t)i * pitch;
      a0 += w * (int32_t)p[0];
      a1 += w * (int32_t)p[1];
      a2 += w * (int32_t)p[2];
    }
    dst[3 * q] = clip8(a0);
    dst[3 * q + 1] = clip8(a1);
    dst[3 * q + 2] = clip8(a2);
  }
}

}  // namespace

int ResizePlan::build(const Region* regions, int n_images, int tw_, int th_, cudaStream_t s) {
  if (n_images <= 0) {
    n = 0;
    return MG_OK;
  }
  if (tw_ <= 0 || th_ <= 0) return fail(MG_ERR_ARG, "thumbnail size must be positive");
  n = n_images;
  tw = tw_;
  th = th_;
  std::vector<int32_t> t;
  std::map<int, int> wtab, htab;  // source width / height -> table offset
  std::vector<ResizeImage> im((size_t)n);
  max_h = 1;
  for (int i = 0; i < n; ++i) {
    const Region& r = regions[i];
    if (r.w <= 0 || r.h <= 0) return fail(MG_ERR_ARG, "empty material image");
    int ho = -1, vo = -1;
    if (r.w != tw) {
      auto it = wtab.find(r.w);
      if (it == wtab.end()) {
        it = wtab.emplace(r.w, (int)t.size()).first;
        build_table(r.w, tw, t);
      }
      ho = it->second;
    }
    if (r.h != th) {
      auto it = htab.find(r.h);
      if (it == htab.end()) {
        it = htab.emplace(r.h, (int)t.size()).first;
        build_table(r.h, th, t);
      }
      vo = it->second;
    }
    im[i] = ResizeImage{r.offset, r.stride, r.w, r.h, ho, vo};
    max_h = std::max(max_h, r.h);
  }
  if (t.empty()) t.push_back(0);
  MG_CHECK(tabs.ensure(sizeof(int32_t) * t.size()));
  MG_CHECK(images.ensure(sizeof(ResizeImage) * im.size()));
  MG_CHECK(inter.ensure((size_t)n * max_h * tw * 3));
  MG_CUDA(cudaMemcpyAsync(tabs.p, t.data(), sizeof(int32_t) * t.size(), cudaMemcpyHostToDevice, s));
  // (from pageable memory: the sources are staged before the calls return)
  MG_CUDA(cudaMemcpyAsync(images.p, im.data(), sizeof(ResizeImage) * im.size(), cudaMemcpyHostToDevice, s));
  return MG_OK;
}

void ResizePlan::release() {
  tabs.release();
  images.release();
  inter.release();
  n = 0;
}

int launch_resize(const uint8_t* base, const ResizePlan& rp, uint8_t* out, cudaStream_t stream) {
  if (rp.n <= 0) return MG_OK;
  const int64_t pitch = (int64_t)rp.max_h * rp.tw * 3;
  const unsigned ys = (unsigned)std::min(16, std::max(1, (rp.max_h * rp.tw + 255) / 256));
  resize_h_kernel<<<dim3((unsigned)rp.n, ys), 256, 0, stream>>>(base, rp.images.as<ResizeImage>(), rp.tabs.as<int32_t>(),
                                                                 rp.tw, rp.inter.as<uint8_t>(), pitch);
  const unsigned yv = (unsigned)std::min(16, std::max(1, (rp.th * rp.tw + 255) / 256));
  resize_v_kernel<<<dim3((unsigned)rp.n, yv), 256, 0, stream>>>(rp.images.as<ResizeImage>(), rp.tabs.as<int32_t>(), rp.tw,
                                                                 rp.th, rp.inter.as<uint8_t>(), pitch, out);
  g_launches += 2;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
