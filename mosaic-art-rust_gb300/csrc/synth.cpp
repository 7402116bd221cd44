// synth.cpp -- seeded synthetic inputs for the mosaic workloads (targets,
// materials, thumbnails).  Host C++; every random draw is Philox4x32-10 keyed
// by (seed lo, seed hi) with counter (a, b, stream, purpose), and every float
// step is explicit (mg_math.h, built with -ffp-contract=off), so x86 and Arm
// hosts produce the same bytes.
//
// Targets: a uniform background colour, then B isotropic Gaussian blobs (centre
// uniform in the image, sigma uniform in 40..200 px, colour uniform in the sRGB
// cube) alpha-blended in order with weight exp(-d^2 / (2 sigma^2)), then
// per-pixel uniform integer noise in [-8, 8], clamped.
// Materials: a base colour uniform in the cube plus a linear gradient (random
// direction, amplitude uniform in 0..32 over half the long side) plus
// per-pixel uniform integer noise in [-16, 16], clamped.
// Thumbnails: area-average (box) resize of each material to the output tile.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "mg_math.h"

using mg::philox;
using mg::u32x4;

namespace {

enum : uint32_t {
  kTgtBg = 0x10, kTgtBlob = 0x11, kTgtNoise = 0x12,
  kMatDims = 0x20, kMatBase = 0x21, kMatDir = 0x22, kMatNoise = 0x23,
};

inline float unit(uint32_t r) { return mg::unit_f32(r); }

template <class F>
void parallel_rows(int n, int threads, F fn) {
  if (threads <= 1 || n <= 1) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  threads = std::min(threads, n);
  auto rows = [=, &fn](int t) {
    for (int i = t; i < n; i += threads) fn(i);
  };
  // A thread that cannot be created (a thread or process limit) leaves its
  // rows, and those of the threads after it, to the calling thread.
  std::vector<std::thread> pool;
  int t = 0;
  for (; t < threads; ++t) {
    try {
      pool.emplace_back(rows, t);
    } catch (const std::exception&) {
      break;
    }
  }
  for (; t < threads; ++t) rows(t);
  for (auto& th : pool) th.join();
}

inline uint8_t clamp_u8(int v) { return (uint8_t)(v < 0 ? 0 : (v > 255 ? 255 : v)); }

struct Blob { float cx, cy, s2x2, cut2; float col[3]; };

}  // namespace

extern "C" {

// Target image, w x h x 3, row stride 3w.
void ms_target(uint8_t* out, int w, int h, int n_blobs, uint64_t seed, uint32_t stream, int threads) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  u32x4 bg = philox(0, 0, stream, kTgtBg, k0, k1);
  const float bgc[3] = {(float)(bg.x >> 24), (float)(bg.y >> 24), (float)(bg.z >> 24)};
  std::vector<Blob> blobs(n_blobs);
  for (int i = 0; i < n_blobs; ++i) {
    u32x4 a = philox((uint32_t)i, 0, stream, kTgtBlob, k0, k1);
    u32x4 c = philox((uint32_t)i, 1, stream, kTgtBlob, k0, k1);
    Blob& b = blobs[i];
    b.cx = unit(a.x) * (float)w;
    b.cy = unit(a.y) * (float)h;
    float sigma = 40.0f + 160.0f * unit(a.z);
    float s2 = sigma * sigma;
    b.s2x2 = 2.0f * s2;
    b.cut2 = 36.0f * s2;  // beyond 6 sigma the weight is below 1.6e-8: skipped
    b.col[0] = (float)(c.x >> 24); b.col[1] = (float)(c.y >> 24); b.col[2] = (float)(c.z >> 24);
  }
  parallel_rows(h, threads, [&](int y) {
    uint8_t* row = out + (size_t)y * w * 3;
    const float fy = (float)y + 0.5f;
    for (int x = 0; x < w; ++x) {
      float c[3] = {bgc[0], bgc[1], bgc[2]};
      const float fx = (float)x + 0.5f;
      for (int i = 0; i < n_blobs; ++i) {
        const Blob& b = blobs[i];
        float dx = fx - b.cx, dy = fy - b.cy;
        float d2 = dx * dx + dy * dy;
        if (!(d2 < b.cut2)) continue;
        float a = mg::exp_spec(-(d2 / b.s2x2));
        for (int k = 0; k < 3; ++k) c[k] = c[k] + a * (b.col[k] - c[k]);
      }
      u32x4 n = philox((uint32_t)x, (uint32_t)y, stream, kTgtNoise, k0, k1);
      const uint32_t nr[3] = {n.x, n.y, n.z};
      for (int k = 0; k < 3; ++k) row[3 * x + k] = clamp_u8((int)std::rintf(c[k]) + (int)(nr[k] % 17u) - 8);
    }
  });
}

// Material sizes.  mode 0: every material side x side.  mode 1: aspect drawn
// uniformly from {1:1, 4:3, 3:4} with long side `side`.
void ms_material_dims(int n, int side, int mode, uint64_t seed, uint32_t stream, int* w, int* h) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int m = 0; m < n; ++m) {
    int ww = side, hh = side;
    if (mode == 1) {
      u32x4 r = philox((uint32_t)m, 0, stream, kMatDims, k0, k1);
      int sel = (int)(r.x % 3u);
      if (sel == 1) hh = side * 3 / 4;
      if (sel == 2) ww = side * 3 / 4;
    }
    w[m] = ww;
    h[m] = hh;
  }
}

// Material pixels into a packed buffer; material m starts at off[m], rows of 3*w[m] bytes.
void ms_materials(uint8_t* out, const int64_t* off, const int* w, const int* h, int n, uint64_t seed,
                  uint32_t stream, int threads) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  parallel_rows(n, threads, [&](int m) {
    u32x4 b = philox((uint32_t)m, 1, stream, kMatBase, k0, k1);
    const float base[3] = {(float)(b.x >> 24), (float)(b.y >> 24), (float)(b.z >> 24)};
    const float amp = 32.0f * unit(b.w);
    float dx = 1.0f, dy = 0.0f;
    for (uint32_t t = 0; t < 64; ++t) {
      u32x4 d = philox((uint32_t)m, 2 + t, stream, kMatDir, k0, k1);
      float ux = unit(d.x) * 2.0f - 1.0f, uy = unit(d.y) * 2.0f - 1.0f;
      float n2 = ux * ux + uy * uy;
      if (n2 > 1e-4f && n2 <= 1.0f) {
        float inv = std::sqrt(n2);
        dx = ux / inv;
        dy = uy / inv;
        break;
      }
    }
    const int W = w[m], H = h[m];
    const float half = (float)std::max(W, H) * 0.5f;
    const float cx = (float)W * 0.5f, cy = (float)H * 0.5f;
    uint8_t* img = out + off[m];
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        float proj = ((float)x + 0.5f - cx) * dx + ((float)y + 0.5f - cy) * dy;
        float g = amp * (proj / half);
        u32x4 nz = philox((uint32_t)(y * W + x), (uint32_t)m, stream, kMatNoise, k0, k1);
        const uint32_t nr[3] = {nz.x, nz.y, nz.z};
        for (int k = 0; k < 3; ++k)
          img[3 * ((size_t)y * W + x) + k] = clamp_u8((int)std::rintf(base[k] + g) + (int)(nr[k] % 33u) - 16);
      }
  });
}

// Area-average resize of every material to tw x th (integer box sums,
// rounded half up).  out: n x th x tw x 3.
void ms_thumbnails(const uint8_t* mats, const int64_t* off, const int* w, const int* h, int n, int tw,
                   int th, uint8_t* out, int threads) {
  parallel_rows(n, threads, [&](int m) {
    const int W = w[m], H = h[m];
    const uint8_t* src = mats + off[m];
    uint8_t* dst = out + (size_t)m * tw * th * 3;
    for (int oy = 0; oy < th; ++oy) {
      int y0 = (int)((int64_t)oy * H / th), y1 = (int)((int64_t)(oy + 1) * H / th);
      if (y1 <= y0) y1 = y0 + 1;
      for (int ox = 0; ox < tw; ++ox) {
        int x0 = (int)((int64_t)ox * W / tw), x1 = (int)((int64_t)(ox + 1) * W / tw);
        if (x1 <= x0) x1 = x0 + 1;
        uint32_t s[3] = {0, 0, 0};
        for (int y = y0; y < y1; ++y)
          for (int x = x0; x < x1; ++x)
            for (int k = 0; k < 3; ++k) s[k] += src[3 * ((size_t)y * W + x) + k];
        uint32_t cnt = (uint32_t)((y1 - y0) * (x1 - x0));
        for (int k = 0; k < 3; ++k) dst[3 * ((size_t)oy * tw + ox) + k] = (uint8_t)((s[k] + cnt / 2) / cnt);
      }
    }
  });
}

}  // extern "C"
