// capi.cu -- the C ABI of mosaic_gpu.h: contexts, host<->device staging, the
// per-stage entry points and the whole-job plan.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda.h>  // driver types only: the entry point is fetched through the runtime

#include "capi_internal.h"

namespace mg {

std::atomic<unsigned long long> g_launches{0};

namespace {
thread_local std::string g_error;
}

void set_error(const std::string& msg) { g_error = msg; }
int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? MG_ERR_OOM : MG_ERR_CUDA;
}

int DevBuf::ensure(size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes <= cap) return MG_OK;
  release();
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    p = nullptr;
    cap = 0;
    cudaGetLastError();
    return fail(MG_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
  }
  cap = bytes;
  return MG_OK;
}
void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}

}  // namespace mg

using namespace mg;


struct mg_plan {
  mg_ctx* ctx = nullptr;
  int device = 0;  // destroy must not touch ctx, which may already be gone
  // geometry and configuration
  int W = 0, H = 0, gw = 0, gh = 0, cw = 0, ch = 0, tw = 0, th = 0, N = 0, P = 0, K = 0, k = 0;
  int64_t iters = 0;
  float weight = 0, strength = 0, t0 = 100.0f, decay = 0.99995f;
  int max_usage = 0, enable_opt = 0, build_sim = 0, device_thumbs = 0, run_sa = 0, scoring = 0;
  uint64_t seed = 0;
  uint32_t stream_id = 0;
  std::vector<int> selected;
  std::vector<Region> h_regions;
  // device buffers
  DevBuf target, mats, regions, thumb_regions, thumbs, pal_lab, thumb_rgb, sim, cell_lab, cell_rgb, cand_idx,
      cand_dist, grid_greedy, resets, init_cost, greedy_job, chain_grids, chain_res, anneal_job, final_grid,
      finals_ptr, best_chain, adj, out, sums, cell_sums, err, usage, gather_src;
  LabIndex index;  // bucket grid over pal_lab for the k-nearest search (when large)
  ResizePlan resize;  // Lanczos3 tables of the selected materials (thumbnails made on the device)
  int thumb_filter = MG_THUMB_LANCZOS3;
  // pinned host staging of the small read-backs (grid, counters, chain results)
  void* h_read = nullptr;
  size_t h_read_cap = 0;
  // pinned host staging of the small uploads of a setup (regions, gather sources,
  // job structs); reused by the next setup, which follows the previous job's
  // read-back (a synchronisation), so no setup has to wait for its own copies
  void* h_up = nullptr;
  size_t h_up_cap = 0, h_up_used = 0;
  // Where the kernels read the target (a device copy, or pinned host memory in place).
  bool zero_copy = false;
  const uint8_t* target_ptr = nullptr;
  int64_t target_stride = 0;
  cudaEvent_t ev[9] = {};  // stage boundaries [0..7]; [8] joins the side stream
  // mg_generate with a pinned image buffer: downloaded band by band on the side
  // stream while the next band is composited (nullptr: one composite, no download)
  uint8_t* out_host = nullptr;
  static constexpr int kBands = 4;
  cudaEvent_t band_ev[kBands] = {};
  cudaEvent_t download_done = nullptr;
  uint8_t* downloaded_to = nullptr;  // where the last run's bands went
  bool events = false;
  int launches = 0;
  bool ran = false;
};

namespace mg {

int check_ctx(mg_ctx* ctx) {
  if (!ctx) return fail(MG_ERR_ARG, "null context");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  return MG_OK;
}

std::vector<float4> to_f4(const float* lab3, int n) {
  std::vector<float4> v((size_t)std::max(n, 1));
  for (int i = 0; i < n; ++i) v[i] = make_float4(lab3[3 * i], lab3[3 * i + 1], lab3[3 * i + 2], 0.0f);
  return v;
}

int upload(mg_ctx* ctx, DevBuf& b, const void* src, size_t bytes) {
  MG_CHECK(b.ensure(bytes));
  if (bytes) MG_CUDA(cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return MG_OK;
}

int finish(mg_ctx* ctx) {
  MG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ctx->err.p) {
    uint32_t e = 0;
    MG_CUDA(cudaMemcpy(&e, ctx->err.p, 4, cudaMemcpyDeviceToHost));
    if (e) {
      MG_CUDA(cudaMemset(ctx->err.p, 0, 4));
      return fail(MG_ERR_TIMEOUT, "a bounded wait inside a kernel ran out");
    }
  }
  return MG_OK;
}

int ensure_err(mg_ctx* ctx) {
  if (!ctx->err.p) {
    MG_CHECK(ctx->err.ensure(16));
    MG_CUDA(cudaMemsetAsync(ctx->err.p, 0, 16, ctx->stream));
  }
  return MG_OK;
}

// Device address of caller memory that kernels may read in place: pinned,
// mapped host memory (reached over the CPU-GPU link).  nullptr otherwise.
const void* device_view(const void* p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Device views of caller buffers for one setup: the first query of a pinned
// allocation also records its extent (the driver's range attributes), so the
// other buffers inside it -- hundreds of materials packed in one pinned block,
// say -- need no query.  Kept for one call only: allocations change between calls.
struct ViewCache {
  struct Range {
    uintptr_t lo, hi;
    intptr_t delta;  // device address - host address
  };
  std::vector<Range> ranges;
  const void* view(const void* p, size_t bytes) {
    const uintptr_t u = (uintptr_t)p;
    for (const Range& r : ranges)
      if (u >= r.lo && u + bytes <= r.hi) return (const void*)(u + r.delta);
    const void* d = device_view(p);
    if (!d) return nullptr;
    using GetAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
    static GetAttr get = [] {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
          q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        fn = nullptr;
      }
      return reinterpret_cast<GetAttr>(fn);
    }();
    CUdeviceptr start = 0;
    size_t size = 0;
    if (get && get(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)u) == CUDA_SUCCESS &&
        get(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)u) == CUDA_SUCCESS && size > 0 && (uintptr_t)start <= u &&
        u + bytes <= (uintptr_t)start + size)
      ranges.push_back(Range{(uintptr_t)start, (uintptr_t)start + size, (intptr_t)(uintptr_t)d - (intptr_t)u});
    return d;
  }
};

const void* device_view_or_device(const void* p) {
  cudaPointerAttributes a;
  if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
    return a.devicePointer;
  return nullptr;
}

bool valid_image(const void* p, int w, int h, int64_t stride) {
  return p && w > 0 && h > 0 && stride >= 3ll * w;
}

const LabConsts* device_lab_consts(mg_ctx* ctx) {
  if (!ctx->lab_consts.p) {
    if (ctx->lab_consts.ensure(sizeof(LabConsts)) != MG_OK) return nullptr;
    if (cudaMemcpy(ctx->lab_consts.p, &host_lab_consts(), sizeof(LabConsts), cudaMemcpyHostToDevice) != cudaSuccess)
      return nullptr;
  }
  return ctx->lab_consts.as<LabConsts>();
}

}  // namespace mg

extern "C" {

int mg_version(void) { return 10000; }
const char* mg_last_error(void) { return g_error.c_str(); }
unsigned long long mg_kernel_launches(void) { return g_launches; }

int mg_ctx_create(int device, mg_ctx** out) {
  if (!out) return fail(MG_ERR_ARG, "null out");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return fail(MG_ERR_CUDA, "no CUDA device available");
  }
  if (device < 0 || device >= n) return fail(MG_ERR_ARG, "device index out of range");
  MG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  MG_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) return fail(MG_ERR_CUDA, "this library is built for sm_103a (Blackwell Ultra)");
  mg_ctx* c = new mg_ctx();
  c->device = device;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(e, "cudaStreamCreate");
  }
  const cudaError_t ue = upload_lab_consts(c->stream);
  int s = ue == cudaSuccess ? MG_OK : cuda_fail(ue, "upload_lab_consts");
  if (s == MG_OK) s = ensure_err(c);
  if (s == MG_OK) s = finish(c);
  if (s != MG_OK) {
    mg_ctx_destroy(c);
    return s;
  }
  *out = c;
  return MG_OK;
}

int mg_ctx_destroy(mg_ctx* ctx) {
  if (!ctx) return MG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->gen_plan) mg_plan_destroy(ctx->gen_plan);
  if (ctx->gen_batch) mg::batch_free(ctx->gen_batch);
  for (int g = 0; g < mg::kGenGroups; ++g) {
    if (ctx->gen_sub_batch[g]) mg::batch_free(ctx->gen_sub_batch[g]);
    if (ctx->gen_sub[g]) mg_ctx_destroy(ctx->gen_sub[g]);
  }
  for (cudaStream_t cs : {ctx->gen_up, ctx->gen_down})
    if (cs) {
      cudaStreamSynchronize(cs);
      cudaStreamDestroy(cs);
    }
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (DevBuf* b : {&ctx->in0, &ctx->in1, &ctx->in2, &ctx->out0, &ctx->out1, &ctx->out2, &ctx->sums, &ctx->regions,
                    &ctx->err, &ctx->lab_consts})
    b->release();
  ctx->nn_index.release();
  ctx->resize.release();
  if (ctx->side) {
    cudaStreamSynchronize(ctx->side);
    cudaStreamDestroy(ctx->side);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MG_OK;
}

int mg_ctx_sync(mg_ctx* ctx) {
  MG_CHECK(check_ctx(ctx));
  return finish(ctx);
}

void* mg_ctx_stream(mg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int mg_ctx_set_nearest_method(mg_ctx* ctx, int method) {
  if (!ctx) return fail(MG_ERR_ARG, "null context");
  if (method != MG_NEAREST_AUTO && method != MG_NEAREST_SCAN && method != MG_NEAREST_GRID)
    return fail(MG_ERR_ARG, "unknown nearest method");
  ctx->nearest_method = method;
  return MG_OK;
}

int mg_ctx_set_thumbnail_filter(mg_ctx* ctx, int filter) {
  if (!ctx) return fail(MG_ERR_ARG, "null context");
  if (filter != MG_THUMB_LANCZOS3 && filter != MG_THUMB_AREA) return fail(MG_ERR_ARG, "unknown thumbnail filter");
  ctx->thumb_filter = filter;
  return MG_OK;
}

int mg_resize(mg_ctx* ctx, const uint8_t* rgb, int w, int h, int64_t stride, int dw, int dh, uint8_t* out) {
  MG_CHECK(check_ctx(ctx));
  if (stride == 0) stride = 3ll * w;
  if (!valid_image(rgb, w, h, stride) || !out || dw <= 0 || dh <= 0) return fail(MG_ERR_ARG, "invalid image or size");
  const void* dev = device_view_or_device(rgb);
  const uint8_t* src = static_cast<const uint8_t*>(dev);
  if (!dev) {
    MG_CHECK(ctx->in2.ensure((size_t)stride * (h - 1) + 3ull * w));
    MG_CUDA(cudaMemcpy2DAsync(ctx->in2.p, (size_t)stride, rgb, (size_t)stride, 3ull * w, (size_t)h,
                              cudaMemcpyHostToDevice, ctx->stream));
    src = ctx->in2.as<uint8_t>();
  }
  const size_t bytes = 3ull * dw * dh;
  MG_CHECK(ctx->out2.ensure(bytes));
  const Region r{0, w, h, stride};
  if (ctx->thumb_filter == MG_THUMB_LANCZOS3) {
    MG_CHECK(ctx->resize.build(&r, 1, dw, dh, ctx->stream));
    MG_CHECK(launch_resize(src, ctx->resize, ctx->out2.as<uint8_t>(), ctx->stream));
  } else {
    MG_CHECK(upload(ctx, ctx->regions, &r, sizeof(r)));
    MG_CHECK(launch_thumbnails(src, ctx->regions.as<Region>(), 1, dw, dh, ctx->out2.as<uint8_t>(), ctx->stream));
  }
  MG_CUDA(cudaMemcpyAsync(out, ctx->out2.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

int mg_ctx_inject_walk_timeout(mg_ctx* ctx, int walks) {
  if (!ctx) return fail(MG_ERR_ARG, "null context");
  if (walks < 0) return fail(MG_ERR_ARG, "negative walk count");
  ctx->inject_walk_timeouts = walks;
  return MG_OK;
}

int mg_ctx_set_scoring(mg_ctx* ctx, int scoring) {
  if (!ctx) return fail(MG_ERR_ARG, "null context");
  if (scoring != MG_SCORING_CLI && scoring != MG_SCORING_GUI) return fail(MG_ERR_ARG, "unknown scoring");
  ctx->scoring = scoring;
  return MG_OK;
}

void* mg_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes ? bytes : 16, cudaHostAllocPortable | cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaHostAlloc failed");
    return nullptr;
  }
  return p;
}
void mg_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

// ---- colour statistics ----------------------------------------------------------
int mg_average_lab(mg_ctx* ctx, const uint8_t* rgb, int w, int h, int64_t stride, float lab[3]) {
  MG_CHECK(check_ctx(ctx));
  if (!lab || !valid_image(rgb, w, h, stride)) return fail(MG_ERR_ARG, "invalid image");
  const size_t row = 3ull * w;
  MG_CHECK(ctx->in0.ensure(row * h));
  MG_CUDA(cudaMemcpy2DAsync(ctx->in0.p, row, rgb, stride, row, h, cudaMemcpyHostToDevice, ctx->stream));
  Region r{0, w, h, (int64_t)row};
  MG_CHECK(upload(ctx, ctx->regions, &r, sizeof(r)));
  MG_CHECK(ctx->sums.ensure(sizeof(RegionSums)));
  MG_CHECK(ctx->out0.ensure(sizeof(float4)));
  MG_CHECK(launch_region_stats(ctx->in0.as<uint8_t>(), nullptr, ctx->regions.as<Region>(), 1, (int64_t)w * h,
                               ctx->out0.as<float4>(), nullptr, ctx->sums.as<RegionSums>(), 1, ctx->stream));
  float4 v;
  MG_CUDA(cudaMemcpyAsync(&v, ctx->out0.p, sizeof(v), cudaMemcpyDeviceToHost, ctx->stream));
  MG_CHECK(finish(ctx));
  lab[0] = v.x;
  lab[1] = v.y;
  lab[2] = v.z;
  return MG_OK;
}

int mg_is_aspect_ratio_match(float img_aspect, float target_aspect, float tolerance) {
  return std::fabs(img_aspect - target_aspect) <= tolerance ? 1 : 0;
}

int mg_cells_lab(mg_ctx* ctx, const uint8_t* img, int w, int h, int64_t stride, int gw, int gh, float* lab_out,
                 uint8_t* avg_rgb_out) {
  MG_CHECK(check_ctx(ctx));
  if (!valid_image(img, w, h, stride) || !lab_out) return fail(MG_ERR_ARG, "invalid image");
  if (gw <= 0 || gh <= 0 || w / gw <= 0 || h / gh <= 0) return fail(MG_ERR_ARG, "grid larger than the image");
  if ((int64_t)gw * gh > kMaxGridCells) return fail(MG_ERR_ARG, "grid too large");
  const int n = gw * gh;
  const size_t row = 3ull * w;
  MG_CHECK(ctx->in0.ensure(row * h));
  MG_CUDA(cudaMemcpy2DAsync(ctx->in0.p, row, img, stride, row, h, cudaMemcpyHostToDevice, ctx->stream));
  CellGeom g{gw, gh, w / gw, h / gh, (int64_t)row};
  MG_CHECK(ctx->sums.ensure(sizeof(RegionSums) * n));
  MG_CHECK(ctx->out0.ensure(sizeof(float4) * n));
  MG_CHECK(ctx->out1.ensure(sizeof(uchar4) * n));
  MG_CHECK(launch_region_stats(ctx->in0.as<uint8_t>(), &g, nullptr, n, (int64_t)g.cw * g.ch, ctx->out0.as<float4>(),
                               ctx->out1.as<uchar4>(), ctx->sums.as<RegionSums>(), 1, ctx->stream));
  std::vector<float4> lab(n);
  std::vector<uchar4> rgb(n);
  MG_CUDA(cudaMemcpyAsync(lab.data(), ctx->out0.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MG_CUDA(cudaMemcpyAsync(rgb.data(), ctx->out1.p, sizeof(uchar4) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MG_CHECK(finish(ctx));
  for (int i = 0; i < n; ++i) {
    lab_out[3 * i] = lab[i].x;
    lab_out[3 * i + 1] = lab[i].y;
    lab_out[3 * i + 2] = lab[i].z;
    if (avg_rgb_out) {
      avg_rgb_out[3 * i] = rgb[i].x;
      avg_rgb_out[3 * i + 1] = rgb[i].y;
      avg_rgb_out[3 * i + 2] = rgb[i].z;
    }
  }
  return MG_OK;
}

int mg_images_lab(mg_ctx* ctx, const uint8_t* const* imgs, const int* w, const int* h, const int64_t* stride, int n,
                  float* lab_out, uint8_t* avg_rgb_out) {
  MG_CHECK(check_ctx(ctx));
  if (n < 0 || (n > 0 && (!imgs || !w || !h || !lab_out))) return fail(MG_ERR_ARG, "invalid image list");
  if (n == 0) return MG_OK;
  std::vector<Region> regs(n);
  int64_t off = 0, maxpx = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t st = stride ? stride[i] : 3ll * w[i];
    if (!valid_image(imgs[i], w[i], h[i], st)) return fail(MG_ERR_ARG, "invalid image " + std::to_string(i));
    regs[i] = Region{off, w[i], h[i], 3ll * w[i]};
    off += 3ll * w[i] * h[i];
    off = (off + 15) & ~15ll;
    maxpx = std::max<int64_t>(maxpx, (int64_t)w[i] * h[i]);
  }
  MG_CHECK(ctx->in0.ensure((size_t)off));
  for (int i = 0; i < n; ++i) {
    const int64_t st = stride ? stride[i] : 3ll * w[i];
    MG_CUDA(cudaMemcpy2DAsync(ctx->in0.as<uint8_t>() + regs[i].offset, 3ull * w[i], imgs[i], st, 3ull * w[i], h[i],
                              cudaMemcpyHostToDevice, ctx->stream));
  }
  MG_CHECK(upload(ctx, ctx->regions, regs.data(), sizeof(Region) * n));
  MG_CHECK(ctx->sums.ensure(sizeof(RegionSums) * n));
  MG_CHECK(ctx->out0.ensure(sizeof(float4) * n));
  MG_CHECK(ctx->out1.ensure(sizeof(uchar4) * n));
  MG_CHECK(launch_region_stats(ctx->in0.as<uint8_t>(), nullptr, ctx->regions.as<Region>(), n, maxpx,
                               ctx->out0.as<float4>(), ctx->out1.as<uchar4>(), ctx->sums.as<RegionSums>(), 1,
                               ctx->stream));
  std::vector<float4> lab(n);
  std::vector<uchar4> rgb(n);
  MG_CUDA(cudaMemcpyAsync(lab.data(), ctx->out0.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MG_CUDA(cudaMemcpyAsync(rgb.data(), ctx->out1.p, sizeof(uchar4) * n, cudaMemcpyDeviceToHost, ctx->stream));
  MG_CHECK(finish(ctx));
  for (int i = 0; i < n; ++i) {
    lab_out[3 * i] = lab[i].x;
    lab_out[3 * i + 1] = lab[i].y;
    lab_out[3 * i + 2] = lab[i].z;
    if (avg_rgb_out) {
      avg_rgb_out[3 * i] = rgb[i].x;
      avg_rgb_out[3 * i + 1] = rgb[i].y;
      avg_rgb_out[3 * i + 2] = rgb[i].z;
    }
  }
  return MG_OK;
}

int mg_select_palette(const int* widths, const int* heights, int n, float target_aspect, float tolerance,
                      int max_materials, int* selected) {
  if (n < 0 || max_materials < 0 || (n > 0 && (!widths || !heights || !selected))) return -MG_ERR_ARG;
  int cnt = 0;
  for (int i = 0; i < n; ++i) {
    if (heights[i] <= 0 || widths[i] <= 0) return -MG_ERR_ARG;
    const float a = (float)widths[i] / (float)heights[i];
    if (mg_is_aspect_ratio_match(a, target_aspect, tolerance)) selected[cnt++] = i;
  }
  if (cnt == 0) {
    const int64_t lim = std::min<int64_t>(n, 2ll * max_materials);
    for (int64_t i = 0; i < lim; ++i) selected[cnt++] = (int)i;
  }
  return std::min(cnt, max_materials);
}

// ---- similarity --------------------------------------------------------------------
int mg_similarity_build(mg_ctx* ctx, const float* lab, int p, int layout, float* out) {
  MG_CHECK(check_ctx(ctx));
  if (p < 0 || (p > 0 && (!lab || !out))) return fail(MG_ERR_ARG, "invalid palette");
  if (layout != MG_SIM_FULL && layout != MG_SIM_TRIANGULAR) return fail(MG_ERR_ARG, "unknown layout");
  if (p == 0) return MG_OK;
  auto pal = to_f4(lab, p);
  MG_CHECK(upload(ctx, ctx->in1, pal.data(), sizeof(float4) * p));
  const size_t count = layout == MG_SIM_FULL ? (size_t)p * p : (size_t)p * (p - 1) / 2;
  MG_CHECK(ctx->out0.ensure(sizeof(float) * count));
  MG_CHECK(launch_similarity(ctx->in1.as<float4>(), p, layout == MG_SIM_TRIANGULAR, ctx->out0.as<float>(), ctx->stream));
  if (count) MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, sizeof(float) * count, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

float mg_lab_distance(const float a[3], const float b[3]) { return lab_distance(a[0], a[1], a[2], b[0], b[1], b[2]); }

// ---- nearest --------------------------------------------------------------------------
int mg_nearest_n(mg_ctx* ctx, const float* palette_lab, int p, const float* query_lab, int nq, int k,
                 uint32_t* idx_out, float* dist_out) {
  MG_CHECK(check_ctx(ctx));
  if (p < 0 || nq < 0 || k <= 0 || k > 100) return fail(MG_ERR_ARG, "need p >= 0, nq >= 0, 1 <= k <= 100");
  if (nq == 0) return MG_OK;
  if (!query_lab || !idx_out || !dist_out || (p > 0 && !palette_lab)) return fail(MG_ERR_ARG, "null buffer");
  MG_CHECK(ensure_err(ctx));
  auto pal = to_f4(palette_lab, p);
  auto q = to_f4(query_lab, nq);
  MG_CHECK(upload(ctx, ctx->in1, pal.data(), sizeof(float4) * std::max(p, 1)));
  MG_CHECK(upload(ctx, ctx->in2, q.data(), sizeof(float4) * nq));
  MG_CHECK(ctx->out0.ensure(sizeof(uint32_t) * (size_t)nq * k));
  MG_CHECK(ctx->out1.ensure(sizeof(float) * (size_t)nq * k));
  MG_CHECK(ctx->nn_index.build(ctx->in1.as<float4>(), p, ctx->nearest_method, k, ctx->stream));
  MG_CHECK(launch_nearest(ctx->in1.as<float4>(), p, ctx->in2.as<float4>(), nq, k, ctx->out0.as<uint32_t>(),
                          ctx->out1.as<float>(), ctx->err.as<uint32_t>(), ctx->stream, 2048, &ctx->nn_index));
  if (p == 0) {
    MG_CHECK(finish(ctx));
    for (size_t i = 0; i < (size_t)nq * k; ++i) {
      idx_out[i] = 0xFFFFFFFFu;
      dist_out[i] = INFINITY;
    }
    return MG_OK;
  }
  MG_CUDA(cudaMemcpyAsync(idx_out, ctx->out0.p, sizeof(uint32_t) * (size_t)nq * k, cudaMemcpyDeviceToHost, ctx->stream));
  MG_CUDA(cudaMemcpyAsync(dist_out, ctx->out1.p, sizeof(float) * (size_t)nq * k, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

// ---- adjacency ----------------------------------------------------------------------------
static int check_grid(const float* pal, int p, const int32_t* grid, int gw, int gh) {
  if (gw <= 0 || gh <= 0 || !grid || p < 0 || (p > 0 && !pal)) return fail(MG_ERR_ARG, "invalid grid or palette");
  if ((int64_t)gw * gh > kMaxGridCells) return fail(MG_ERR_ARG, "grid too large");
  for (int i = 0; i < gw * gh; ++i)
    if (grid[i] < -1 || grid[i] >= p) return fail(MG_ERR_ARG, "grid entry out of palette range");
  return MG_OK;
}

int mg_penalty_batch(mg_ctx* ctx, const float* palette_lab, int p, const int32_t* grid, int gw, int gh, float weight,
                     const int32_t* cxy, int n, float* out) {
  MG_CHECK(check_ctx(ctx));
  MG_CHECK(check_grid(palette_lab, p, grid, gw, gh));
  if (n < 0 || (n > 0 && (!cxy || !out))) return fail(MG_ERR_ARG, "invalid items");
  if (n == 0) return MG_OK;
  std::vector<int4> items(n);
  for (int i = 0; i < n; ++i) {
    items[i] = make_int4(cxy[3 * i], cxy[3 * i + 1], cxy[3 * i + 2], 0);
    if (items[i].x < 0 || items[i].x >= p || items[i].y < 0 || items[i].y >= gw || items[i].z < 0 || items[i].z >= gh)
      return fail(MG_ERR_ARG, "item out of range");
  }
  auto pal = to_f4(palette_lab, p);
  MG_CHECK(upload(ctx, ctx->in0, pal.data(), sizeof(float4) * std::max(p, 1)));
  MG_CHECK(upload(ctx, ctx->in1, grid, sizeof(int32_t) * gw * gh));
  MG_CHECK(upload(ctx, ctx->in2, items.data(), sizeof(int4) * n));
  MG_CHECK(ctx->out0.ensure(sizeof(float) * n));
  MG_CHECK(launch_penalty(ctx->in0.as<float4>(), ctx->in1.as<int32_t>(), gw, gh, weight, ctx->in2.as<int4>(), n,
                          ctx->out0.as<float>(), ctx->stream));
  MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

int mg_total_cost(mg_ctx* ctx, const float* palette_lab, int p, const int32_t* grid, int gw, int gh, float* out) {
  MG_CHECK(check_ctx(ctx));
  if (!out) return fail(MG_ERR_ARG, "null out");
  if (gh == 0 || gw == 0) {  // adjacency.rs:92-95: an empty grid costs 0
    *out = 0.0f;
    return MG_OK;
  }
  MG_CHECK(check_grid(palette_lab, p, grid, gw, gh));
  auto pal = to_f4(palette_lab, p);
  MG_CHECK(upload(ctx, ctx->in0, pal.data(), sizeof(float4) * std::max(p, 1)));
  MG_CHECK(upload(ctx, ctx->in1, grid, sizeof(int32_t) * gw * gh));
  MG_CHECK(ctx->out0.ensure(sizeof(float)));
  MG_CHECK(launch_total_cost(ctx->in0.as<float4>(), ctx->in1.as<int32_t>(), gw, gh, ctx->out0.as<float>(), ctx->stream));
  MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

int mg_swap_delta_batch(mg_ctx* ctx, const float* palette_lab, int p, const int32_t* grid, int gw, int gh,
                        const int32_t* pairs, int n, float* out) {
  MG_CHECK(check_ctx(ctx));
  MG_CHECK(check_grid(palette_lab, p, grid, gw, gh));
  if (n < 0 || (n > 0 && (!pairs || !out))) return fail(MG_ERR_ARG, "invalid pairs");
  if (n == 0) return MG_OK;
  for (int i = 0; i < n; ++i) {
    const int* q = pairs + 4 * i;
    if (q[0] < 0 || q[0] >= gw || q[2] < 0 || q[2] >= gw || q[1] < 0 || q[1] >= gh || q[3] < 0 || q[3] >= gh)
      return fail(MG_ERR_ARG, "position out of range");
  }
  auto pal = to_f4(palette_lab, p);
  MG_CHECK(upload(ctx, ctx->in0, pal.data(), sizeof(float4) * std::max(p, 1)));
  MG_CHECK(upload(ctx, ctx->in1, grid, sizeof(int32_t) * gw * gh));
  MG_CHECK(upload(ctx, ctx->in2, pairs, sizeof(int4) * n));
  MG_CHECK(ctx->out0.ensure(sizeof(float) * n));
  MG_CHECK(launch_swap_delta(ctx->in0.as<float4>(), ctx->in1.as<int32_t>(), gw, gh, ctx->in2.as<int4>(), n,
                             ctx->out0.as<float>(), ctx->stream));
  MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

// ---- greedy --------------------------------------------------------------------------------
int mg_place_greedy(mg_ctx* ctx, const float* palette_lab, int p, const float* cell_lab, int gw, int gh,
                    const mg_place_config* cfg, int32_t* grid_out, int* n_resets) {
  MG_CHECK(check_ctx(ctx));
  if (!cfg || !cell_lab || !grid_out || gw <= 0 || gh <= 0 || p < 0 || (p > 0 && !palette_lab) ||
      (int64_t)gw * gh > kMaxGridCells)
    return fail(MG_ERR_ARG, "invalid arguments");
  if (cfg->max_usage_per_image < 0) return fail(MG_ERR_ARG, "negative max usage");
  const int n = gw * gh;
  if (p == 0) {  // main.rs:341-345: no tiles -> nothing placed
    for (int i = 0; i < n; ++i) grid_out[i] = -1;
    if (n_resets) *n_resets = 0;
    return MG_OK;
  }
  MG_CHECK(ensure_err(ctx));
  const int k = std::min(p, 100);
  auto pal = to_f4(palette_lab, p);
  auto q = to_f4(cell_lab, n);
  MG_CHECK(upload(ctx, ctx->in0, pal.data(), sizeof(float4) * p));
  MG_CHECK(upload(ctx, ctx->in1, q.data(), sizeof(float4) * n));
  MG_CHECK(ctx->out0.ensure(sizeof(uint32_t) * padded_cells(n) * k));
  MG_CHECK(ctx->out1.ensure(sizeof(float) * padded_cells(n) * k));
  MG_CHECK(ctx->out2.ensure(sizeof(int32_t) * n + 64));
  MG_CHECK(ctx->sums.ensure(sizeof(uint32_t) * p));
  MG_CHECK(ctx->nn_index.build(ctx->in0.as<float4>(), p, ctx->nearest_method, k, ctx->stream));
  MG_CHECK(launch_nearest(ctx->in0.as<float4>(), p, ctx->in1.as<float4>(), n, k, ctx->out0.as<uint32_t>(),
                          ctx->out1.as<float>(), ctx->err.as<uint32_t>(), ctx->stream, 2048, &ctx->nn_index));
  if (ctx->scoring == MG_SCORING_GUI) MG_CHECK(launch_sqrt_inplace(ctx->out1.as<float>(), (size_t)n * k, ctx->stream));
  int32_t* d_grid = ctx->out2.as<int32_t>();
  int* d_resets = reinterpret_cast<int*>(d_grid + n);
  GreedyJob job{ctx->out0.as<uint32_t>(), ctx->out1.as<float>(), d_grid, gw, gh, k,
                (uint32_t)cfg->max_usage_per_image, cfg->adjacency_penalty_weight, d_resets, nullptr};
  MG_CHECK(upload(ctx, ctx->regions, &job, sizeof(job)));
  const bool inject = ctx->inject_walk_timeouts > 0;
  if (inject) --ctx->inject_walk_timeouts;
  MG_CHECK(launch_greedy(ctx->in0.as<float4>(), p, ctx->regions.as<GreedyJob>(), 1, k, gw, n,
                         ctx->sums.as<uint32_t>(), ctx->err.as<uint32_t>(), ctx->stream, false, inject));
  MG_CUDA(cudaMemcpyAsync(grid_out, d_grid, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
  int resets = 0;
  MG_CUDA(cudaMemcpyAsync(&resets, d_resets, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MG_CHECK(finish(ctx));
  if (n_resets) *n_resets = resets;
  return MG_OK;
}

// ---- annealing --------------------------------------------------------------------------------
void mg_sa_config_default(mg_sa_config* cfg) {
  if (!cfg) return;
  cfg->max_iterations = 1000;
  cfg->initial_temperature = 100.0f;
  cfg->temperature_decay = 0.99995f;
  cfg->chains = 1;
  cfg->seed = 0x5eed5eed5eedull;
  cfg->stream = 0;
  cfg->greedy_only = 0;
}

float mg_improvement_percentage(const mg_sa_result* r) {
  if (!r) return 0.0f;
  if (r->initial_cost > 0.0f) return ((r->initial_cost - r->final_cost) / r->initial_cost) * 100.0f;
  return 0.0f;
}

static void to_result(const ChainResult& c, int64_t iters, int chain, mg_sa_result* r) {
  r->initial_cost = c.initial_cost;
  r->final_cost = c.final_cost;
  r->best_cost = c.best_cost;
  r->improved_count = c.improved;
  r->accepted_count = c.accepted;
  r->iterations = iters;
  r->best_chain = chain;
}

int mg_optimize(mg_ctx* ctx, const float* palette_lab, int p, int32_t* grid, int gw, int gh, const mg_sa_config* cfg,
                mg_sa_result* best, mg_sa_result* per_chain, int32_t* chain_grids) {
  MG_CHECK(check_ctx(ctx));
  if (!cfg || !best) return fail(MG_ERR_ARG, "null config or result");
  if (cfg->chains < 1 || cfg->max_iterations < 0) return fail(MG_ERR_ARG, "need chains >= 1, iterations >= 0");
  if (gh == 0 || gw == 0) {  // optimizer.rs:42-46: empty grid -> default result
    std::memset(best, 0, sizeof(*best));
    best->best_chain = 0;
    return MG_OK;
  }
  MG_CHECK(check_grid(palette_lab, p, grid, gw, gh));
  const int n = gw * gh, K = cfg->chains;
  auto pal = to_f4(palette_lab, p);
  MG_CHECK(upload(ctx, ctx->in0, pal.data(), sizeof(float4) * std::max(p, 1)));
  MG_CHECK(upload(ctx, ctx->in1, grid, sizeof(int32_t) * n));
  MG_CHECK(ctx->out0.ensure(sizeof(int32_t) * (size_t)n * K));
  MG_CHECK(ctx->out1.ensure(sizeof(ChainResult) * K));
  MG_CHECK(ctx->out2.ensure(sizeof(int32_t) * n + 64));
  AnnealJob job{};
  job.grid_in = ctx->in1.as<int32_t>();
  job.chain_grids = ctx->out0.as<int32_t>();
  job.results = ctx->out1.as<ChainResult>();
  job.initial_cost = nullptr;
  job.gw = gw;
  job.gh = gh;
  job.chains = K;
  job.iters = cfg->max_iterations;
  job.t0 = cfg->initial_temperature;
  job.decay = cfg->temperature_decay;
  job.key0 = (uint32_t)cfg->seed;
  job.key1 = (uint32_t)(cfg->seed >> 32);
  job.stream = cfg->stream;
  job.greedy_only = cfg->greedy_only;
  struct {
    AnnealJob job;
    int32_t* final_ptr;
  } blob{job, ctx->out2.as<int32_t>()};
  MG_CHECK(upload(ctx, ctx->regions, &blob, sizeof(blob)));
  const AnnealJob* d_job = ctx->regions.as<AnnealJob>();
  int32_t* const* d_final = reinterpret_cast<int32_t* const*>(ctx->regions.as<uint8_t>() + offsetof(decltype(blob), final_ptr));
  int* d_best = reinterpret_cast<int*>(ctx->out2.as<int32_t>() + n);
  MG_CHECK(launch_anneal(ctx->in0.as<float4>(), std::max(p, 1), d_job, nullptr, nullptr, K, n, ctx->stream));
  MG_CHECK(launch_select_best(d_job, 1, d_final, d_best, ctx->stream));
  std::vector<ChainResult> res(K);
  int bc = 0;
  MG_CUDA(cudaMemcpyAsync(res.data(), ctx->out1.p, sizeof(ChainResult) * K, cudaMemcpyDeviceToHost, ctx->stream));
  MG_CUDA(cudaMemcpyAsync(&bc, d_best, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MG_CUDA(cudaMemcpyAsync(grid, ctx->out2.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
  if (chain_grids)
    MG_CUDA(cudaMemcpyAsync(chain_grids, ctx->out0.p, sizeof(int32_t) * (size_t)n * K, cudaMemcpyDeviceToHost,
                            ctx->stream));
  MG_CHECK(finish(ctx));
  to_result(res[bc], cfg->max_iterations, bc, best);
  if (per_chain)
    for (int c = 0; c < K; ++c) to_result(res[c], cfg->max_iterations, c, per_chain + c);
  return MG_OK;
}

// ---- colour adjustment -----------------------------------------------------------------------------
mg_color_adjustment mg_color_adjustment_new(float brightness, float contrast, float hue_shift, float saturation) {
  Adjust a = adjustment_new(brightness, contrast, hue_shift, saturation);
  return mg_color_adjustment{a.brightness, a.contrast, a.hue_shift, a.saturation};
}

int mg_optimal_adjustment_batch(mg_ctx* ctx, const uint8_t* tile_rgb, const uint8_t* target_rgb, int n, float strength,
                                mg_color_adjustment* out) {
  MG_CHECK(check_ctx(ctx));
  if (n < 0 || (n > 0 && (!tile_rgb || !target_rgb || !out))) return fail(MG_ERR_ARG, "invalid arguments");
  if (n == 0) return MG_OK;
  MG_CHECK(upload(ctx, ctx->in0, tile_rgb, 3ull * n));
  MG_CHECK(upload(ctx, ctx->in1, target_rgb, 3ull * n));
  MG_CHECK(ctx->out0.ensure(sizeof(float4) * n));
  MG_CHECK(launch_optimal_adjustment(ctx->in0.as<uint8_t>(), ctx->in1.as<uint8_t>(), n, strength,
                                     ctx->out0.as<float4>(), ctx->stream));
  static_assert(sizeof(mg_color_adjustment) == sizeof(float4), "layout");
  MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

int mg_apply_adjustment(mg_ctx* ctx, const mg_color_adjustment* adj, const uint8_t* rgb, int w, int h, int64_t stride,
                        uint8_t* out) {
  MG_CHECK(check_ctx(ctx));
  if (!adj || !out || !valid_image(rgb, w, h, stride)) return fail(MG_ERR_ARG, "invalid arguments");
  const size_t row = 3ull * w;
  MG_CHECK(ctx->in0.ensure(row * h));
  MG_CUDA(cudaMemcpy2DAsync(ctx->in0.p, row, rgb, stride, row, h, cudaMemcpyHostToDevice, ctx->stream));
  MG_CHECK(ctx->out0.ensure(row * h));
  MG_CHECK(launch_adjust_image(make_float4(adj->brightness, adj->contrast, adj->hue_shift, adj->saturation),
                               ctx->in0.as<uint8_t>(), w, h, (int64_t)row, ctx->out0.as<uint8_t>(), ctx->stream));
  MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, row * h, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

int mg_composite(mg_ctx* ctx, const int32_t* grid, int gw, int gh, const uint8_t* thumbs, int p, int tw, int th,
                 const uint8_t* cell_avg_rgb, float strength, uint8_t* out) {
  MG_CHECK(check_ctx(ctx));
  if (!grid || !out || gw <= 0 || gh <= 0 || tw <= 0 || th <= 0 || p < 0 || (p > 0 && !thumbs) ||
      (int64_t)gw * gh > kMaxGridCells || (int64_t)gw * tw > INT32_MAX / 3 || (int64_t)gh * th > INT32_MAX)
    return fail(MG_ERR_ARG, "invalid arguments");
  const bool adjust = strength > 0.0f;
  if (adjust && !cell_avg_rgb) return fail(MG_ERR_ARG, "cell_avg_rgb required when strength > 0");
  const int n = gw * gh;
  for (int i = 0; i < n; ++i)
    if (grid[i] < -1 || grid[i] >= p) return fail(MG_ERR_ARG, "grid entry out of palette range");
  const size_t tb = 3ull * tw * th;
  MG_CHECK(upload(ctx, ctx->in0, thumbs, tb * std::max(p, 1) * (p > 0)));
  MG_CHECK(upload(ctx, ctx->in1, grid, sizeof(int32_t) * n));
  MG_CHECK(ctx->out0.ensure(tb * n));
  if (adjust && p > 0) {
    // thumbnail means (main.rs:557) and cell means -> per-cell adjustment
    std::vector<Region> regs(p);
    for (int i = 0; i < p; ++i) regs[i] = Region{(int64_t)(tb * i), tw, th, 3ll * tw};
    MG_CHECK(upload(ctx, ctx->regions, regs.data(), sizeof(Region) * p));
    MG_CHECK(ctx->sums.ensure(sizeof(RegionSums) * p));
    MG_CHECK(ctx->out1.ensure(sizeof(uchar4) * p + sizeof(uchar4) * n + sizeof(float4) * n + 64));
    uchar4* thumb_rgb = ctx->out1.as<uchar4>();
    uchar4* cell_rgb = thumb_rgb + p;
    float4* adjv = reinterpret_cast<float4*>(ctx->out1.as<uint8_t>() + (((sizeof(uchar4) * (p + n)) + 15) & ~15ull));
    MG_CHECK(launch_region_stats(ctx->in0.as<uint8_t>(), nullptr, ctx->regions.as<Region>(), p, (int64_t)tw * th,
                                 nullptr, thumb_rgb, ctx->sums.as<RegionSums>(), 0, ctx->stream));
    std::vector<uchar4> crgb(n);
    for (int i = 0; i < n; ++i) crgb[i] = make_uchar4(cell_avg_rgb[3 * i], cell_avg_rgb[3 * i + 1], cell_avg_rgb[3 * i + 2], 0);
    MG_CUDA(cudaMemcpyAsync(cell_rgb, crgb.data(), sizeof(uchar4) * n, cudaMemcpyHostToDevice, ctx->stream));
    MG_CHECK(launch_cell_adjust(ctx->in1.as<int32_t>(), n, thumb_rgb, cell_rgb, strength, adjv,
                                ctx->stream));
    MG_CHECK(launch_composite(ctx->in1.as<int32_t>(), gw, gh, ctx->in0.as<uint8_t>(), tw, th, adjv, 1,
                              ctx->out0.as<uint8_t>(), ctx->stream));
    MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, tb * n, cudaMemcpyDeviceToHost, ctx->stream));
    return finish(ctx);
  }
  MG_CHECK(launch_composite(ctx->in1.as<int32_t>(), gw, gh, ctx->in0.as<uint8_t>(), tw, th, nullptr, 0,
                            ctx->out0.as<uint8_t>(), ctx->stream));
  MG_CUDA(cudaMemcpyAsync(out, ctx->out0.p, tb * n, cudaMemcpyDeviceToHost, ctx->stream));
  return finish(ctx);
}

// ---- the whole job -------------------------------------------------------------------------------
void mg_request_default(mg_request* r) {
  if (!r) return;
  std::memset(r, 0, sizeof(*r));
  r->grid_w = 50;  // main.rs:37-43 defaults
  r->grid_h = 28;
  r->max_materials = 500;
  r->aspect_tolerance = 0.1f;
  r->max_usage_per_image = 3;
  r->adjacency_penalty_weight = 0.3f;
  r->color_adjustment_strength = 0.3f;
  r->enable_optimization = 1;
  r->optimization_iterations = 1000;
  r->initial_temperature = 100.0f;
  r->temperature_decay = 0.99995f;
  r->chains = 1;
  r->seed = 0x5eed5eed5eedull;
  r->build_similarity = 1;
}

}  // extern "C"

namespace {

void plan_release(mg_plan* pl) {
  if (pl->h_up) cudaFreeHost(pl->h_up);
  pl->h_up = nullptr;
  pl->h_up_cap = pl->h_up_used = 0;
  if (pl->h_read) cudaFreeHost(pl->h_read);
  pl->h_read = nullptr;
  pl->h_read_cap = 0;
  for (DevBuf* b : {&pl->target, &pl->mats, &pl->regions, &pl->thumb_regions, &pl->thumbs, &pl->pal_lab,
                    &pl->thumb_rgb, &pl->sim, &pl->cell_lab, &pl->cell_rgb, &pl->cand_idx, &pl->cand_dist,
                    &pl->grid_greedy, &pl->resets, &pl->init_cost, &pl->greedy_job, &pl->chain_grids, &pl->chain_res,
                    &pl->anneal_job, &pl->final_grid, &pl->finals_ptr, &pl->best_chain, &pl->adj, &pl->out, &pl->sums, &pl->cell_sums, &pl->usage, &pl->gather_src,
                    &pl->err})
    b->release();
  pl->index.release();
  pl->resize.release();
  if (pl->events)
    for (auto& e : pl->ev) cudaEventDestroy(e);
  if (pl->download_done) {
    for (auto& e : pl->band_ev) cudaEventDestroy(e);
    cudaEventDestroy(pl->download_done);
    pl->download_done = nullptr;
  }
  pl->events = false;
}

// Validate the request, select the palette and upload the inputs.
int plan_setup(mg_plan* pl, mg_ctx* ctx, const mg_request* r, bool zero_copy) {
  if (!r) return fail(MG_ERR_ARG, "null request");
  if (!valid_image(r->target, r->target_w, r->target_h, r->target_stride ? r->target_stride : 3ll * r->target_w))
    return fail(MG_ERR_ARG, "invalid target image");
  if (r->grid_w <= 0 || r->grid_h <= 0) return fail(MG_ERR_ARG, "grid dimensions must be positive");
  if (r->target_w / r->grid_w <= 0 || r->target_h / r->grid_h <= 0) return fail(MG_ERR_ARG, "grid larger than the target");
  if (r->n_materials < 0 || (r->n_materials > 0 && (!r->materials || !r->material_w || !r->material_h)))
    return fail(MG_ERR_ARG, "invalid material list");
  if (r->max_materials < 0 || r->max_usage_per_image < 0 || r->tile_w < 0 || r->tile_h < 0)
    return fail(MG_ERR_ARG, "negative size parameter");
  if (r->enable_optimization && (r->chains < 1 || r->optimization_iterations < 0))
    return fail(MG_ERR_ARG, "need chains >= 1 and iterations >= 0");
  pl->ctx = ctx;
  pl->device = ctx->device;
  pl->zero_copy = zero_copy;
  pl->W = r->target_w;
  pl->H = r->target_h;
  pl->gw = r->grid_w;
  pl->gh = r->grid_h;
  pl->cw = pl->W / pl->gw;
  pl->ch = pl->H / pl->gh;
  pl->tw = r->tile_w ? r->tile_w : pl->cw;
  pl->th = r->tile_h ? r->tile_h : pl->ch;
  // cell indices and output rows are 32-bit on the device
  if ((int64_t)pl->gw * pl->gh > kMaxGridCells || (int64_t)pl->gw * pl->tw > INT32_MAX / 3 ||
      (int64_t)pl->gh * pl->th > INT32_MAX)
    return fail(MG_ERR_ARG, "grid or output image too large");
  pl->N = pl->gw * pl->gh;
  pl->weight = r->adjacency_penalty_weight;
  pl->strength = rclamp(r->color_adjustment_strength, 0.0f, 1.0f);
  pl->max_usage = r->max_usage_per_image;
  pl->enable_opt = r->enable_optimization;
  pl->iters = r->optimization_iterations;
  pl->t0 = r->initial_temperature;
  pl->decay = r->temperature_decay;
  pl->K = r->enable_optimization ? r->chains : 0;
  pl->seed = r->seed;
  pl->stream_id = r->stream;
  pl->build_sim = r->build_similarity;
  pl->scoring = ctx->scoring;
  // palette selection (main.rs:166-261)
  pl->selected.assign(std::max(r->n_materials, 1), 0);
  const float target_aspect = (float)r->target_w / (float)r->target_h;
  int P = mg_select_palette(r->material_w, r->material_h, r->n_materials, target_aspect, r->aspect_tolerance,
                            r->max_materials, pl->selected.data());
  if (P < 0) return fail(MG_ERR_ARG, "invalid material sizes");
  pl->selected.resize(P);
  pl->P = P;
  pl->k = std::min(P, 100);
  if (P >= 65535) return fail(MG_ERR_ARG, "palette too large (max 65534 materials)");
  pl->run_sa = pl->enable_opt && pl->weight > 0.0f && P > 0;  // main.rs:608
  if (pl->run_sa && (size_t)pl->N * 2 > 200 * 1024) return fail(MG_ERR_ARG, "grid too large for the annealer");
  cudaStream_t s = ctx->stream;
  // Inputs in pinned host memory are read by the kernels in place over the
  // CPU-GPU link when the plan allows it (mg_generate); otherwise (and for
  // mg_plan_create, whose point is device-resident inputs) they are copied.
  // Regions carry absolute device addresses, so both kinds mix freely.
  // target
  const size_t trow = 3ull * pl->W;
  const int64_t tstride = r->target_stride ? r->target_stride : (int64_t)trow;
  const void* tdev = pl->zero_copy ? device_view(r->target) : nullptr;
  if (tdev) {
    pl->target_ptr = static_cast<const uint8_t*>(tdev);
    pl->target_stride = tstride;
  } else {
    MG_CHECK(pl->target.ensure(trow * pl->H));
    MG_CUDA(cudaMemcpy2DAsync(pl->target.p, trow, r->target, tstride, trow, pl->H, cudaMemcpyHostToDevice, s));
    pl->target_ptr = pl->target.as<uint8_t>();
    pl->target_stride = (int64_t)trow;
  }
  // the small uploads go through the plan's pinned staging block
  {
    const size_t need = 2 * sizeof(Region) * std::max(P, 1) + sizeof(int64_t) * std::max(P, 1) + sizeof(GreedyJob) +
                        sizeof(AnnealJob) + sizeof(int32_t*) + 16 * 8;
    if (pl->h_up_cap < need) {
      if (pl->h_up) cudaFreeHost(pl->h_up);
      pl->h_up = nullptr;
      pl->h_up_cap = 0;
      MG_CUDA(cudaHostAlloc(&pl->h_up, need, cudaHostAllocDefault));
      pl->h_up_cap = need;
    }
    pl->h_up_used = 0;
  }
  auto upload_staged = [&](void* dst, const void* src, size_t bytes) -> int {
    uint8_t* hp = static_cast<uint8_t*>(pl->h_up) + pl->h_up_used;
    if (pl->h_up_used + bytes > pl->h_up_cap) return fail(MG_ERR_STATE, "upload staging overflow");
    std::memcpy(hp, src, bytes);
    pl->h_up_used += (bytes + 15) & ~(size_t)15;
    MG_CUDA(cudaMemcpyAsync(dst, hp, bytes, cudaMemcpyHostToDevice, s));
    return MG_OK;
  };
  // selected materials
  pl->h_regions.resize(std::max(P, 1));
  std::vector<const void*> mdev(std::max(P, 1), nullptr);
  ViewCache views;
  int64_t off = 0;
  for (int i = 0; i < P; ++i) {
    const int m = pl->selected[i];
    const int64_t st = r->material_stride ? r->material_stride[m] : 3ll * r->material_w[m];
    if (!valid_image(r->materials[m], r->material_w[m], r->material_h[m], st))
      return fail(MG_ERR_ARG, "invalid material " + std::to_string(m));
    mdev[i] = pl->zero_copy ? views.view(r->materials[m], (size_t)st * (r->material_h[m] - 1) + 3ull * r->material_w[m])
                            : nullptr;
    if (mdev[i]) {
      pl->h_regions[i] = Region{(int64_t)(uintptr_t)mdev[i], r->material_w[m], r->material_h[m], st};
    } else {
      pl->h_regions[i] = Region{off, r->material_w[m], r->material_h[m], 3ll * r->material_w[m]};
      off += 3ll * r->material_w[m] * r->material_h[m];
      off = (off + 15) & ~15ll;
    }
  }
  if (off > 0) MG_CHECK(pl->mats.ensure((size_t)off));
  for (int i = 0; i < P; ++i) {
    if (mdev[i]) continue;
    const int m = pl->selected[i];
    const int64_t st = r->material_stride ? r->material_stride[m] : 3ll * r->material_w[m];
    MG_CUDA(cudaMemcpy2DAsync(pl->mats.as<uint8_t>() + pl->h_regions[i].offset, 3ull * r->material_w[m],
                              r->materials[m], st, 3ull * r->material_w[m], r->material_h[m], cudaMemcpyHostToDevice, s));
    pl->h_regions[i].offset += (int64_t)(uintptr_t)pl->mats.p;
  }
  MG_CHECK(pl->regions.ensure(sizeof(Region) * std::max(P, 1)));
  MG_CHECK(upload_staged(pl->regions.p, pl->h_regions.data(), sizeof(Region) * std::max(P, 1)));
  // thumbnails (input, or resized on the device in mg_plan_run)
  const size_t tb = 3ull * pl->tw * pl->th;
  MG_CHECK(pl->thumbs.ensure(tb * std::max(P, 1)));
  pl->device_thumbs = r->thumbnails == nullptr;
  pl->thumb_filter = ctx->thumb_filter;
  if (pl->device_thumbs && pl->thumb_filter == MG_THUMB_LANCZOS3)
    MG_CHECK(pl->resize.build(pl->h_regions.data(), P, pl->tw, pl->th, s));
  if (!pl->device_thumbs) {
    const void* thdev = pl->zero_copy && P > 0 ? device_view(r->thumbnails) : nullptr;
    if (thdev) {
      // One gather kernel pulls the selected thumbnails across the link.
      std::vector<int64_t> src(P);
      for (int i = 0; i < P; ++i) src[i] = (int64_t)(uintptr_t)thdev + (int64_t)(tb * pl->selected[i]);
      MG_CHECK(pl->gather_src.ensure(sizeof(int64_t) * P));
      MG_CHECK(upload_staged(pl->gather_src.p, src.data(), sizeof(int64_t) * P));
      MG_CHECK(launch_gather(pl->gather_src.as<int64_t>(), P, tb, pl->thumbs.as<uint8_t>(), s));
    } else {
      int i = 0;
      while (i < P) {  // merge runs of consecutive selected materials into one copy
        int j = i + 1;
        while (j < P && pl->selected[j] == pl->selected[j - 1] + 1) ++j;
        MG_CUDA(cudaMemcpyAsync(pl->thumbs.as<uint8_t>() + tb * i, r->thumbnails + tb * pl->selected[i], tb * (j - i),
                                cudaMemcpyHostToDevice, s));
        i = j;
      }
    }
  }
  std::vector<Region> tregs(std::max(P, 1));
  for (int i = 0; i < P; ++i) tregs[i] = Region{(int64_t)(tb * i), pl->tw, pl->th, 3ll * pl->tw};
  MG_CHECK(pl->thumb_regions.ensure(sizeof(Region) * std::max(P, 1)));
  MG_CHECK(upload_staged(pl->thumb_regions.p, tregs.data(), sizeof(Region) * std::max(P, 1)));
  // working buffers
  const int N = pl->N, K = std::max(pl->K, 1), k = std::max(pl->k, 1);
  MG_CHECK(pl->pal_lab.ensure(sizeof(float4) * std::max(P, 1)));
  MG_CHECK(pl->thumb_rgb.ensure(sizeof(uchar4) * std::max(P, 1)));
  if (pl->build_sim) MG_CHECK(pl->sim.ensure(sizeof(float) * (size_t)std::max(P, 1) * std::max(P, 1)));
  MG_CHECK(pl->cell_lab.ensure(sizeof(float4) * N));
  MG_CHECK(pl->cell_rgb.ensure(sizeof(uchar4) * N));
  MG_CHECK(pl->cand_idx.ensure(sizeof(uint32_t) * padded_cells(N) * k));
  MG_CHECK(pl->usage.ensure(sizeof(uint32_t) * std::max(P, 1)));
  MG_CHECK(pl->cand_dist.ensure(sizeof(float) * padded_cells(N) * k));
  MG_CHECK(pl->grid_greedy.ensure(sizeof(int32_t) * N));
  MG_CHECK(pl->resets.ensure(16));
  MG_CHECK(pl->init_cost.ensure(16));
  MG_CHECK(pl->chain_grids.ensure(sizeof(int32_t) * (size_t)N * K));
  MG_CHECK(pl->chain_res.ensure(sizeof(ChainResult) * K));
  MG_CHECK(pl->final_grid.ensure(sizeof(int32_t) * N));
  MG_CHECK(pl->best_chain.ensure(16));
  MG_CHECK(pl->adj.ensure(sizeof(float4) * N));
  MG_CHECK(pl->out.ensure(tb * N));
  MG_CHECK(pl->sums.ensure(sizeof(RegionSums) * std::max(P, 1)));
  MG_CHECK(pl->cell_sums.ensure(sizeof(RegionSums) * std::max(N, 1)));
  MG_CHECK(pl->err.ensure(16));
  MG_CUDA(cudaMemsetAsync(pl->err.p, 0, 16, s));
  MG_CUDA(cudaMemsetAsync(pl->resets.p, 0, 16, s));
  GreedyJob gj{pl->cand_idx.as<uint32_t>(), pl->cand_dist.as<float>(), pl->grid_greedy.as<int32_t>(), pl->gw, pl->gh,
               pl->k, (uint32_t)pl->max_usage, pl->weight, pl->resets.as<int>(), pl->init_cost.as<float>()};
  MG_CHECK(pl->greedy_job.ensure(sizeof(GreedyJob)));
  MG_CHECK(upload_staged(pl->greedy_job.p, &gj, sizeof(gj)));
  AnnealJob aj{};
  aj.grid_in = pl->grid_greedy.as<int32_t>();
  aj.chain_grids = pl->chain_grids.as<int32_t>();
  aj.results = pl->chain_res.as<ChainResult>();
  aj.initial_cost = pl->init_cost.as<float>();
  aj.gw = pl->gw;
  aj.gh = pl->gh;
  aj.chains = K;
  aj.iters = pl->iters;
  aj.t0 = pl->t0;
  aj.decay = pl->decay;
  aj.key0 = (uint32_t)pl->seed;
  aj.key1 = (uint32_t)(pl->seed >> 32);
  aj.stream = pl->stream_id;
  aj.greedy_only = 0;
  MG_CHECK(pl->anneal_job.ensure(sizeof(AnnealJob)));
  MG_CHECK(upload_staged(pl->anneal_job.p, &aj, sizeof(aj)));
  int32_t* fp = pl->final_grid.as<int32_t>();
  MG_CHECK(pl->finals_ptr.ensure(sizeof(int32_t*)));
  MG_CHECK(upload_staged(pl->finals_ptr.p, &fp, sizeof(fp)));
  if (!pl->events) {
    for (auto& e : pl->ev) MG_CUDA(cudaEventCreate(&e));
    pl->events = true;
  }
  // mg_plan_create returns with the caller's inputs consumed; mg_generate
  // (zero_copy) reads them during the run and synchronises at its end
  if (!zero_copy) MG_CUDA(cudaStreamSynchronize(s));
  pl->ran = false;
  return MG_OK;
}

int plan_run(mg_plan* pl) {
  mg_ctx* ctx = pl->ctx;
  cudaStream_t s = ctx->stream;
  const unsigned long long l0 = g_launches;
  const int P = pl->P, N = pl->N;
  MG_CUDA(cudaEventRecord(pl->ev[0], s));
  // [2] cell Lab + cell mean RGB needs only the target: on the side stream,
  // overlapping [0] and [1]; joined back before [3]
  cudaStream_t s2 = ctx->side;
  MG_CUDA(cudaStreamWaitEvent(s2, pl->ev[0], 0));
  CellGeom g{pl->gw, pl->gh, pl->cw, pl->ch, pl->target_stride};
  MG_CHECK(launch_region_stats(pl->target_ptr, &g, nullptr, N, (int64_t)pl->cw * pl->ch, pl->cell_lab.as<float4>(),
                               pl->cell_rgb.as<uchar4>(), pl->cell_sums.as<RegionSums>(), 1, s2));
  MG_CUDA(cudaEventRecord(pl->ev[8], s2));
  // [0] palette ingestion: thumbnails (when not given), material Lab, thumbnail means
  if (P > 0) {
    if (pl->device_thumbs && pl->thumb_filter == MG_THUMB_LANCZOS3)
      MG_CHECK(launch_resize(nullptr, pl->resize, pl->thumbs.as<uint8_t>(), s));
    else if (pl->device_thumbs)
      MG_CHECK(launch_thumbnails(nullptr, pl->regions.as<Region>(), P, pl->tw, pl->th,
                                 pl->thumbs.as<uint8_t>(), s));
    int64_t maxpx = 0;
    for (int i = 0; i < P; ++i) maxpx = std::max<int64_t>(maxpx, (int64_t)pl->h_regions[i].w * pl->h_regions[i].h);
    MG_CHECK(launch_region_stats(nullptr, nullptr, pl->regions.as<Region>(), P, maxpx,
                                 pl->pal_lab.as<float4>(), nullptr, pl->sums.as<RegionSums>(), 1, s));
    if (pl->strength > 0.0f)
      MG_CHECK(launch_region_stats(pl->thumbs.as<uint8_t>(), nullptr, pl->thumb_regions.as<Region>(), P,
                                   (int64_t)pl->tw * pl->th, nullptr, pl->thumb_rgb.as<uchar4>(),
                                   pl->sums.as<RegionSums>(), 0, s));
  }
  MG_CUDA(cudaEventRecord(pl->ev[1], s));
  // [1] similarity database (main.rs:120-143)
  if (pl->build_sim && P > 0)
    MG_CHECK(launch_similarity(pl->pal_lab.as<float4>(), P, 0, pl->sim.as<float>(), s));
  MG_CUDA(cudaEventRecord(pl->ev[2], s));
  // [2] (the rest of) cell Lab: the join
  MG_CUDA(cudaStreamWaitEvent(s, pl->ev[8], 0));
  MG_CUDA(cudaEventRecord(pl->ev[3], s));
  // [3] k nearest per cell
  if (P > 0) {
    MG_CHECK(pl->index.build(pl->pal_lab.as<float4>(), P, ctx->nearest_method, pl->k, s));
    MG_CHECK(launch_nearest(pl->pal_lab.as<float4>(), P, pl->cell_lab.as<float4>(), N, pl->k, pl->cand_idx.as<uint32_t>(),
                            pl->cand_dist.as<float>(), pl->err.as<uint32_t>(), s, 2048, &pl->index));
    if (pl->scoring == MG_SCORING_GUI)
      MG_CHECK(launch_sqrt_inplace(pl->cand_dist.as<float>(), (size_t)N * pl->k, s));
  }
  MG_CUDA(cudaEventRecord(pl->ev[4], s));
  // [4] greedy placement
  if (P > 0) {
    const bool inject = pl->ctx->inject_walk_timeouts > 0;
    if (inject) --pl->ctx->inject_walk_timeouts;
    MG_CHECK(launch_greedy(pl->pal_lab.as<float4>(), P, pl->greedy_job.as<GreedyJob>(), 1, pl->k, pl->gw, N,
                           pl->usage.as<uint32_t>(), pl->err.as<uint32_t>(), s, false, inject));
  } else {
    MG_CUDA(cudaMemsetAsync(pl->grid_greedy.p, 0xFF, sizeof(int32_t) * N, s));
  }
  MG_CUDA(cudaEventRecord(pl->ev[5], s));
  // [5] annealing chains + best-chain selection
  const int32_t* final_grid = pl->grid_greedy.as<int32_t>();
  if (pl->run_sa) {
    MG_CHECK(launch_anneal(pl->pal_lab.as<float4>(), P, pl->anneal_job.as<AnnealJob>(), nullptr, nullptr, pl->K, N, s));
    MG_CHECK(launch_select_best(pl->anneal_job.as<AnnealJob>(), 1, pl->finals_ptr.as<int32_t*>(),
                                pl->best_chain.as<int>(), s));
    final_grid = pl->final_grid.as<int32_t>();
  }
  MG_CUDA(cudaEventRecord(pl->ev[6], s));
  // [6] colour adjustment + composite
  const bool adjust = pl->strength > 0.0f && P > 0;
  if (adjust)
    MG_CHECK(launch_cell_adjust(final_grid, N, pl->thumb_rgb.as<uchar4>(), pl->cell_rgb.as<uchar4>(), pl->strength,
                                pl->adj.as<float4>(), s));
  pl->downloaded_to = nullptr;
  if (!pl->out_host || pl->gh < mg_plan::kBands) {
    MG_CHECK(launch_composite(final_grid, pl->gw, pl->gh, pl->thumbs.as<uint8_t>(), pl->tw, pl->th,
                              pl->adj.as<float4>(), adjust ? 1 : 0, pl->out.as<uint8_t>(), s));
  } else {
    // bands of tile rows: band b composited on the stream, then copied to the
    // caller's buffer on the side stream while band b + 1 is composited
    if (!pl->download_done) {
      for (auto& e : pl->band_ev) MG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      MG_CUDA(cudaEventCreateWithFlags(&pl->download_done, cudaEventDisableTiming));
    }
    const size_t row_bytes = 3ull * pl->gw * pl->tw * pl->th;  // one row of tiles in the output
    for (int b = 0; b < mg_plan::kBands; ++b) {
      const int r0 = (int)((int64_t)pl->gh * b / mg_plan::kBands), r1 = (int)((int64_t)pl->gh * (b + 1) / mg_plan::kBands);
      MG_CHECK(launch_composite(final_grid + (size_t)r0 * pl->gw, pl->gw, r1 - r0, pl->thumbs.as<uint8_t>(), pl->tw,
                                pl->th, pl->adj.as<float4>() + (size_t)r0 * pl->gw, adjust ? 1 : 0,
                                pl->out.as<uint8_t>() + row_bytes * r0, s));
      MG_CUDA(cudaEventRecord(pl->band_ev[b], s));
      MG_CUDA(cudaStreamWaitEvent(ctx->side, pl->band_ev[b], 0));
      MG_CUDA(cudaMemcpyAsync(pl->out_host + row_bytes * r0, pl->out.as<uint8_t>() + row_bytes * r0,
                              row_bytes * (r1 - r0), cudaMemcpyDeviceToHost, ctx->side));
    }
    MG_CUDA(cudaEventRecord(pl->download_done, ctx->side));
    pl->downloaded_to = pl->out_host;
  }
  MG_CUDA(cudaEventRecord(pl->ev[7], s));
  pl->launches = (int)(g_launches - l0);
  pl->ran = true;
  return MG_OK;
}

int plan_read(mg_plan* pl, mg_result* res) {
  if (!pl->ran) return fail(MG_ERR_STATE, "plan has not run");
  mg_ctx* ctx = pl->ctx;
  cudaStream_t s = ctx->stream;
  const int N = pl->N;
  const int32_t* final_grid = pl->run_sa ? pl->final_grid.as<int32_t>() : pl->grid_greedy.as<int32_t>();
  ChainResult cr{};
  int bc = -1, resets = 0;
  if (pl->downloaded_to) MG_CUDA(cudaStreamWaitEvent(s, pl->download_done, 0));  // the bands' copies, joined back
  if (res->image && res->image != pl->downloaded_to)
    MG_CUDA(cudaMemcpyAsync(res->image, pl->out.p, 3ull * pl->tw * pl->th * N, cudaMemcpyDeviceToHost, s));
  // every small read-back into one pinned staging block, then one synchronisation:
  // [grid N x int32][resets, kernel error, context error, best chain][chain results]
  const size_t n_chains = pl->run_sa ? (size_t)std::max(pl->K, 1) : 0;
  const size_t words = ((size_t)N + 4 + 3) & ~(size_t)3;  // keeps the chain results 16-byte aligned
  const size_t need = words * 4 + sizeof(ChainResult) * n_chains;
  if (pl->h_read_cap < need) {
    if (pl->h_read) cudaFreeHost(pl->h_read);
    pl->h_read = nullptr;
    pl->h_read_cap = 0;
    MG_CUDA(cudaHostAlloc(&pl->h_read, need, cudaHostAllocDefault));
    pl->h_read_cap = need;
  }
  int32_t* h_grid = static_cast<int32_t*>(pl->h_read);
  uint32_t* h_words = reinterpret_cast<uint32_t*>(h_grid + N);
  ChainResult* h_chains = reinterpret_cast<ChainResult*>(static_cast<uint32_t*>(pl->h_read) + words);
  h_words[0] = h_words[1] = h_words[2] = 0u;
  h_words[3] = 0xFFFFFFFFu;
  MG_CUDA(cudaMemcpyAsync(h_grid, final_grid, sizeof(int32_t) * N, cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(&h_words[0], pl->resets.p, 4, cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(&h_words[1], pl->err.p, 4, cudaMemcpyDeviceToHost, s));
  if (ctx->err.p) MG_CUDA(cudaMemcpyAsync(&h_words[2], ctx->err.p, 4, cudaMemcpyDeviceToHost, s));
  if (pl->run_sa) {
    MG_CUDA(cudaMemcpyAsync(&h_words[3], pl->best_chain.p, 4, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(h_chains, pl->chain_res.p, sizeof(ChainResult) * n_chains, cudaMemcpyDeviceToHost, s));
  }
  MG_CUDA(cudaStreamSynchronize(s));
  if (h_words[2]) {
    MG_CUDA(cudaMemset(ctx->err.p, 0, 4));
    return fail(MG_ERR_TIMEOUT, "a bounded wait inside a kernel ran out");
  }
  if (h_words[1]) {
    MG_CUDA(cudaMemset(pl->err.p, 0, 4));  // reported once; the plan can run again
    return fail(MG_ERR_TIMEOUT, "a bounded wait inside a kernel ran out");
  }
  resets = (int)h_words[0];
  if (pl->run_sa) {
    bc = (int)h_words[3];
    if (bc >= 0 && bc < (int)n_chains) cr = h_chains[bc];
  }
  const int32_t* grid = h_grid;
  if (res->grid)
    for (int i = 0; i < N; ++i) res->grid[i] = grid[i] < 0 ? -1 : pl->selected[grid[i]];
  res->out_w = pl->gw * pl->tw;
  res->out_h = pl->gh * pl->th;
  res->palette_size = pl->P;
  res->n_resets = resets;
  res->best_chain = bc;
  res->initial_cost = cr.initial_cost;
  res->final_cost = cr.final_cost;
  res->best_cost = cr.best_cost;
  res->accepted_count = cr.accepted;
  res->improved_count = cr.improved;
  return MG_OK;
}

}  // namespace

extern "C" {

int mg_plan_create(mg_ctx* ctx, const mg_request* req, mg_plan** out) {
  MG_CHECK(check_ctx(ctx));
  if (!out) return fail(MG_ERR_ARG, "null out");
  *out = nullptr;
  mg_plan* pl = new mg_plan();
  int s = plan_setup(pl, ctx, req, false);
  if (s != MG_OK) {
    std::string msg = g_error;
    plan_release(pl);
    delete pl;
    set_error(msg);
    return s;
  }
  *out = pl;
  return MG_OK;
}

int mg_plan_run(mg_plan* pl) {
  if (!pl) return fail(MG_ERR_ARG, "null plan");
  MG_CHECK(check_ctx(pl->ctx));
  return plan_run(pl);
}

int mg_plan_read(mg_plan* pl, mg_result* res) {
  if (!pl || !res) return fail(MG_ERR_ARG, "null plan or result");
  MG_CHECK(check_ctx(pl->ctx));
  return plan_read(pl, res);
}

int mg_plan_destroy(mg_plan* pl) {
  if (!pl) return MG_OK;
  cudaSetDevice(pl->device);
  cudaDeviceSynchronize();
  plan_release(pl);
  delete pl;
  return MG_OK;
}

int mg_plan_stage_ms(mg_plan* pl, float* ms, int cap) {
  if (!pl || !ms) return fail(MG_ERR_ARG, "null argument");
  if (!pl->ran) return fail(MG_ERR_STATE, "plan has not run");
  MG_CHECK(check_ctx(pl->ctx));
  MG_CUDA(cudaEventSynchronize(pl->ev[7]));
  int n = 0;
  for (int i = 0; i < 7 && n < cap; ++i, ++n) MG_CUDA(cudaEventElapsedTime(&ms[n], pl->ev[i], pl->ev[i + 1]));
  if (n < cap) {
    MG_CUDA(cudaEventElapsedTime(&ms[n], pl->ev[0], pl->ev[7]));
    ++n;
  }
  return n;
}

int mg_plan_launches(mg_plan* pl) { return pl ? pl->launches : 0; }

int mg_generate(mg_ctx* ctx, const mg_request* req, mg_result* res) {
  MG_CHECK(check_ctx(ctx));
  if (!res) return fail(MG_ERR_ARG, "null result");
  if (!ctx->gen_plan) ctx->gen_plan = new mg_plan();
  mg_plan* pl = ctx->gen_plan;
  MG_CHECK(plan_setup(pl, ctx, req, true));
  // a pinned image buffer is filled band by band during the run (a pageable one
  // would make each band's copy wait on the host)
  pl->out_host = device_view(res->image) ? static_cast<uint8_t*>(res->image) : nullptr;
  int st = plan_run(pl);
  pl->out_host = nullptr;
  if (st == MG_OK) st = plan_read(pl, res);
  return st;
}

}  // extern "C"
