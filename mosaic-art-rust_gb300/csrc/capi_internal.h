// capi_internal.h -- the context object and host helpers shared by the C ABI
// translation units (capi.cu, capi_batch.cu).
#pragma once
#include <vector>

#include "mg_internal.h"

namespace mg {
constexpr int kGenGroups = 4;  // streams of a large mg_generate_batch
}  // namespace mg

struct mg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // forked from `stream` for stages that can overlap, joined back
  mg::DevBuf in0, in1, in2, out0, out1, out2, sums, regions, err, lab_consts;
  mg_plan* gen_plan = nullptr;
  int nearest_method = mg::kNearestAuto;  // MG_NEAREST_*
  int scoring = 0;                        // MG_SCORING_*
  int inject_walk_timeouts = 0;           // mg_ctx_inject_walk_timeout: walks left to fail on purpose
  int thumb_filter = 0;                   // MG_THUMB_*: how missing thumbnails are made
  mg::ResizePlan resize;                  // mg_resize's tables
  mg::LabIndex nn_index;                  // grid of the last single-call palette
  mg_batch* gen_batch = nullptr;          // mg_generate_batch's buffers, kept for the next call
  // mg_generate_batch's groups of a large batch: a context (stream) and buffers each
  mg_ctx* gen_sub[mg::kGenGroups] = {};
  mg_batch* gen_sub_batch[mg::kGenGroups] = {};
  cudaStream_t gen_up = nullptr, gen_down = nullptr;  // their target uploads, their image downloads
};

namespace mg {
int check_ctx(mg_ctx* ctx);
void batch_free(mg_batch* b);  // synchronises the device, releases the batch's buffers, deletes it
std::vector<float4> to_f4(const float* lab3, int n);
int upload(mg_ctx* ctx, DevBuf& b, const void* src, size_t bytes);
int finish(mg_ctx* ctx);
int ensure_err(mg_ctx* ctx);
// Device address of caller memory that kernels may read in place: pinned,
// mapped host memory (reached over the CPU-GPU link).  nullptr otherwise.
const void* device_view(const void* p);
// Like device_view, and also device memory itself.
const void* device_view_or_device(const void* p);
bool valid_image(const void* p, int w, int h, int64_t stride);
// Device copy of the Lab conversion constants (for kernels outside k_lab.cu).
const LabConsts* device_lab_consts(mg_ctx* ctx);
}  // namespace mg
