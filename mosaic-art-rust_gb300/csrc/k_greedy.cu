// k_greedy.cu -- (d) the standalone greedy placement kernel: one warp per
// mosaic; the walk itself is greedy_walk.cuh.
#include "greedy_walk.cuh"

namespace mg {
namespace {
using namespace greedy_detail;

template <bool kLabSmem, bool kUsageSmem>
__global__ void __launch_bounds__(32) greedy_kernel(const float4* __restrict__ pal, int p,
                                                    const GreedyJob* __restrict__ jobs, uint32_t* usage_global,
                                                    uint32_t* err) {
  extern __shared__ __align__(128) uint8_t smem[];
  const GreedyJob J = jobs[blockIdx.x];
  greedy_walk<kLabSmem, kUsageSmem>(pal, p, J, smem, usage_global ? usage_global + (size_t)blockIdx.x * p : nullptr,
                                    err);
}

}  // namespace

size_t greedy_shared_bytes(int k, int gw, int p, bool lab_smem, bool usage_smem) {
  return greedy_smem_bytes(k, gw, p, lab_smem, usage_smem);
}

int launch_greedy(const float4* pal, int p, const GreedyJob* jobs_dev, int n_jobs, int k, int max_gw,
                  uint32_t* usage_scratch, uint32_t* err, cudaStream_t stream) {
  if (n_jobs <= 0) return MG_OK;
  if (k < 1 || k > 100) return fail(MG_ERR_ARG, "candidate count must be in 1..100");
  constexpr size_t kMaxSmem = 220 * 1024;
  bool lab_smem = true, usage_smem = true;
  size_t bytes = greedy_smem_bytes(k, max_gw, p, lab_smem, usage_smem);
  if (bytes > kMaxSmem) {
    lab_smem = false;
    bytes = greedy_smem_bytes(k, max_gw, p, lab_smem, usage_smem);
  }
  if (bytes > kMaxSmem) {
    usage_smem = false;
    bytes = greedy_smem_bytes(k, max_gw, p, lab_smem, usage_smem);
  }
  if (bytes > kMaxSmem) return fail(MG_ERR_ARG, "grid row too wide for the greedy walk");
  if (!usage_smem && !usage_scratch) return fail(MG_ERR_ARG, "usage scratch required for this palette size");
  static int configured_device = -1;
  int dev = 0;
  MG_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    MG_CUDA(cudaFuncSetAttribute(greedy_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxSmem));
    configured_device = dev;
  }
  if (lab_smem)
    greedy_kernel<true, true><<<n_jobs, 32, bytes, stream>>>(pal, p, jobs_dev, usage_scratch, err);
  else if (usage_smem)
    greedy_kernel<false, true><<<n_jobs, 32, bytes, stream>>>(pal, p, jobs_dev, usage_scratch, err);
  else
    greedy_kernel<false, false><<<n_jobs, 32, bytes, stream>>>(pal, p, jobs_dev, usage_scratch, err);
  g_launches += 1;
  MG_CUDA(cudaGetLastError());
  return MG_OK;
}

}  // namespace mg
