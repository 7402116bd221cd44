// mg_internal.h -- shared declarations of the CUDA library behind mosaic_gpu.h.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

#include "../../include/mosaic_gpu.h"
#include "mg_math.h"

namespace mg {

// ---- errors -----------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define MG_CUDA(call)                                        \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return ::mg::cuda_fail(_e, #call); \
  } while (0)

#define MG_CHECK(status)           \
  do {                             \
    int _s = (status);             \
    if (_s != MG_OK) return _s;    \
  } while (0)

// ---- device buffers ------------------------------------------------------------
// A grow-only device allocation, reused across calls on one context.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes);
  void release();
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Error word written by kernels whose waits are bounded (a wait that runs out
// sets it and the kernel returns); read back by the host after a launch.
enum KernelError : uint32_t { kErrNone = 0, kErrTimeout = 1, kErrRange = 2 };

// Region of an RGB8 image: byte offset of its first pixel, size, row stride.
struct Region {
  int64_t offset;
  int32_t w, h;
  int64_t stride;
};

// Per-region sums from the Lab reduction: fixed-point L, a, b and u64 R, G, B.
struct RegionSums {
  long long lab[3];
  unsigned long long rgb[3];
};

// Grid geometry for cell regions of a target image.
struct CellGeom {
  int gw, gh, cw, ch;
  int64_t stride;
};

// ---- kernels (launchers; all asynchronous on `stream`) -----------------------
// (a) Lab + mean RGB of regions.  Cells of a target (geom != nullptr) or an
// explicit region list.  out_lab: float4 (L, a, b, 0); out_rgb: uchar4.
int launch_region_stats(const uint8_t* base, const CellGeom* geom, const Region* regions, int n_regions,
                        int64_t max_region_px, float4* out_lab, uchar4* out_rgb, RegionSums* scratch,
                        int want_lab, cudaStream_t stream);
cudaError_t upload_lab_consts(cudaStream_t stream);

// Copy n items of `bytes` each from device-readable addresses src[i] to
// dst + i*bytes (16-byte vector copies when aligned).
int launch_gather(const int64_t* src, int n, size_t bytes, uint8_t* dst, cudaStream_t stream);

// Lanczos3 thumbnails of regions at tw x th (k_resize.cu): ResizePlan::build
// makes the weight tables of the regions' sizes on the host and uploads them
// (once per palette or plan); launch_resize runs the two passes.
struct ResizeImage {
  int64_t offset, stride;
  int32_t w, h;
  int32_t htab, vtab;  // table offsets; -1: the dimension keeps its size
};
struct ResizePlan {
  DevBuf tabs, images, inter;
  int n = 0, tw = 0, th = 0, max_h = 0;
  int build(const Region* regions, int n_images, int tw, int th, cudaStream_t s);
  void release();
};
int launch_resize(const uint8_t* base, const ResizePlan& rp, uint8_t* out, cudaStream_t stream);

// Area-average thumbnails of regions at tw x th.
int launch_thumbnails(const uint8_t* base, const Region* regions, int n, int tw, int th, uint8_t* out,
                      cudaStream_t stream);

// (b) k nearest palette entries for every query (ties -> lowest index).
// chunk: palette entries per shared-memory stage (1024, 2048 or 4096).
// index: a grid built over `pal` (LabIndex::build); when it has buckets the
// grid search runs instead of the scan.
struct LabIndex;
int launch_nearest(const float4* pal, int p, const float4* queries, int nq, int k, uint32_t* idx,
                   float* dist, uint32_t* err, cudaStream_t stream, int chunk = 2048,
                   const LabIndex* index = nullptr);
// v[i] = sqrt(v[i]) for i < n (the GUI generator's colour term over candidate distances).
int launch_sqrt_inplace(float* v, size_t n, cudaStream_t stream);

// (b) the same search through a bucket grid over the palette's Lab colours
// (k_nearest_grid.cu): identical results, far fewer distances for P >> k.
enum NearestMethod { kNearestAuto = 0, kNearestScan = 1, kNearestGrid = 2 };
struct LabGrid {
  float lo[3], inv[3];  // bucket of v on axis c: floor((v - lo[c]) * inv[c]), clamped to [0, g)
  int g, p;
};
struct LabIndex {
  DevBuf hdr, sorted, start;  // LabGrid; P float4 (L, a, b, index bits) by bucket; g^3 + 1 ints
  int g = 0;                  // buckets per axis; 0: no index (the scan runs)
  int build(const float4* pal, int p, int method, int k, cudaStream_t s);
  void release();
};
// Buckets per axis the method picks for a palette of p entries (0: scan).
int lab_grid_dim(int method, int p, int k);
int launch_nearest_grid(const LabIndex& index, const float4* queries, int nq, int keff, int k, uint32_t* idx,
                        float* dist, cudaStream_t stream);

// (c) similarity matrix, full (P x P) or strict upper triangle.
int launch_similarity(const float4* pal, int p, int triangular, float* out, cudaStream_t stream);

// (d) greedy placement of one or more mosaics.
struct GreedyJob {
  const uint32_t* cand_idx;  // N x k
  const float* cand_dist;    // N x k
  int32_t* grid;             // N (palette index)
  int gw, gh, k;
  uint32_t max_usage;
  float weight;
  int* n_resets;             // 1 int
  float* total_cost;         // 1 float: calculate_total_cost of the placed grid
};
// Candidate arrays must hold ceil(N/16)*16 rows (the walk streams 16 rows per copy).
// one_warp: every job walks in the one-warp form (else the three-CTA form when
// every job allows it).  inject_timeout (three-CTA form only): the scouts
// withhold their records and the walker waits at most a few thousand polls,
// so its bounded wait runs out -- an injected fault for tests.  A walk that
// gives up sets kErrTimeout in *err and leaves every cell of its grid empty.
int launch_greedy(const float4* pal, int p, const GreedyJob* jobs_dev, int n_jobs, int k, int max_gw,
                  int max_cells, uint32_t* usage_scratch, uint32_t* err, cudaStream_t stream, bool one_warp = false,
                  bool inject_timeout = false);
inline size_t padded_cells(int n) { return ((size_t)n + 15) / 16 * 16; }
// Most cells of one mosaic, or of all the mosaics of one batch (indices stay 32-bit).
constexpr int64_t kMaxGridCells = int64_t(1) << 28;
// Whether a mosaic of gw x (n / gw) cells over a palette of p walks in the
// three-CTA form (else one warp).
bool greedy_scouted_fits(int gw, int n, int p);

// (e) annealing chains.
struct ChainResult {
  float initial_cost, final_cost, best_cost, pad;
  long long accepted, improved, cooled, pad2;
};
struct AnnealJob {
  const int32_t* grid_in;   // N
  int32_t* chain_grids;     // chains x N
  ChainResult* results;     // chains
  const float* initial_cost;  // 1 float (calculate_total_cost of grid_in); nullptr -> computed
  int gw, gh, chains;
  long long iters;
  float t0, decay;
  uint32_t key0, key1, stream;
  int greedy_only;
};
// min_cells: the smallest grid among the chains (< 0: max_cells), which picks
// the round size.
int launch_anneal(const float4* pal, int p, const AnnealJob* jobs_dev, const int* chain_job_dev,
                  const int* chain_id_dev, int total_chains, int max_cells, cudaStream_t stream, int min_cells = -1);
// Per job: the chain with the lowest final cost (ties: the lowest chain) into
// its final grid; a job with no chains copies grid_in and records -1.
int launch_select_best(const AnnealJob* jobs_dev, int n_jobs, int32_t* const* final_grids_dev,
                       int* best_chain_dev, cudaStream_t stream);
int launch_total_cost(const float4* pal, const int32_t* grid, int gw, int gh, float* out, cudaStream_t stream);
int launch_swap_delta(const float4* pal, const int32_t* grid, int gw, int gh, const int4* pairs, int n, float* out,
                      cudaStream_t stream);
int launch_penalty(const float4* pal, const int32_t* grid, int gw, int gh, float weight, const int4* cxy, int n,
                   float* out, cudaStream_t stream);

// ---- batches of mosaics over one resident palette (k_batch.cu) --------------
struct BatchMosaic {
  const uint8_t* target;  // device-readable RGB8
  int64_t stride;
  int gw, gh, cw, ch, n, cell_base;  // cell_base: first of the mosaic's cells in the flat cell arrays (multiple of 16)
  uint32_t max_usage;
  float weight, strength;
  int run_sa, chains;
  long long iters;
  float t0, decay;
  uint32_t key0, key1, stream;
  int32_t* grid;          // greedy grid (n)
  int32_t* chain_grids;   // chains x n
  ChainResult* results;   // chains
  int32_t* final_grid;    // n
  int* n_resets;
  float* init_cost;
  int* best_chain;
  uint8_t* out;           // (gh*th) x (gw*tw) x 3
};
const LabConsts& host_lab_consts();
int launch_batch_cells(const BatchMosaic* mos, int nm, int total_cells, const LabConsts* consts, float4* lab,
                       uchar4* rgb, int warps, cudaStream_t stream);
int launch_batch_finish(const BatchMosaic* mos, int nm, int total_cells, const uchar4* thumb_rgb,
                        const uchar4* cell_rgb, float4* adj, const uint8_t* thumbs, int tw, int th, cudaStream_t stream);

// (f) colour adjustment + composite.
int launch_cell_adjust(const int32_t* grid, int n_cells, const uchar4* thumb_rgb, const uchar4* cell_rgb,
                       float strength, float4* adj, cudaStream_t stream);
int launch_composite(const int32_t* grid, int gw, int gh, const uint8_t* thumbs, int tw, int th, const float4* adj,
                     int do_adjust, uint8_t* out, cudaStream_t stream);
int launch_adjust_image(const float4 adj, const uint8_t* in, int w, int h, int64_t stride, uint8_t* out,
                        cudaStream_t stream);
int launch_optimal_adjustment(const uint8_t* tile_rgb, const uint8_t* target_rgb, int n, float strength,
                              float4* out, cudaStream_t stream);

// Number of kernel launches issued by this library since load (for reporting).
extern std::atomic<unsigned long long> g_launches;

}  // namespace mg
