/*
 * mosaic_gpu.h -- C ABI of the GB300 (sm_103a) tile matching-and-placement
 * library, a drop-in for mosaic-art-rust's hot path.
 *
 * Conventions
 *   - Every entry point returns an int status (MG_OK = 0); on failure
 *     mg_last_error() gives a message for the calling thread.  Nothing aborts,
 *     traps or unwinds across this boundary.
 *   - Host buffers belong to the caller and are never freed by the library.
 *     Device buffers belong to the context (mg_ctx) or to a plan (mg_plan).
 *   - RGB8 images are interleaved, row-major, `stride` bytes between rows.
 *   - Lab colours are float triples (L, a, b).  Material identity is an int
 *     index; a grid cell holding -1 has no tile (the reference's
 *     Option<PathBuf> = None).
 *   - A context is externally synchronised: one thread at a time.  All work of
 *     a context runs on its own CUDA stream; calls with host outputs return
 *     after the results are on the host.
 *
 * Each declaration cites the reference interface it replaces
 * (path:line inside naporin0624/mosaic-art-rust).
 */
#ifndef MOSAIC_GPU_H
#define MOSAIC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MG_OK 0
#define MG_ERR_ARG 1     /* invalid argument (size, null pointer, empty grid) */
#define MG_ERR_OOM 2     /* device or pinned-host allocation failed */
#define MG_ERR_CUDA 3    /* a CUDA runtime call failed */
#define MG_ERR_TIMEOUT 4 /* a bounded wait inside a kernel ran out */
#define MG_ERR_BUDGET 5  /* request does not fit the device-memory budget */
#define MG_ERR_STATE 6   /* call not valid in the object's current state */

#define MG_SIM_FULL 0       /* P x P, symmetric, zero diagonal */
#define MG_SIM_TRIANGULAR 1 /* strict upper triangle, row order (similarity.rs:38-41) */

typedef struct mg_ctx mg_ctx;
typedef struct mg_plan mg_plan;

/* ---- library, context, memory --------------------------------------------- */
int mg_version(void);
const char* mg_last_error(void);
/* Number of kernels this library has launched in the process. */
unsigned long long mg_kernel_launches(void);
int mg_ctx_create(int device, mg_ctx** out);
int mg_ctx_destroy(mg_ctx* ctx);
int mg_ctx_sync(mg_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t), so a caller can order its own
 * device work (and timing events) with the library's. */
void* mg_ctx_stream(mg_ctx* ctx);
/* Pinned host memory (for fast host<->device copies); NULL on failure. */
void* mg_host_alloc(size_t bytes);
void mg_host_free(void* p);

/* ---- colour statistics ------------------------------------------------------ */
/* lib.rs:94-119 MosaicGenerator::calculate_average_lab: mean of per-pixel Lab. */
int mg_average_lab(mg_ctx* ctx, const uint8_t* rgb, int w, int h, int64_t stride, float lab[3]);
/* lib.rs:121-123 MosaicGenerator::is_aspect_ratio_match (returns 0 or 1). */
int mg_is_aspect_ratio_match(float img_aspect, float target_aspect, float tolerance);
/* main.rs:495-496, 537-541 (cell crop + calculate_average_lab) and main.rs:687-708
 * (calculate_average_rgb) for every cell of a gw x gh grid, cell size
 * (w/gw) x (h/gh).  lab_out: gw*gh*3 floats; avg_rgb_out (nullable): gw*gh*3. */
int mg_cells_lab(mg_ctx* ctx, const uint8_t* img, int w, int h, int64_t stride, int gw, int gh,
                 float* lab_out, uint8_t* avg_rgb_out);
/* No counterpart in the reference.  mg_cells_lab for callers that cannot
 * allocate device memory where they call it -- e.g. a serving process whose
 * device memory belongs to its own pool allocator under a fixed budget, or
 * code that must not incur the device-wide synchronisation of cudaMalloc /
 * cudaFree between other work.  Everything is caller-owned and
 * device-accessible: d_img (stride bytes per row), d_lab4 (gw*gh x 4 floats:
 * L, a, b, 0; 16-byte aligned), d_rgb4 (nullable, gw*gh x 4 bytes: R, G, B, 0).
 * Work is queued on `stream` (a cudaStream_t, NULL = default stream) and no
 * memory is allocated: a cell is reduced by one warp, or, from 8192 pixels
 * per cell, by several warps whose partial sums meet in a fixed device array
 * the library reserves on each GPU that loads it (1.5 MB), so at most 32768
 * cells per call (MG_ERR_ARG beyond).  The first call on a device resolves that
 * array's address and uploads constants (it synchronises the device), so make
 * it before any stream capture.  All calls share the array: calls whose work
 * overlaps on the GPU (other streams, other threads) race and must be ordered
 * by the caller.  Results equal mg_cells_lab's bit for bit. */
int mg_cells_lab_noalloc(const uint8_t* d_img, int w, int h, int64_t stride, int gw, int gh, float* d_lab4,
                         uint8_t* d_rgb4, void* stream);
/* How missing thumbnails are made on the device (mg_request / mg_palette_desc
 * with thumbnails NULL, and mg_resize).  MG_THUMB_LANCZOS3 (the default) is
 * main.rs:710-738 resize_image: fast_image_resize's default, a Lanczos3
 * convolution, here as the published convolution resampler it follows (taps
 * at pixel centres, support 3 x the downscale factor, weights normalised and
 * rounded to 22-bit fixed point, a horizontal then a vertical pass through an
 * 8-bit intermediate; exact integer arithmetic).  MG_THUMB_AREA: the mean of
 * each output pixel's source box, rounded.  Applies to plans, mg_generate
 * calls and palettes set up on the context afterwards. */
#define MG_THUMB_LANCZOS3 0
#define MG_THUMB_AREA 1
int mg_ctx_set_thumbnail_filter(mg_ctx* ctx, int filter);
/* main.rs:710-738 resize_image: one RGB8 image (stride bytes per row, 0 ->
 * 3*w) to dw x dh with the context's thumbnail filter; out: dh x dw x 3. */
int mg_resize(mg_ctx* ctx, const uint8_t* rgb, int w, int h, int64_t stride, int dw, int dh, uint8_t* out);
/* main.rs:193-208, 244-253 (process_tile -> calculate_average_lab for each
 * material) in one launch.  lab_out: n*3; avg_rgb_out (nullable): n*3. */
int mg_images_lab(mg_ctx* ctx, const uint8_t* const* imgs, const int* w, const int* h,
                  const int64_t* stride, int n, float* lab_out, uint8_t* avg_rgb_out);
/* main.rs:166-261 load_tiles selection (aspect filter in input order, the
 * unfiltered fallback of main.rs:215-253, truncation to max_materials).
 * Writes the chosen material indices to `selected`; returns the count (>= 0)
 * or -MG_ERR_ARG. */
int mg_select_palette(const int* widths, const int* heights, int n, float target_aspect,
                      float tolerance, int max_materials, int* selected);

/* ---- image files: the two ends of the path (host code) --------------------------- */
/* main.rs:492, 548 image::open + DynamicImage::to_rgb8 (image 0.25.6 / png
 * 0.17.16) for PNG data held in memory, and main.rs:672 DynamicImage::save
 * for a .png path.  Every PNG 1.2 colour type, bit depth and interlace is
 * read: grey is replicated to three channels, alpha dropped, palette indices
 * looked up, 1/2/4-bit grey scaled to 8 bits, 16-bit samples rounded to 8
 * bits.  Chunk CRCs and the zlib checksum are checked (MG_ERR_ARG with a
 * message on any defect).  These calls need no context or GPU and may run on
 * any thread. */
/* Width and height of the PNG file data[0..n). */
int mg_png_info(const uint8_t* data, size_t n, int* w, int* h);
/* Decodes into out: h rows of `stride` bytes (>= 3*w), e.g. pinned memory from
 * mg_host_alloc that mg_generate then reads in place.  On failure the
 * contents of out are unspecified. */
int mg_png_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride);
/* `count` files on up to `threads` host threads (<= 0: one per hardware
 * thread); status (nullable) receives each file's code; returns the first
 * failure's code (its message names the file's position). */
int mg_png_decode_batch(const uint8_t* const* data, const size_t* n, int count, uint8_t* const* out,
                        const int64_t* stride, int threads, int* status);
/* Largest file mg_png_encode writes for a w x h image (0 for invalid sizes). */
size_t mg_png_encode_bound(int w, int h);
/* Encodes an RGB8 image as an 8-bit RGB PNG: per row the filter with the
 * smallest sum of absolute residuals; level 0 stores the rows uncompressed,
 * level 1 codes each 64 KB block with its own Huffman code (or stores it when
 * that is smaller).  The blocks share no back-references and a private
 * ancillary chunk ("mgIX", ignored by other readers) indexes them, so
 * mg_png_decode inflates a large file of this library's on all threads.
 * out must hold mg_png_encode_bound(w, h) bytes (else MG_ERR_ARG with
 * *len = that bound); *len receives the file size. */
int mg_png_encode(const uint8_t* rgb, int w, int h, int64_t stride, int level, int threads, uint8_t* out,
                  size_t cap, size_t* len);

/* main.rs:172-185, 492, 548: load_tiles also takes jpg/jpeg materials, opened
 * by image::open (zune-jpeg 0.4.18).  This library's own decoder (ITU-T T.81,
 * JFIF): Huffman JPEG with 8-bit samples, sequential (baseline and extended)
 * and progressive (spectral selection, successive approximation), grey,
 * YCbCr or RGB-coded (Adobe transform 0, or 'R' 'G' 'B' components without
 * JFIF) with sampling factors 1 or 2, restart intervals; lossless,
 * hierarchical and arithmetic-coded files fail with MG_ERR_ARG.  The inverse DCT
 * is the FP32 separable form of T.81 A.3.3, chroma is upsampled by
 * replication and converted with the JFIF equations, so pixels may differ
 * from zune-jpeg's by a few levels (not pinned: that crate cannot run here).
 * Same conventions as the PNG calls: no context, any thread, RGB8 out. */
int mg_jpeg_info(const uint8_t* data, size_t n, int* w, int* h);
int mg_jpeg_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride);
/* main.rs:672 output_img.save(path) of a .jpg / .jpeg path (image's JPEG
 * encoder, quality 75).  This library's own baseline JFIF encoder: 4:2:0
 * YCbCr, the T.81 Annex K quantisation tables scaled by quality (1..100, the
 * IJG rule), Huffman codes from the image's own symbol counts, one restart
 * interval per row of 16-pixel MCUs (the rows are coded on up to `threads`
 * host threads; <= 0: all).  Bytes differ from the crate's encoder's (not
 * pinned).  w, h in 1..65535; out must hold mg_jpeg_encode_bound(w, h) bytes
 * (else MG_ERR_ARG with *len = that bound); *len receives the file size. */
size_t mg_jpeg_encode_bound(int w, int h);
int mg_jpeg_encode(const uint8_t* rgb, int w, int h, int64_t stride, int quality, int threads, uint8_t* out,
                   size_t cap, size_t* len);
/* PNG or JPEG, told apart by the file's signature (image::open's format
 * detection for the two formats read here). */
int mg_image_info(const uint8_t* data, size_t n, int* w, int* h);
int mg_image_decode(const uint8_t* data, size_t n, uint8_t* out, int64_t stride);
/* A material folder of PNG and JPEG files on up to `threads` host threads
 * (<= 0: one per hardware thread); status (nullable) receives each file's
 * code; returns the first failure's code (its message names the file). */
int mg_image_decode_batch(const uint8_t* const* data, const size_t* n, int count, uint8_t* const* out,
                          const int64_t* stride, int threads, int* status);

/* ---- similarity database --------------------------------------------------------- */
/* similarity.rs:69-82 build_similarities (+ similarity.rs:141-146
 * calculate_lab_distance) on the device.  layout MG_SIM_FULL or
 * MG_SIM_TRIANGULAR; out: p*p or p*(p-1)/2 floats. */
int mg_similarity_build(mg_ctx* ctx, const float* lab, int p, int layout, float* out);
/* similarity.rs:141-146 calculate_lab_distance. */
float mg_lab_distance(const float a[3], const float b[3]);

/* ---- k nearest (replaces kiddo nearest_n, main.rs:145-151, 348-352) ---------- */
/* For each of nq query Lab colours, the k nearest of p palette colours by
 * squared Euclidean distance, ascending, ties to the lowest index.
 * idx_out, dist_out: nq*k. */
int mg_nearest_n(mg_ctx* ctx, const float* palette_lab, int p, const float* query_lab, int nq, int k,
                 uint32_t* idx_out, float* dist_out);

/* How this context searches: MG_NEAREST_SCAN compares every query with every
 * palette colour; MG_NEAREST_GRID first sorts the palette into a bucket grid
 * over its Lab bounding box and compares each query only with the buckets
 * that can hold its k nearest; MG_NEAREST_AUTO (the default) takes the grid
 * for palettes of at least 2048 colours and 16k.  Results are identical.
 * Applies to mg_nearest_n, mg_place_greedy, mg_generate and to palettes
 * created afterwards (mg_palette_create builds the grid once). */
#define MG_NEAREST_AUTO 0
#define MG_NEAREST_SCAN 1
#define MG_NEAREST_GRID 2
int mg_ctx_set_nearest_method(mg_ctx* ctx, int method);

/* How this context scores a candidate in the greedy placement:
 * MG_SCORING_CLI (the default) as main.rs:335-418, squared Lab distance +
 * adjacency penalty; MG_SCORING_GUI as the GUI generator,
 * gui/app_full.rs:1396-1470 find_best_tile_primary, Lab distance (its square
 * root) + adjacency penalty.  Candidates, usage limits, the same-neighbour ban
 * and the fallbacks are the same in both; the GUI's fixed 100 candidates are
 * min(P, 100) like the CLI's, and its lack of colour adjustment is strength 0.
 * Applies to mg_place_greedy, and to plans, mg_generate calls, batches and
 * servers set up on the context afterwards. */
#define MG_SCORING_CLI 0
#define MG_SCORING_GUI 1
int mg_ctx_set_scoring(mg_ctx* ctx, int scoring);

/* No counterpart in the reference (which has no device waits): fault
 * injection for tests of the timeout path.  Every wait inside this library's
 * kernels is bounded; a wait that runs out makes the kernel give up, and the
 * call reports MG_ERR_TIMEOUT ("a bounded wait inside a kernel ran out")
 * instead of hanging the GPU.  After this call the next `walks` greedy walks
 * on this context in the three-CTA form (mg_place_greedy, mg_generate,
 * mg_plan_run; rows of at least 8 cells, palettes of at most 65535) run with
 * their candidate records withheld and a short wait limit, so the walker's
 * wait for its first record runs out within about a millisecond: the call
 * returns MG_ERR_TIMEOUT, the walk's grid is left empty (-1), and the context
 * and its plans stay usable.  0 cancels. */
int mg_ctx_inject_walk_timeout(mg_ctx* ctx, int walks);

/* ---- adjacency ------------------------------------------------------------------ */
/* adjacency.rs:63-88 calculate_penalty for n (candidate, x, y) triples
 * (cxy: n*3 ints) against one grid; out: n floats (weighted). */
int mg_penalty_batch(mg_ctx* ctx, const float* palette_lab, int p, const int32_t* grid, int gw, int gh,
                     float weight, const int32_t* cxy, int n, float* out);
/* adjacency.rs:91-130 calculate_total_cost (unweighted). */
int mg_total_cost(mg_ctx* ctx, const float* palette_lab, int p, const int32_t* grid, int gw, int gh,
                  float* out);
/* adjacency.rs:133-214 calculate_swap_delta for n position pairs
 * (pairs: n*4 ints x1, y1, x2, y2); out: n floats. */
int mg_swap_delta_batch(mg_ctx* ctx, const float* palette_lab, int p, const int32_t* grid, int gw, int gh,
                        const int32_t* pairs, int n, float* out);

/* ---- greedy placement (main.rs:335-475 over the grid, main.rs:529-545) ------------ */
typedef struct mg_place_config {
  int max_usage_per_image;        /* main.rs:53-55, UsageTracker cap */
  float adjacency_penalty_weight; /* main.rs:57-59; <= 0 disables the penalty */
} mg_place_config;
/* Row-major greedy placement from per-cell Lab colours.  grid_out: gw*gh
 * palette indices (-1 only when p == 0).  n_resets (nullable): how many
 * cells fell back to the global usage reset of main.rs:428. */
int mg_place_greedy(mg_ctx* ctx, const float* palette_lab, int p, const float* cell_lab, int gw, int gh,
                    const mg_place_config* cfg, int32_t* grid_out, int* n_resets);

/* ---- annealing (optimizer.rs) ------------------------------------------------------ */
typedef struct mg_sa_config {      /* optimizer.rs:7-27 OptimizationConfig + chains */
  int64_t max_iterations;          /* default 1000 */
  float initial_temperature;       /* default 100.0 */
  float temperature_decay;         /* default 0.99995 */
  int chains;                      /* independent chains, >= 1 */
  uint64_t seed;                   /* Philox key */
  uint32_t stream;                 /* Philox stream id (e.g. request id) */
  int greedy_only;                 /* 1 = optimizer.rs:132-198 optimize_greedy */
} mg_sa_config;
typedef struct mg_sa_result {      /* optimizer.rs:203-221 OptimizationResult */
  float initial_cost, final_cost, best_cost;
  int64_t improved_count, accepted_count, iterations;
  int best_chain;
} mg_sa_result;
void mg_sa_config_default(mg_sa_config* cfg);
/* optimizer.rs:41-129 MosaicOptimizer::optimize, run as cfg->chains chains
 * from the same start grid.  On return `grid` holds the final grid of the
 * chain with the lowest final cost (ties: lowest chain).  per_chain
 * (nullable): chains results; chain_grids (nullable): chains*gw*gh. */
int mg_optimize(mg_ctx* ctx, const float* palette_lab, int p, int32_t* grid, int gw, int gh,
                const mg_sa_config* cfg, mg_sa_result* best, mg_sa_result* per_chain, int32_t* chain_grids);
/* optimizer.rs:205-220 OptimizationResult::improvement_percentage. */
float mg_improvement_percentage(const mg_sa_result* r);

/* ---- colour adjustment (color_adjustment.rs) ---------------------------------------- */
typedef struct mg_color_adjustment { /* color_adjustment.rs:6-15 */
  float brightness, contrast, hue_shift, saturation;
} mg_color_adjustment;
/* color_adjustment.rs:30-37 ColorAdjustment::new (clamps). */
mg_color_adjustment mg_color_adjustment_new(float brightness, float contrast, float hue_shift,
                                            float saturation);
/* color_adjustment.rs:99-154 calculate_optimal_adjustment for n (tile, target)
 * mean-RGB pairs (each n*3 bytes); out: n adjustments. */
int mg_optimal_adjustment_batch(mg_ctx* ctx, const uint8_t* tile_rgb, const uint8_t* target_rgb, int n,
                                float strength, mg_color_adjustment* out);
/* color_adjustment.rs:40-51 apply_to_image (adjust_pixel of every pixel). */
int mg_apply_adjustment(mg_ctx* ctx, const mg_color_adjustment* adj, const uint8_t* rgb, int w, int h,
                        int64_t stride, uint8_t* out);
/* main.rs:548-592 / 627-664: composite p thumbnails (p x th x tw x 3) into the
 * (gw*tw) x (gh*th) output by grid (palette indices), colour-adjusting each
 * cell when strength > 0 (cell_avg_rgb: gw*gh*3 target means). */
int mg_composite(mg_ctx* ctx, const int32_t* grid, int gw, int gh, const uint8_t* thumbs, int p, int tw, int th,
                 const uint8_t* cell_avg_rgb, float strength, uint8_t* out);

/* ---- the whole generate_mosaic job (main.rs:105-164 new + main.rs:477-685) ------------ */
typedef struct mg_request {
  const uint8_t* target;          /* target RGB8 image */
  int target_w, target_h;
  int64_t target_stride;          /* 0 -> 3*target_w */
  int n_materials;
  const uint8_t* const* materials; /* n_materials RGB8 images (decoded tiles) */
  const int* material_w;
  const int* material_h;
  const int64_t* material_stride;  /* nullable -> 3*w */
  const uint8_t* thumbnails;       /* nullable: n_materials x tile_h x tile_w x 3, the resized tiles
                                      (main.rs:549); NULL -> resized on the device with the
                                      context's thumbnail filter (Lanczos3 by default) */
  int tile_w, tile_h;              /* output tile size; 0 -> cell size (main.rs:495-496) */
  int grid_w, grid_h;              /* main.rs:37-43 */
  int max_materials;               /* main.rs:45-47 */
  float aspect_tolerance;          /* main.rs:49-51 */
  int max_usage_per_image;         /* main.rs:53-55 */
  float adjacency_penalty_weight;  /* main.rs:57-59 */
  float color_adjustment_strength; /* main.rs:77-79, clamped to [0,1] (main.rs:162) */
  int enable_optimization;         /* main.rs:61-63 */
  int64_t optimization_iterations; /* main.rs:65-67 */
  float initial_temperature;       /* optimizer.rs:21 */
  float temperature_decay;         /* optimizer.rs:22 */
  int chains;                      /* annealing chains (>= 1) */
  uint64_t seed;
  uint32_t stream;
  int build_similarity;            /* 1: build the P x P similarity DB (main.rs:120-143) */
} mg_request;

typedef struct mg_result {
  int32_t* grid;          /* nullable, grid_w*grid_h: ORIGINAL material index or -1 */
  uint8_t* image;         /* nullable, out_h x out_w x 3 */
  int out_w, out_h;       /* set by the call */
  int palette_size;       /* tiles kept by load_tiles */
  int n_resets;           /* cells that used the global usage reset */
  int best_chain;         /* -1 when the optimiser did not run */
  float initial_cost, final_cost, best_cost;
  int64_t accepted_count, improved_count;
} mg_result;

void mg_request_default(mg_request* req);
/* One complete job from host buffers to host buffers.  Inputs in pinned host
 * memory (mg_host_alloc) are read in place over the CPU-GPU link.  A grid holds
 * at most 2^28 cells and an output row at most 2^31 / 3 pixels (MG_ERR_ARG
 * beyond; a batch's cells together obey the same cell limit). */
int mg_generate(mg_ctx* ctx, const mg_request* req, mg_result* res);

/* Device-resident form of the same job: mg_plan_create uploads the inputs
 * (palette selection, target, selected materials, thumbnails) into device
 * memory; mg_plan_run runs the whole device pipeline on them (no host copies);
 * mg_plan_read copies results to the host. */
int mg_plan_create(mg_ctx* ctx, const mg_request* req, mg_plan** out);
int mg_plan_run(mg_plan* plan);
int mg_plan_read(mg_plan* plan, mg_result* res);
int mg_plan_destroy(mg_plan* plan);
/* Device time of each stage of the last mg_plan_run, in ms (CUDA events):
 * [0] material Lab, [1] similarity, [2] cell Lab, [3] nearest, [4] greedy,
 * [5] anneal, [6] composite, [7] total.  Cell Lab runs on a second stream
 * beside [0] and [1]; [2] is the part of it that outlasts them.  Returns the
 * count written. */
int mg_plan_stage_ms(mg_plan* plan, float* ms, int cap);
/* Number of kernels one mg_plan_run launches. */
int mg_plan_launches(mg_plan* plan);

/* ---- resident palettes and batches of mosaics ---------------------------------------
 * No single reference function: the reference builds its palette once per
 * process (MosaicGenerator::new, main.rs:105-164) and then generates one
 * mosaic (main.rs:477-685).  Here the palette stays in device memory and many
 * mosaics of uneven size run through one batched pipeline: the data-parallel
 * stages over the cells of every mosaic at once, every greedy walk in one
 * launch and every annealing chain in one launch; results equal mg_generate's
 * for each mosaic bit for bit. */
typedef struct mg_palette mg_palette;
typedef struct mg_batch mg_batch;

typedef struct mg_palette_desc {
  int n_materials;
  const uint8_t* const* materials;
  const int* material_w;
  const int* material_h;
  const int64_t* material_stride;  /* nullable -> 3*w */
  const uint8_t* thumbnails;       /* nullable: n x tile_h x tile_w x 3; NULL -> the context's thumbnail filter */
  int tile_w, tile_h;              /* output tile size of every mosaic using the palette (> 0) */
  float target_aspect;             /* load_tiles selection (main.rs:166-261) for this target aspect */
  float aspect_tolerance;
  int max_materials;
  int build_similarity;            /* 1: keep the P x P similarity database resident */
} mg_palette_desc;

typedef struct mg_mosaic {         /* one request: a target and the generate_mosaic settings */
  const uint8_t* target;           /* host (pinned or pageable) or device memory */
  int target_w, target_h;
  int64_t target_stride;           /* 0 -> 3*target_w */
  int grid_w, grid_h;
  int max_usage_per_image;
  float adjacency_penalty_weight;
  float color_adjustment_strength;
  int enable_optimization;
  int64_t optimization_iterations;
  float initial_temperature, temperature_decay;
  int chains;
  uint64_t seed;
  uint32_t stream;
} mg_mosaic;

void mg_palette_desc_default(mg_palette_desc* desc);
int mg_palette_create(mg_ctx* ctx, const mg_palette_desc* desc, mg_palette** out);
int mg_palette_size(const mg_palette* pal);
int64_t mg_palette_device_bytes(const mg_palette* pal);
/* similarity.rs:105-109 get_lab_color for every tile: P x 3 floats. */
int mg_palette_read_lab(mg_palette* pal, float* lab_out);
/* The resident similarity database (similarity.rs:69-103), P x P floats. */
int mg_palette_read_similarity(mg_palette* pal, float* out);
int mg_palette_destroy(mg_palette* pal);

void mg_mosaic_default(mg_mosaic* m);
/* A batch with its inputs copied to device memory; the first mg_batch_run
 * autotunes launch shapes, later runs replay one CUDA graph. */
int mg_batch_create(mg_ctx* ctx, mg_palette* pal, const mg_mosaic* mosaics, int n, mg_batch** out);
int mg_batch_run(mg_batch* batch);
/* Mosaic i's grid (original material indices), image (grid_h*tile_h x
 * grid_w*tile_w x 3) and annealing summary. */
int mg_batch_read(mg_batch* batch, int i, mg_result* res);
/* [0] cell statistics, [1] k-nearest, [2] walks + chains, [3] adjust +
 * composite, [4] total; ms of the last run. */
int mg_batch_stage_ms(mg_batch* batch, float* ms, int cap);
/* The launch shapes the autotuner picked: cells per CTA of the cell
 * statistics, and the palette chunk of the k-nearest scan (0: the palette's
 * bucket grid serves the search, which has no chunk size).  Chains are not a
 * tuned shape: each annealing chain is one 4-warp CTA and an SM runs as many
 * chain CTAs as fit, so putting several chains in one CTA would serialise them. */
int mg_batch_tuning(mg_batch* batch, int* cells_per_cta, int* nearest_chunk);
int mg_batch_launches(mg_batch* batch);
int mg_batch_destroy(mg_batch* batch);
/* One batch from host buffers to host buffers (targets in pinned host memory
 * are read in place).  The context keeps the batch's device buffers for its
 * next call (they only grow; mg_ctx_destroy releases them). */
int mg_generate_batch(mg_ctx* ctx, mg_palette* pal, const mg_mosaic* mosaics, int n, mg_result* results);

/* ---- serving: a request loop over one resident palette ------------------------------
 * No counterpart in the reference.  Requests submitted from any thread wait in
 * a FIFO queue; a dispatcher admits them, within the device-memory budget, into
 * the next free slot (a stream with reusable batch buffers) as one batch, so
 * requests that arrive while others run are folded into the next batch and
 * batches overlap on the device; a completion thread copies each request's
 * grid and image into the caller's buffers.  A request's results do not depend
 * on which requests share its batch.  Buffers passed to mg_server_submit (the
 * target and the outputs) must stay valid until the request completes. */
typedef struct mg_server mg_server;
typedef struct mg_server_config {
  int slots;                   /* batches in flight (streams), default 3 */
  int max_batch;               /* requests per batch, default 64 */
  int64_t memory_budget_bytes; /* device memory the admitted requests may use, default 120 GB */
} mg_server_config;
typedef struct mg_server_stats {
  int64_t submitted, completed, rejected, batches, pending, bytes_in_use, peak_bytes_in_use;
} mg_server_stats;
void mg_server_config_default(mg_server_config* cfg);
int mg_server_create(mg_ctx* ctx, mg_palette* pal, const mg_server_config* cfg, mg_server** out);
/* grid_out: grid_w*grid_h ints; image_out: (grid_h*tile_h) x (grid_w*tile_w) x 3 (both nullable). */
int mg_server_submit(mg_server* srv, const mg_mosaic* m, int32_t* grid_out, uint8_t* image_out, uint64_t* ticket);
/* Status of a finished request (MG_OK, or MG_ERR_BUDGET when it can never fit
 * the budget), or -1 while it is still pending.  latency_ms: submission to
 * results on the host. */
int mg_server_poll(mg_server* srv, uint64_t ticket, mg_result* res, double* latency_ms);
int mg_server_wait(mg_server* srv, uint64_t ticket, mg_result* res, double* latency_ms);
int mg_server_get_stats(mg_server* srv, mg_server_stats* stats);
/* Device bytes the request would hold while admitted (what admission counts
 * against the budget); -1 on a null argument. */
int64_t mg_server_request_bytes(mg_server* srv, const mg_mosaic* m);
/* Finishes queued and in-flight requests, then stops. */
int mg_server_destroy(mg_server* srv);

#ifdef __cplusplus
}
#endif
#endif
