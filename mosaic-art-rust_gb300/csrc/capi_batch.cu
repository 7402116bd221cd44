// capi_batch.cu -- resident palettes and batches of mosaics (mosaic_gpu.h:
// mg_palette_*, mg_batch_*, mg_generate_batch).
//
// A palette is what the reference's MosaicGenerator::new builds
// (main.rs:105-164): the load_tiles selection for one target aspect, the
// materials' mean Lab, the similarity database, plus the thumbnails and their
// mean RGB; here it stays in device memory and serves any number of mosaics.
// A batch runs many mosaics over one palette through the batched pipeline of
// k_batch.cu; after its first run the batch's launches are captured in a CUDA
// graph and replayed.  The first run also autotunes two launch shapes by
// timing each candidate on the batch itself: cells per CTA of the cell
// statistics (4 or 8) and the palette chunk of the k-nearest scan (1024, 2048
// or 4096 entries per shared-memory stage; none when the palette's bucket grid
// serves the search).
#include <algorithm>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace mg;

struct mg_palette {
  mg_ctx* ctx = nullptr;
  int device = 0;  // destroy must not touch ctx, which may already be gone
  int P = 0, tw = 0, th = 0, k = 0;
  std::vector<int> selected;
  std::vector<Region> h_regions;
  DevBuf mats, regions, thumbs, thumb_regions, pal_lab, thumb_rgb, sim, sums;
  LabIndex index;  // bucket grid over pal_lab for the k-nearest search (when large)
  ResizePlan resize;  // Lanczos3 tables when the thumbnails are made on the device
  bool has_sim = false;
  size_t device_bytes = 0;
};

struct mg_batch {
  mg_ctx* ctx = nullptr;
  int device = 0;  // destroy must not touch ctx, which may already be gone
  mg_palette* pal = nullptr;
  int n = 0, total_cells = 0, max_gw = 0, max_cells = 0, max_sa_cells = 0, min_sa_cells = 0;
  int total_chains = 0;
  std::vector<BatchMosaic> h_mos;
  std::vector<int> cells, out_w, out_h, chains;
  std::vector<size_t> out_off;
  int grid_total = 0;
  DevBuf targets, mos, cell_lab, cell_rgb, cand_idx, cand_dist, grids, finals, chain_grids, results, resets,
      init_cost, best, adj, out, err, gjobs, usage, ajobs, chain_job, chain_id, finals_ptr;
  // walk jobs (gjobs): the n_wide mosaics that walk in the three-CTA form first, then the rest
  int n_wide = 0, wide_gw = 0, wide_cells = 0, narrow_gw = 0, narrow_cells = 0;
  // tuned launch shapes
  int cells_warps = 8, nn_chunk = 2048;
  int scoring = 0;  // MG_SCORING_* of the context when the batch was set up
  bool tuned = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t ev[5] = {};
  // mg_generate_batch groups: targets uploaded on another stream (up_done), images
  // downloaded on another stream after the run (run_done)
  cudaEvent_t up_done = nullptr, run_done = nullptr;
  bool ran = false;
  bool capturing = false;
  int launches = 0;
};

namespace {

int palette_setup(mg_palette* pl, mg_ctx* ctx, const mg_palette_desc* d) {
  if (!d) return fail(MG_ERR_ARG, "null palette description");
  if (d->n_materials < 0 || (d->n_materials > 0 && (!d->materials || !d->material_w || !d->material_h)))
    return fail(MG_ERR_ARG, "invalid material list");
  if (d->tile_w <= 0 || d->tile_h <= 0) return fail(MG_ERR_ARG, "a palette needs a positive tile size");
  if (d->max_materials < 0) return fail(MG_ERR_ARG, "negative max_materials");
  pl->ctx = ctx;
  pl->device = ctx->device;
  pl->tw = d->tile_w;
  pl->th = d->tile_h;
  pl->selected.assign(std::max(d->n_materials, 1), 0);
  const int P = mg_select_palette(d->material_w, d->material_h, d->n_materials, d->target_aspect,
                                  d->aspect_tolerance, d->max_materials, pl->selected.data());
  if (P < 0) return fail(MG_ERR_ARG, "invalid material sizes");
  if (P >= 65535) return fail(MG_ERR_ARG, "palette too large (max 65534 materials)");
  pl->selected.resize(P);
  pl->P = P;
  pl->k = std::min(P, 100);
  cudaStream_t s = ctx->stream;
  pl->h_regions.resize(std::max(P, 1));
  int64_t off = 0;
  for (int i = 0; i < P; ++i) {
    const int m = pl->selected[i];
    const int64_t st = d->material_stride ? d->material_stride[m] : 3ll * d->material_w[m];
    if (!valid_image(d->materials[m], d->material_w[m], d->material_h[m], st))
      return fail(MG_ERR_ARG, "invalid material " + std::to_string(m));
    pl->h_regions[i] = Region{off, d->material_w[m], d->material_h[m], 3ll * d->material_w[m]};
    off += 3ll * d->material_w[m] * d->material_h[m];
    off = (off + 15) & ~15ll;
  }
  MG_CHECK(pl->mats.ensure((size_t)std::max<int64_t>(off, 16)));
  for (int i = 0; i < P; ++i) {
    const int m = pl->selected[i];
    const int64_t st = d->material_stride ? d->material_stride[m] : 3ll * d->material_w[m];
    MG_CUDA(cudaMemcpy2DAsync(pl->mats.as<uint8_t>() + pl->h_regions[i].offset, 3ull * d->material_w[m],
                              d->materials[m], st, 3ull * d->material_w[m], d->material_h[m], cudaMemcpyHostToDevice, s));
  }
  MG_CHECK(upload(ctx, pl->regions, pl->h_regions.data(), sizeof(Region) * std::max(P, 1)));
  const size_t tb = 3ull * pl->tw * pl->th;
  MG_CHECK(pl->thumbs.ensure(tb * std::max(P, 1)));
  std::vector<Region> tregs(std::max(P, 1));
  for (int i = 0; i < P; ++i) tregs[i] = Region{(int64_t)(tb * i), pl->tw, pl->th, 3ll * pl->tw};
  MG_CHECK(upload(ctx, pl->thumb_regions, tregs.data(), sizeof(Region) * std::max(P, 1)));
  if (d->thumbnails) {
    for (int i = 0; i < P; ++i)
      MG_CUDA(cudaMemcpyAsync(pl->thumbs.as<uint8_t>() + tb * i, d->thumbnails + tb * pl->selected[i], tb,
                              cudaMemcpyHostToDevice, s));
  } else if (P > 0 && ctx->thumb_filter == MG_THUMB_LANCZOS3) {
    MG_CHECK(pl->resize.build(pl->h_regions.data(), P, pl->tw, pl->th, s));
    MG_CHECK(launch_resize(pl->mats.as<uint8_t>(), pl->resize, pl->thumbs.as<uint8_t>(), s));
  } else if (P > 0) {
    MG_CHECK(launch_thumbnails(pl->mats.as<uint8_t>(), pl->regions.as<Region>(), P, pl->tw, pl->th,
                               pl->thumbs.as<uint8_t>(), s));
  }
  MG_CHECK(pl->pal_lab.ensure(sizeof(float4) * std::max(P, 1)));
  MG_CHECK(pl->thumb_rgb.ensure(sizeof(uchar4) * std::max(P, 1)));
  MG_CHECK(pl->sums.ensure(sizeof(RegionSums) * std::max(P, 1)));
  if (P > 0) {
    int64_t maxpx = 0;
    for (int i = 0; i < P; ++i) maxpx = std::max<int64_t>(maxpx, (int64_t)pl->h_regions[i].w * pl->h_regions[i].h);
    MG_CHECK(launch_region_stats(pl->mats.as<uint8_t>(), nullptr, pl->regions.as<Region>(), P, maxpx,
                                 pl->pal_lab.as<float4>(), nullptr, pl->sums.as<RegionSums>(), 1, s));
    MG_CHECK(launch_region_stats(pl->thumbs.as<uint8_t>(), nullptr, pl->thumb_regions.as<Region>(), P,
                                 (int64_t)pl->tw * pl->th, nullptr, pl->thumb_rgb.as<uchar4>(),
                                 pl->sums.as<RegionSums>(), 0, s));
    if (d->build_similarity) {
      MG_CHECK(pl->sim.ensure(sizeof(float) * (size_t)P * P));
      MG_CHECK(launch_similarity(pl->pal_lab.as<float4>(), P, 0, pl->sim.as<float>(), s));
      pl->has_sim = true;
    }
    MG_CHECK(pl->index.build(pl->pal_lab.as<float4>(), P, ctx->nearest_method, std::min(P, 100), s));
  }
  MG_CHECK(finish(ctx));
  pl->device_bytes = pl->mats.cap + pl->thumbs.cap + pl->pal_lab.cap + pl->thumb_rgb.cap + pl->sim.cap +
                     pl->index.hdr.cap + pl->index.sorted.cap + pl->index.start.cap;
  return MG_OK;
}

void release(std::initializer_list<DevBuf*> bufs) {
  for (DevBuf* b : bufs) b->release();
}

void batch_release(mg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t* e : {&b->up_done, &b->run_done}) {
    if (*e) cudaEventDestroy(*e);
    *e = nullptr;
  }
  release({&b->targets, &b->mos, &b->cell_lab, &b->cell_rgb, &b->cand_idx, &b->cand_dist, &b->grids, &b->finals,
           &b->chain_grids, &b->results, &b->resets, &b->init_cost, &b->best, &b->adj, &b->out, &b->err,
           &b->gjobs, &b->usage, &b->ajobs, &b->chain_job, &b->chain_id, &b->finals_ptr});
}

// wait: return after the uploads have completed (else they may still be in
// flight, ahead of anything enqueued on the context's stream next).
// copy_stream: the stream that copies the targets (nullptr: the context's);
// the context's stream waits for them.
int batch_setup(mg_batch* b, mg_ctx* ctx, mg_palette* pal, const mg_mosaic* ms, int n, bool zero_copy,
                bool wait = true, cudaStream_t copy_stream = nullptr) {
  if (!pal || (n > 0 && !ms) || n < 0) return fail(MG_ERR_ARG, "invalid batch");
  b->ctx = ctx;
  b->device = ctx->device;
  b->scoring = ctx->scoring;
  b->pal = pal;
  b->n = n;
  const int tw = pal->tw, th = pal->th, k = std::max(pal->k, 1);
  cudaStream_t s = ctx->stream;
  b->h_mos.assign(std::max(n, 1), BatchMosaic{});
  b->cells.assign(n, 0);
  b->out_w.assign(n, 0);
  b->out_h.assign(n, 0);
  b->chains.assign(n, 0);
  b->out_off.assign(n, 0);
  std::vector<int64_t> tgt_off(n, -1);
  int64_t tgt_bytes = 0;
  size_t out_bytes = 0, chain_cells = 0, n_results = 0;
  int cell_base = 0, grid_base = 0;
  b->total_chains = 0;
  b->max_gw = b->max_cells = b->max_sa_cells = b->min_sa_cells = 0;
  for (int i = 0; i < n; ++i) {
    const mg_mosaic& r = ms[i];
    const int64_t st = r.target_stride ? r.target_stride : 3ll * r.target_w;
    if (!valid_image(r.target, r.target_w, r.target_h, st)) return fail(MG_ERR_ARG, "invalid target " + std::to_string(i));
    if (r.grid_w <= 0 || r.grid_h <= 0 || r.target_w / r.grid_w <= 0 || r.target_h / r.grid_h <= 0)
      return fail(MG_ERR_ARG, "invalid grid of mosaic " + std::to_string(i));
    if (r.max_usage_per_image < 0) return fail(MG_ERR_ARG, "negative max usage");
    // cell indices (over the whole batch) and output rows are 32-bit on the device
    if ((int64_t)r.grid_w * r.grid_h > kMaxGridCells || (int64_t)r.grid_w * tw > INT32_MAX / 3 ||
        (int64_t)r.grid_h * th > INT32_MAX || (int64_t)cell_base + (int64_t)r.grid_w * r.grid_h + 16 > kMaxGridCells)
      return fail(MG_ERR_ARG, "grid or output image too large in mosaic " + std::to_string(i));
    const int N = r.grid_w * r.grid_h;
    const bool run_sa = r.enable_optimization && r.adjacency_penalty_weight > 0.0f && pal->P > 0;  // main.rs:608
    if (run_sa && (r.chains < 1 || r.chains > 65535 || r.optimization_iterations < 0))
      return fail(MG_ERR_ARG, "need 1 <= chains <= 65535 and iterations >= 0");
    BatchMosaic& M = b->h_mos[i];
    M.stride = st;
    M.gw = r.grid_w;
    M.gh = r.grid_h;
    M.cw = r.target_w / r.grid_w;
    M.ch = r.target_h / r.grid_h;
    M.n = N;
    M.cell_base = cell_base;
    M.max_usage = (uint32_t)r.max_usage_per_image;
    M.weight = r.adjacency_penalty_weight;
    M.strength = rclamp(r.color_adjustment_strength, 0.0f, 1.0f);  // main.rs:162
    M.run_sa = run_sa ? 1 : 0;
    M.chains = run_sa ? r.chains : 0;
    M.iters = r.optimization_iterations;
    M.t0 = r.initial_temperature;
    M.decay = r.temperature_decay;
    M.key0 = (uint32_t)r.seed;
    M.key1 = (uint32_t)(r.seed >> 32);
    M.stream = r.stream;
    const void* dv = zero_copy ? device_view_or_device(r.target) : nullptr;
    if (dv) {
      M.target = static_cast<const uint8_t*>(dv);
    } else {
      tgt_off[i] = tgt_bytes;
      tgt_bytes += (3ll * r.target_w * r.target_h + 15) & ~15ll;
      M.stride = 3ll * r.target_w;
    }
    b->cells[i] = N;
    b->chains[i] = M.chains;
    b->out_w[i] = r.grid_w * tw;
    b->out_h[i] = r.grid_h * th;
    b->out_off[i] = out_bytes;
    out_bytes += ((size_t)b->out_w[i] * b->out_h[i] * 3 + 15) & ~(size_t)15;
    chain_cells += (size_t)M.chains * N;
    n_results += M.chains;
    cell_base += (int)padded_cells(N);
    grid_base += N;
    b->total_chains += M.chains;
    b->max_gw = std::max(b->max_gw, r.grid_w);
    b->max_cells = std::max(b->max_cells, N);
    if (run_sa) {
      b->min_sa_cells = b->max_sa_cells == 0 ? N : std::min(b->min_sa_cells, N);
      b->max_sa_cells = std::max(b->max_sa_cells, N);
    }
    if (run_sa && (size_t)N * 2 > 180 * 1024) return fail(MG_ERR_ARG, "mosaic too large for the annealer");
  }
  b->total_cells = cell_base;
  b->grid_total = grid_base;
  // device buffers
  if (tgt_bytes > 0) MG_CHECK(b->targets.ensure((size_t)tgt_bytes));
  MG_CHECK(b->cell_lab.ensure(sizeof(float4) * std::max(cell_base, 1)));
  MG_CHECK(b->cell_rgb.ensure(sizeof(uchar4) * std::max(cell_base, 1)));
  MG_CHECK(b->cand_idx.ensure(sizeof(uint32_t) * (size_t)std::max(cell_base, 16) * k));
  MG_CHECK(b->cand_dist.ensure(sizeof(float) * (size_t)std::max(cell_base, 16) * k));
  MG_CHECK(b->grids.ensure(sizeof(int32_t) * std::max(grid_base, 1)));
  MG_CHECK(b->finals.ensure(sizeof(int32_t) * std::max(grid_base, 1)));
  MG_CHECK(b->chain_grids.ensure(sizeof(int32_t) * std::max<size_t>(chain_cells, 1)));
  MG_CHECK(b->results.ensure(sizeof(ChainResult) * std::max<size_t>(n_results, 1)));
  MG_CHECK(b->resets.ensure(sizeof(int) * std::max(n, 1)));
  MG_CHECK(b->init_cost.ensure(sizeof(float) * std::max(n, 1)));
  MG_CHECK(b->best.ensure(sizeof(int) * std::max(n, 1)));
  MG_CHECK(b->adj.ensure(sizeof(float4) * std::max(cell_base, 1)));
  MG_CHECK(b->out.ensure(std::max<size_t>(out_bytes, 16)));
  MG_CHECK(b->err.ensure(16));
  MG_CUDA(cudaMemsetAsync(b->err.p, 0, 16, s));
  for (int i = 0; i < n; ++i)
    if (tgt_off[i] >= 0) b->h_mos[i].target = b->targets.as<uint8_t>() + tgt_off[i];
  // per-mosaic device pointers
  size_t gpos = 0, cpos = 0, rpos = 0;
  for (int i = 0; i < n; ++i) {
    BatchMosaic& M = b->h_mos[i];
    M.grid = b->grids.as<int32_t>() + gpos;
    M.final_grid = b->finals.as<int32_t>() + gpos;
    M.chain_grids = b->chain_grids.as<int32_t>() + cpos;
    M.results = b->results.as<ChainResult>() + rpos;
    M.n_resets = b->resets.as<int>() + i;
    M.init_cost = b->init_cost.as<float>() + i;
    M.best_chain = b->best.as<int>() + i;
    M.out = b->out.as<uint8_t>() + b->out_off[i];
    gpos += M.n;
    cpos += (size_t)M.chains * M.n;
    rpos += M.chains;
  }
  MG_CHECK(upload(ctx, b->mos, b->h_mos.data(), sizeof(BatchMosaic) * std::max(n, 1)));
  // largest mosaic first: walks, then chains
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return b->cells[a] > b->cells[c]; });
  // walk jobs: those that walk in the three-CTA form first (one launch), the
  // rest (narrow grids, grids too large for its shared memory) one warp each
  std::vector<GreedyJob> jobs;
  jobs.reserve(std::max(n, 1));
  b->n_wide = b->wide_gw = b->wide_cells = b->narrow_gw = b->narrow_cells = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i : order) {
      const BatchMosaic& M = b->h_mos[i];
      if (greedy_scouted_fits(M.gw, M.n, pal->P) != (pass == 0)) continue;
      jobs.push_back(GreedyJob{b->cand_idx.as<uint32_t>() + (size_t)M.cell_base * k,
                               b->cand_dist.as<float>() + (size_t)M.cell_base * k, M.grid, M.gw, M.gh, k, M.max_usage,
                               M.weight, M.n_resets, M.init_cost});
      if (pass == 0) {
        ++b->n_wide;
        b->wide_gw = std::max(b->wide_gw, M.gw);
        b->wide_cells = std::max(b->wide_cells, M.n);
      } else {
        b->narrow_gw = std::max(b->narrow_gw, M.gw);
        b->narrow_cells = std::max(b->narrow_cells, M.n);
      }
    }
  }
  MG_CHECK(upload(ctx, b->gjobs, jobs.data(), sizeof(GreedyJob) * std::max<size_t>(jobs.size(), 1)));
  // counters in global memory for the one-warp walk when a palette's do not fit in shared memory
  if (pal->P > 32768) MG_CHECK(b->usage.ensure(sizeof(uint32_t) * (size_t)n * pal->P));
  // chain jobs (one per mosaic, in mosaic order: the selection writes best_chain[i]),
  // the chains largest mosaic first, and the final-grid pointers
  std::vector<AnnealJob> ajobs(std::max(n, 1));
  std::vector<int32_t*> finals(std::max(n, 1), nullptr);
  std::vector<int> cjob, cid;
  cjob.reserve(std::max(b->total_chains, 1));
  cid.reserve(std::max(b->total_chains, 1));
  for (int i = 0; i < n; ++i) {
    const BatchMosaic& M = b->h_mos[i];
    AnnealJob& A = ajobs[i];
    A = AnnealJob{};
    A.grid_in = M.grid;
    A.chain_grids = M.chain_grids;
    A.results = M.results;
    A.initial_cost = M.init_cost;
    A.gw = M.gw;
    A.gh = M.gh;
    A.chains = M.chains;
    A.iters = M.iters;
    A.t0 = M.t0;
    A.decay = M.decay;
    A.key0 = M.key0;
    A.key1 = M.key1;
    A.stream = M.stream;
    A.greedy_only = 0;
    finals[i] = M.final_grid;
  }
  for (int i : order)
    for (int c = 0; c < b->h_mos[i].chains; ++c) {
      cjob.push_back(i);
      cid.push_back(c);
    }
  cjob.resize(std::max<size_t>(cjob.size(), 1));
  cid.resize(std::max<size_t>(cid.size(), 1));
  MG_CHECK(upload(ctx, b->ajobs, ajobs.data(), sizeof(AnnealJob) * ajobs.size()));
  MG_CHECK(upload(ctx, b->finals_ptr, finals.data(), sizeof(int32_t*) * finals.size()));
  MG_CHECK(upload(ctx, b->chain_job, cjob.data(), sizeof(int) * cjob.size()));
  MG_CHECK(upload(ctx, b->chain_id, cid.data(), sizeof(int) * cid.size()));
  for (auto& e : b->ev)
    if (!e) MG_CUDA(cudaEventCreate(&e));
  // targets that are not read in place, copied last: a copy from pageable host
  // memory (the uploads above) may wait for the stream's earlier work
  const cudaStream_t cs = copy_stream ? copy_stream : s;
  for (int i = 0; i < n; ++i) {
    if (tgt_off[i] < 0) continue;
    const mg_mosaic& r = ms[i];
    const int64_t st = r.target_stride ? r.target_stride : 3ll * r.target_w;
    MG_CUDA(cudaMemcpy2DAsync(b->targets.as<uint8_t>() + tgt_off[i], 3ull * r.target_w, r.target, st,
                              3ull * r.target_w, r.target_h, cudaMemcpyDefault, cs));
  }
  if (cs != s) {
    if (!b->up_done) MG_CUDA(cudaEventCreateWithFlags(&b->up_done, cudaEventDisableTiming));
    MG_CUDA(cudaEventRecord(b->up_done, cs));
    MG_CUDA(cudaStreamWaitEvent(s, b->up_done, 0));
  }
  if (wait) MG_CUDA(cudaStreamSynchronize(s));
  b->ran = false;
  return MG_OK;
}

// A timing event: during graph capture it must be an external record node to
// be recorded when the graph runs.
cudaError_t record(mg_batch* b, cudaEvent_t e, cudaStream_t s) {
  return b->capturing ? cudaEventRecordWithFlags(e, s, cudaEventRecordExternal) : cudaEventRecord(e, s);
}

// Enqueue one run of the batch (no synchronisation).
int batch_enqueue(mg_batch* b, bool with_events) {
  mg_ctx* ctx = b->ctx;
  mg_palette* pal = b->pal;
  cudaStream_t s = ctx->stream;
  const int n = b->n, P = pal->P, k = std::max(pal->k, 1);
  if (n == 0) return MG_OK;
  const unsigned long long l0 = g_launches;
  if (with_events) MG_CUDA(record(b, b->ev[0], s));
  MG_CHECK(launch_batch_cells(b->mos.as<BatchMosaic>(), n, b->total_cells, device_lab_consts(ctx),
                              b->cell_lab.as<float4>(), b->cell_rgb.as<uchar4>(), b->cells_warps, s));
  if (with_events) MG_CUDA(record(b, b->ev[1], s));
  if (P > 0)
    MG_CHECK(launch_nearest(pal->pal_lab.as<float4>(), P, b->cell_lab.as<float4>(), b->total_cells, k,
                            b->cand_idx.as<uint32_t>(), b->cand_dist.as<float>(), b->err.as<uint32_t>(), s, b->nn_chunk,
                            &pal->index));
  if (P > 0 && b->scoring == MG_SCORING_GUI)
    MG_CHECK(launch_sqrt_inplace(b->cand_dist.as<float>(), (size_t)b->total_cells * k, s));
  if (with_events) MG_CUDA(record(b, b->ev[2], s));
  if (P > 0) {
    // every greedy walk: rows of >= 8 cells by the scouted walk, the rest one
    // warp each (k_greedy.cu), largest mosaic first
    uint32_t* usage = b->usage.cap ? b->usage.as<uint32_t>() : nullptr;
    if (b->n_wide > 0)
      MG_CHECK(launch_greedy(pal->pal_lab.as<float4>(), P, b->gjobs.as<GreedyJob>(), b->n_wide, k, b->wide_gw,
                             b->wide_cells, usage, b->err.as<uint32_t>(), s));
    if (b->n - b->n_wide > 0)
      MG_CHECK(launch_greedy(pal->pal_lab.as<float4>(), P, b->gjobs.as<GreedyJob>() + b->n_wide, b->n - b->n_wide, k,
                             b->narrow_gw, b->narrow_cells, usage ? usage + (size_t)b->n_wide * P : nullptr,
                             b->err.as<uint32_t>(), s, true));
    // every annealing chain of every mosaic (k_anneal.cu), then per mosaic the
    // best chain -- or the greedy grid when it is not optimised -- as its final grid
    MG_CHECK(launch_anneal(pal->pal_lab.as<float4>(), P, b->ajobs.as<AnnealJob>(), b->chain_job.as<int>(),
                           b->chain_id.as<int>(), b->total_chains, b->max_sa_cells, s, b->min_sa_cells));
    MG_CHECK(launch_select_best(b->ajobs.as<AnnealJob>(), n, b->finals_ptr.as<int32_t*>(), b->best.as<int>(), s));
  } else {
    MG_CUDA(cudaMemsetAsync(b->finals.p, 0xFF, b->finals.cap, s));
  }
  if (with_events) MG_CUDA(record(b, b->ev[3], s));
  MG_CHECK(launch_batch_finish(b->mos.as<BatchMosaic>(), n, b->total_cells, pal->thumb_rgb.as<uchar4>(),
                               b->cell_rgb.as<uchar4>(), b->adj.as<float4>(), pal->thumbs.as<uint8_t>(), pal->tw,
                               pal->th, s));
  if (with_events) MG_CUDA(record(b, b->ev[4], s));
  b->launches = (int)(g_launches - l0);
  return MG_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t c) {
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, c);
  return ms;
}

// Time each candidate launch shape on the batch itself; keep the fastest.
int batch_tune(mg_batch* b) {
  cudaStream_t s = b->ctx->stream;
  float best = 1e30f;
  int best_cw = 8;
  for (int cw : {4, 8}) {
    b->cells_warps = cw;
    for (int rep = 0; rep < 2; ++rep) MG_CHECK(batch_enqueue(b, true));
    MG_CUDA(cudaStreamSynchronize(s));
    const float t = elapsed(b->ev[0], b->ev[1]);
    if (t < best) {
      best = t;
      best_cw = cw;
    }
  }
  b->cells_warps = best_cw;
  best = 1e30f;
  int best_nn = 2048;
  for (int ch : {1024, 2048, 4096}) {
    if (b->pal->index.g > 0) break;  // the grid search has no chunk size
    b->nn_chunk = ch;
    MG_CHECK(batch_enqueue(b, true));
    MG_CUDA(cudaStreamSynchronize(s));
    const float t = elapsed(b->ev[1], b->ev[2]);
    if (t < best) {
      best = t;
      best_nn = ch;
    }
  }
  b->nn_chunk = best_nn;
  b->tuned = true;
  return MG_OK;
}

int batch_check(mg_batch* b) {
  uint32_t e = 0;
  MG_CUDA(cudaMemcpy(&e, b->err.p, 4, cudaMemcpyDeviceToHost));
  if (e) return fail(MG_ERR_TIMEOUT, "a bounded wait inside a batch kernel ran out");
  return MG_OK;
}

int batch_run(mg_batch* b) {
  cudaStream_t s = b->ctx->stream;
  if (!b->tuned) {
    MG_CHECK(batch_tune(b));
    MG_CHECK(batch_enqueue(b, true));
    MG_CUDA(cudaStreamSynchronize(s));
    MG_CHECK(batch_check(b));
  } else if (!b->exec) {
    // Capture the launch sequence once; later runs replay it.
    MG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    b->capturing = true;
    int st = batch_enqueue(b, true);
    b->capturing = false;
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (st != MG_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    b->graph = g;
    MG_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    MG_CUDA(cudaGraphLaunch(b->exec, s));
  } else {
    MG_CUDA(cudaGraphLaunch(b->exec, s));
  }
  b->ran = true;
  return MG_OK;
}

// Mosaic i's result from its final grid (palette indices), reset count, best
// chain and chain summaries, read back.
void fill_result(const mg_batch* b, int i, const int32_t* grid, int resets, int best, const ChainResult* chains,
                 int n_chains, mg_result* res) {
  const BatchMosaic& M = b->h_mos[i];
  ChainResult cr{};
  if (M.run_sa && best >= 0 && best < n_chains) cr = chains[best];
  if (res->grid)
    for (int c = 0; c < M.n; ++c) res->grid[c] = grid[c] < 0 ? -1 : b->pal->selected[grid[c]];
  res->out_w = b->out_w[i];
  res->out_h = b->out_h[i];
  res->palette_size = b->pal->P;
  res->n_resets = b->pal->P > 0 ? resets : 0;
  res->best_chain = M.run_sa ? best : -1;
  res->initial_cost = cr.initial_cost;
  res->final_cost = cr.final_cost;
  res->best_cost = cr.best_cost;
  res->accepted_count = cr.accepted;
  res->improved_count = cr.improved;
}

int batch_read(mg_batch* b, int i, mg_result* res) {
  if (!b->ran) return fail(MG_ERR_STATE, "batch has not run");
  if (i < 0 || i >= b->n) return fail(MG_ERR_ARG, "mosaic index out of range");
  mg_ctx* ctx = b->ctx;
  cudaStream_t s = ctx->stream;
  const BatchMosaic& M = b->h_mos[i];
  std::vector<int32_t> grid(M.n);
  int best = -1, resets = 0;
  // every chain's summary comes back with the grid, so one synchronisation serves the read
  std::vector<ChainResult> chains(M.run_sa && M.chains > 0 ? M.chains : 0);
  if (res->image)
    MG_CUDA(cudaMemcpyAsync(res->image, M.out, (size_t)b->out_w[i] * b->out_h[i] * 3, cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(grid.data(), M.final_grid, sizeof(int32_t) * M.n, cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(&resets, M.n_resets, sizeof(int), cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(&best, M.best_chain, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (!chains.empty())
    MG_CUDA(cudaMemcpyAsync(chains.data(), M.results, sizeof(ChainResult) * chains.size(), cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaStreamSynchronize(s));
  MG_CHECK(batch_check(b));
  fill_result(b, i, grid.data(), resets, best, chains.data(), (int)chains.size(), res);
  return MG_OK;
}

// Every mosaic's image into its result buffer (asynchronous when the buffer
// is pinned host memory), on `stream` after the run (nullptr: the context's).
int batch_copy_images(mg_batch* b, mg_result* res, cudaStream_t stream = nullptr) {
  cudaStream_t s = b->ctx->stream;
  if (stream && stream != s) {
    if (!b->run_done) MG_CUDA(cudaEventCreateWithFlags(&b->run_done, cudaEventDisableTiming));
    MG_CUDA(cudaEventRecord(b->run_done, s));
    MG_CUDA(cudaStreamWaitEvent(stream, b->run_done, 0));
    s = stream;
  }
  for (int i = 0; i < b->n; ++i)
    if (res[i].image)
      MG_CUDA(cudaMemcpyAsync(res[i].image, b->h_mos[i].out, (size_t)b->out_w[i] * b->out_h[i] * 3,
                              cudaMemcpyDeviceToHost, s));
  return MG_OK;
}

// Every mosaic's other results: all final grids, reset counts, best chains and
// chain summaries in one copy each (they are contiguous on the device), and
// one synchronisation.
int batch_read_rest(mg_batch* b, mg_result* res) {
  if (!b->ran) return fail(MG_ERR_STATE, "batch has not run");
  const int n = b->n;
  if (n == 0) return MG_OK;
  cudaStream_t s = b->ctx->stream;
  std::vector<int32_t> grids(std::max(b->grid_total, 1));
  std::vector<int> resets(n), best(n);
  std::vector<ChainResult> chains(std::max(b->total_chains, 1));
  MG_CUDA(cudaMemcpyAsync(grids.data(), b->finals.p, sizeof(int32_t) * b->grid_total, cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(resets.data(), b->resets.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaMemcpyAsync(best.data(), b->best.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  if (b->total_chains > 0)
    MG_CUDA(cudaMemcpyAsync(chains.data(), b->results.p, sizeof(ChainResult) * b->total_chains,
                            cudaMemcpyDeviceToHost, s));
  MG_CUDA(cudaStreamSynchronize(s));
  MG_CHECK(batch_check(b));
  size_t gpos = 0, rpos = 0;
  for (int i = 0; i < n; ++i) {
    const BatchMosaic& M = b->h_mos[i];
    fill_result(b, i, grids.data() + gpos, resets[i], best[i], chains.data() + rpos, M.chains, res + i);
    gpos += M.n;
    rpos += M.chains;
  }
  return MG_OK;
}

// mg_generate_batch of at least kGroupCells cells runs its mosaics as up to
// kGenGroups groups (contiguous runs of about equal cells), each a batch on a
// stream of its own: the groups' targets are copied in one after another on
// one stream and their images out one after another on another, so a group's
// kernels start once its own targets are in, its images leave as soon as it
// is done, and the groups' kernels overlap one another.  (Compositing straight into pinned caller buffers over
// the CPU-GPU link measured slower than compositing in device memory and
// copying.)
constexpr int64_t kGroupCells = 16384;

int generate_grouped(mg_ctx* ctx, mg_palette* pal, const mg_mosaic* ms, int n, mg_result* res, int groups) {
  std::vector<int> lo(groups + 1, n);
  int64_t total = 0;
  for (int i = 0; i < n; ++i) total += (int64_t)ms[i].grid_w * ms[i].grid_h;
  lo[0] = 0;
  int64_t acc = 0;
  for (int i = 0, g = 1; i < n && g < groups; ++i) {
    acc += (int64_t)ms[i].grid_w * ms[i].grid_h;
    if (acc * groups >= total * g) lo[g++] = i + 1;
  }
  for (int g = 1; g <= groups; ++g) lo[g] = std::max(lo[g], lo[g - 1]);
  int st = MG_OK;
  for (int g = 0; g < groups && st == MG_OK; ++g) {
    if (!ctx->gen_sub[g]) st = mg_ctx_create(ctx->device, &ctx->gen_sub[g]);
    if (st == MG_OK && !ctx->gen_sub_batch[g]) ctx->gen_sub_batch[g] = new mg_batch();
  }
  for (cudaStream_t* cs : {&ctx->gen_up, &ctx->gen_down})
    if (st == MG_OK && !*cs && cudaStreamCreateWithFlags(cs, cudaStreamNonBlocking) != cudaSuccess)
      st = cuda_fail(cudaGetLastError(), "cudaStreamCreateWithFlags");
  for (int g = 0; g < groups && st == MG_OK; ++g) {
    mg_ctx* sc = ctx->gen_sub[g];
    sc->scoring = ctx->scoring;
    mg_batch* b = ctx->gen_sub_batch[g];
    b->ran = false;
    st = batch_setup(b, sc, pal, ms + lo[g], lo[g + 1] - lo[g], false, false, ctx->gen_up);
    if (st == MG_OK) {
      b->tuned = true;
      st = batch_enqueue(b, false);
      b->ran = st == MG_OK;
    }
    if (st == MG_OK) st = batch_copy_images(b, res + lo[g], ctx->gen_down);
  }
  for (int g = 0; g < groups; ++g) {
    if (!ctx->gen_sub[g]) continue;
    if (st == MG_OK) st = batch_read_rest(ctx->gen_sub_batch[g], res + lo[g]);
    cudaStreamSynchronize(ctx->gen_sub[g]->stream);
  }
  for (cudaStream_t cs : {ctx->gen_up, ctx->gen_down})
    if (cs && cudaStreamSynchronize(cs) != cudaSuccess && st == MG_OK)
      st = cuda_fail(cudaGetLastError(), "cudaStreamSynchronize");
  return st;
}

}  // namespace

extern "C" {

void mg_palette_desc_default(mg_palette_desc* d) {
  if (!d) return;
  std::memset(d, 0, sizeof(*d));
  d->target_aspect = 4.0f / 3.0f;
  d->aspect_tolerance = 0.1f;
  d->max_materials = 500;
  d->build_similarity = 1;
}

int mg_palette_create(mg_ctx* ctx, const mg_palette_desc* desc, mg_palette** out) {
  MG_CHECK(check_ctx(ctx));
  if (!out) return fail(MG_ERR_ARG, "null out");
  *out = nullptr;
  mg_palette* p = new mg_palette();
  int st = palette_setup(p, ctx, desc);
  if (st != MG_OK) {
    mg_palette_destroy(p);
    return st;
  }
  *out = p;
  return MG_OK;
}

int mg_palette_size(const mg_palette* pal) { return pal ? pal->P : -MG_ERR_ARG; }

int64_t mg_palette_device_bytes(const mg_palette* pal) { return pal ? (int64_t)pal->device_bytes : -MG_ERR_ARG; }

int mg_palette_read_lab(mg_palette* pal, float* lab_out) {
  if (!pal || !lab_out) return fail(MG_ERR_ARG, "null argument");
  MG_CHECK(check_ctx(pal->ctx));
  std::vector<float4> v(std::max(pal->P, 1));
  MG_CUDA(cudaMemcpy(v.data(), pal->pal_lab.p, sizeof(float4) * pal->P, cudaMemcpyDeviceToHost));
  for (int i = 0; i < pal->P; ++i) {
    lab_out[3 * i] = v[i].x;
    lab_out[3 * i + 1] = v[i].y;
    lab_out[3 * i + 2] = v[i].z;
  }
  return MG_OK;
}

int mg_palette_read_similarity(mg_palette* pal, float* out) {
  if (!pal || !out) return fail(MG_ERR_ARG, "null argument");
  if (!pal->has_sim) return fail(MG_ERR_STATE, "palette built without the similarity database");
  MG_CHECK(check_ctx(pal->ctx));
  MG_CUDA(cudaMemcpy(out, pal->sim.p, sizeof(float) * (size_t)pal->P * pal->P, cudaMemcpyDeviceToHost));
  return MG_OK;
}

int mg_palette_destroy(mg_palette* pal) {
  if (!pal) return MG_OK;
  cudaSetDevice(pal->device);
  cudaDeviceSynchronize();
  release({&pal->mats, &pal->regions, &pal->thumbs, &pal->thumb_regions, &pal->pal_lab, &pal->thumb_rgb, &pal->sim,
           &pal->sums});
  pal->index.release();
  pal->resize.release();
  delete pal;
  return MG_OK;
}

void mg_mosaic_default(mg_mosaic* m) {
  if (!m) return;
  std::memset(m, 0, sizeof(*m));
  m->grid_w = 50;
  m->grid_h = 28;
  m->max_usage_per_image = 3;
  m->adjacency_penalty_weight = 0.3f;
  m->color_adjustment_strength = 0.3f;
  m->enable_optimization = 1;
  m->optimization_iterations = 1000;
  m->initial_temperature = 100.0f;
  m->temperature_decay = 0.99995f;
  m->chains = 1;
  m->seed = 0x5eed5eed5eedull;
}

int mg_batch_create(mg_ctx* ctx, mg_palette* pal, const mg_mosaic* mosaics, int n, mg_batch** out) {
  MG_CHECK(check_ctx(ctx));
  if (!out) return fail(MG_ERR_ARG, "null out");
  *out = nullptr;
  mg_batch* b = new mg_batch();
  int st = batch_setup(b, ctx, pal, mosaics, n, false);
  if (st != MG_OK) {
    std::string msg = mg_last_error();
    batch_release(b);
    delete b;
    fail(st, msg);
    return st;
  }
  *out = b;
  return MG_OK;
}

int mg_batch_run(mg_batch* b) {
  if (!b) return fail(MG_ERR_ARG, "null batch");
  MG_CHECK(check_ctx(b->ctx));
  return batch_run(b);
}

int mg_batch_read(mg_batch* b, int i, mg_result* res) {
  if (!b || !res) return fail(MG_ERR_ARG, "null argument");
  MG_CHECK(check_ctx(b->ctx));
  return batch_read(b, i, res);
}

int mg_batch_stage_ms(mg_batch* b, float* ms, int cap) {
  if (!b || !ms) return fail(MG_ERR_ARG, "null argument");
  if (!b->ran) return fail(MG_ERR_STATE, "batch has not run");
  MG_CUDA(cudaEventSynchronize(b->ev[4]));
  int nout = 0;
  for (int i = 0; i < 4 && nout < cap; ++i) ms[nout++] = elapsed(b->ev[i], b->ev[i + 1]);
  if (nout < cap) ms[nout++] = elapsed(b->ev[0], b->ev[4]);
  return nout;
}

int mg_batch_tuning(mg_batch* b, int* cells_per_cta, int* nearest_chunk) {
  if (!b) return fail(MG_ERR_ARG, "null batch");
  if (cells_per_cta) *cells_per_cta = b->cells_warps;
  if (nearest_chunk) *nearest_chunk = b->pal->index.g > 0 ? 0 : b->nn_chunk;
  return b->tuned ? MG_OK : fail(MG_ERR_STATE, "batch has not run");
}

int mg_batch_launches(mg_batch* b) { return b ? b->launches : 0; }

int mg_batch_destroy(mg_batch* b) {
  if (!b) return MG_OK;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  batch_release(b);
  delete b;
  return MG_OK;
}

int mg_generate_batch(mg_ctx* ctx, mg_palette* pal, const mg_mosaic* mosaics, int n, mg_result* results) {
  MG_CHECK(check_ctx(ctx));
  if (n > 0 && !results) return fail(MG_ERR_ARG, "null results");
  if (!pal || (n > 0 && !mosaics) || n < 0) return fail(MG_ERR_ARG, "invalid batch");
  int64_t cells = 0;
  for (int i = 0; i < n; ++i) cells += (int64_t)std::max(mosaics[i].grid_w, 0) * std::max(mosaics[i].grid_h, 0);
  if (cells >= kGroupCells && n >= 2) return generate_grouped(ctx, pal, mosaics, n, results, std::min(n, kGenGroups));
  // the context keeps the batch (its device buffers only grow) for the next call
  if (!ctx->gen_batch) ctx->gen_batch = new mg_batch();
  mg_batch* b = ctx->gen_batch;
  b->ran = false;
  int st = batch_setup(b, ctx, pal, mosaics, n, true);
  if (st == MG_OK) {
    b->tuned = true;  // one-shot: default shapes, no tuning runs
    st = batch_enqueue(b, true);
    b->ran = st == MG_OK;
  }
  if (st == MG_OK) st = batch_copy_images(b, results);
  if (st == MG_OK) st = batch_read_rest(b, results);
  cudaStreamSynchronize(ctx->stream);
  return st;
}

}  // extern "C"

// ---- hooks for the request loop (capi_server.cu) ----------------------------------
namespace mg {

mg_batch* server_batch_new() { return new mg_batch(); }

void batch_free(mg_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  batch_release(b);
  delete b;
}

// Reuses the batch's device buffers (they only grow); inputs in pinned host or
// device memory are read in place; default launch shapes, no graph.
int server_batch_setup(mg_batch* b, mg_ctx* ctx, mg_palette* pal, const mg_mosaic* ms, int n) {
  MG_CHECK(check_ctx(ctx));
  MG_CHECK(batch_setup(b, ctx, pal, ms, n, true));
  b->tuned = true;
  return MG_OK;
}

int server_batch_enqueue(mg_batch* b) {
  MG_CHECK(batch_enqueue(b, false));
  b->ran = true;
  return MG_OK;
}

// Request i's results, read as soon as they are on the host (its latency ends there).
int server_batch_read(mg_batch* b, int i, mg_result* res) { return batch_read(b, i, res); }

// Device bytes a request adds to a batch (upper bound; a target in host memory
// that cannot be read in place counts as copied).
int64_t server_request_bytes(const mg_palette* pal, const mg_mosaic* m) {
  const int64_t N = (int64_t)m->grid_w * m->grid_h;
  const int64_t padded = (int64_t)padded_cells((int)N);
  const int64_t k = std::max(pal->k, 1);
  const int64_t chains = m->enable_optimization ? std::max(m->chains, 1) : 0;
  int64_t bytes = padded * (16 + 4 + 8 * k + 16) + N * 8 + chains * (N * 4 + 32) +
                  N * pal->tw * pal->th * 3 + 4096 + (int64_t)sizeof(GreedyJob);
  if (!device_view_or_device(m->target)) bytes += 3ll * m->target_w * m->target_h;
  if (pal->P > 32768) bytes += 4ll * pal->P;  // the walk's counters in global memory
  return bytes;
}

}  // namespace mg
