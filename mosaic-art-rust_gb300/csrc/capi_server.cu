// capi_server.cu -- the request loop of the serving pattern (mg_server_*).
//
// No counterpart in the reference (its CLI makes one mosaic per process).  A
// server keeps one palette resident and serves mosaic requests submitted from
// any thread:
//  - requests wait in a FIFO queue;
//  - a dispatcher thread admits requests from the front of the queue into a
//    batch whenever a slot (a stream with its own reusable batch buffers) is
//    free, as long as the admitted requests' device memory stays within the
//    server's budget; a request that alone exceeds the budget fails with
//    MG_ERR_BUDGET.  Requests that arrive while other batches run are admitted
//    into the next free slot, so the work of successive batches overlaps on the
//    device (continuous batching at batch granularity);
//  - a completion thread waits for each batch, copies every request's grid and
//    image into the caller's buffers, records its latency (submission to
//    results on the host) and releases its memory.
// A request's results depend only on the request (its own seed and stream id),
// never on which other requests share its batch.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "capi_internal.h"

using namespace mg;
using Clock = std::chrono::steady_clock;

namespace mg {
// capi_batch.cu
int server_batch_setup(mg_batch* b, mg_ctx* ctx, mg_palette* pal, const mg_mosaic* ms, int n);
int server_batch_enqueue(mg_batch* b);
int server_batch_read(mg_batch* b, int i, mg_result* res);
mg_batch* server_batch_new();
void batch_free(mg_batch* b);
int64_t server_request_bytes(const mg_palette* pal, const mg_mosaic* m);
}  // namespace mg

namespace {

struct Request {
  uint64_t ticket;
  mg_mosaic m;
  int32_t* grid_out;
  uint8_t* image_out;
  int64_t bytes;
  Clock::time_point submitted;
};

struct Done {
  int status = MG_OK;
  mg_result res{};
  double latency_ms = 0.0;
};

struct Slot {
  mg_ctx* ctx = nullptr;
  mg_batch* batch = nullptr;
  std::vector<Request> reqs;
  cudaEvent_t done = nullptr;
  bool busy = false;
  int status = MG_OK;
  int64_t bytes = 0;
};

}  // namespace

struct mg_server {
  mg_palette* pal = nullptr;
  int device = 0;
  int max_batch = 64;
  int64_t budget = 0, in_use = 0, peak_in_use = 0;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv_dispatch, cv_complete, cv_done;
  std::deque<Request> pending;
  std::deque<int> inflight;  // slots in dispatch order
  std::map<uint64_t, Done> done;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread dispatcher, completer;
  // statistics
  int64_t submitted = 0, completed = 0, batches = 0, rejected = 0;
};

namespace {

void dispatch_loop(mg_server* S) {
  cudaSetDevice(S->device);
  for (;;) {
    std::vector<Request> take;
    int slot = -1;
    int64_t bytes = 0;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      for (;;) {
        if (S->stop) return;
        slot = -1;
        for (size_t i = 0; i < S->slots.size(); ++i)
          if (!S->slots[i].busy) {
            slot = (int)i;
            break;
          }
        if (slot >= 0 && !S->pending.empty()) {
          // FIFO admission within the budget
          while (!S->pending.empty() && (int)take.size() < S->max_batch) {
            Request& r = S->pending.front();
            if (r.bytes > S->budget) {  // can never fit
              Done d;
              d.status = MG_ERR_BUDGET;
              S->done[r.ticket] = d;
              ++S->rejected;
              S->pending.pop_front();
              S->cv_done.notify_all();
              continue;
            }
            if (S->in_use + bytes + r.bytes > S->budget) break;
            bytes += r.bytes;
            take.push_back(r);
            S->pending.pop_front();
          }
          if (!take.empty()) break;
        }
        S->cv_dispatch.wait(lk);
      }
      Slot& sl = S->slots[slot];
      sl.busy = true;
      sl.bytes = bytes;
      S->in_use += bytes;
      S->peak_in_use = std::max(S->peak_in_use, S->in_use);
      ++S->batches;
    }
    Slot& sl = S->slots[slot];
    sl.reqs = take;
    std::vector<mg_mosaic> ms;
    for (auto& r : take) ms.push_back(r.m);
    int st = server_batch_setup(sl.batch, sl.ctx, S->pal, ms.data(), (int)ms.size());
    if (st == MG_OK) st = server_batch_enqueue(sl.batch);
    if (st == MG_OK && cudaEventRecord(sl.done, sl.ctx->stream) != cudaSuccess) st = MG_ERR_CUDA;
    sl.status = st;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      S->inflight.push_back(slot);
    }
    S->cv_complete.notify_all();
  }
}

void complete_loop(mg_server* S) {
  cudaSetDevice(S->device);
  for (;;) {
    int slot = -1;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_complete.wait(lk, [&] { return S->stop || !S->inflight.empty(); });
      if (S->inflight.empty()) return;  // stopping
      slot = S->inflight.front();
      S->inflight.pop_front();
    }
    Slot& sl = S->slots[slot];
    if (sl.status == MG_OK && cudaEventSynchronize(sl.done) != cudaSuccess) sl.status = MG_ERR_CUDA;
    std::vector<Done> results(sl.reqs.size());
    for (size_t i = 0; i < sl.reqs.size(); ++i) {
      Done& d = results[i];
      d.status = sl.status;
      d.res.grid = sl.reqs[i].grid_out;
      d.res.image = sl.reqs[i].image_out;
      if (d.status == MG_OK) d.status = server_batch_read(sl.batch, (int)i, &d.res);
      d.latency_ms = std::chrono::duration<double, std::milli>(Clock::now() - sl.reqs[i].submitted).count();
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      for (size_t i = 0; i < sl.reqs.size(); ++i) S->done[sl.reqs[i].ticket] = results[i];
      S->completed += (int64_t)sl.reqs.size();
      S->in_use -= sl.bytes;
      sl.busy = false;
      sl.reqs.clear();
    }
    S->cv_done.notify_all();
    S->cv_dispatch.notify_all();
  }
}

}  // namespace

extern "C" {

void mg_server_config_default(mg_server_config* c) {
  if (!c) return;
  c->slots = 3;
  c->max_batch = 64;
  c->memory_budget_bytes = 120ll << 30;  // 120 GB
}

int mg_server_create(mg_ctx* ctx, mg_palette* pal, const mg_server_config* cfg, mg_server** out) {
  MG_CHECK(check_ctx(ctx));
  if (!pal || !cfg || !out) return fail(MG_ERR_ARG, "null argument");
  if (cfg->slots < 1 || cfg->max_batch < 1 || cfg->memory_budget_bytes <= 0)
    return fail(MG_ERR_ARG, "need slots >= 1, max_batch >= 1 and a positive budget");
  *out = nullptr;
  mg_server* S = new mg_server();
  S->pal = pal;
  S->device = ctx->device;
  S->max_batch = cfg->max_batch;
  S->budget = cfg->memory_budget_bytes;
  S->slots.resize(cfg->slots);
  for (auto& sl : S->slots) {
    int st = mg_ctx_create(ctx->device, &sl.ctx);
    if (st == MG_OK) sl.ctx->scoring = ctx->scoring;  // the creator's greedy scoring
    if (st == MG_OK && cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) st = MG_ERR_CUDA;
    if (st != MG_OK) {
      mg_server_destroy(S);
      return st;
    }
    sl.batch = server_batch_new();
  }
  try {
    S->dispatcher = std::thread(dispatch_loop, S);
    S->completer = std::thread(complete_loop, S);
  } catch (const std::exception&) {
    mg_server_destroy(S);  // nothing submitted yet: stops and joins whichever thread started
    return fail(MG_ERR_OOM, "cannot start the server's dispatcher and completion threads");
  }
  *out = S;
  return MG_OK;
}

int mg_server_submit(mg_server* S, const mg_mosaic* m, int32_t* grid_out, uint8_t* image_out, uint64_t* ticket) {
  if (!S || !m || !ticket) return fail(MG_ERR_ARG, "null argument");
  if (m->grid_w <= 0 || m->grid_h <= 0 || !m->target) return fail(MG_ERR_ARG, "invalid request");
  Request r;
  r.m = *m;
  r.grid_out = grid_out;
  r.image_out = image_out;
  r.bytes = server_request_bytes(S->pal, m);
  r.submitted = Clock::now();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->stop) return fail(MG_ERR_STATE, "server is stopping");
    r.ticket = S->next_ticket++;
    *ticket = r.ticket;
    S->pending.push_back(r);
    ++S->submitted;
  }
  S->cv_dispatch.notify_all();
  return MG_OK;
}

static int take_done(mg_server* S, uint64_t ticket, mg_result* res, double* latency_ms) {
  auto it = S->done.find(ticket);
  Done d = it->second;
  S->done.erase(it);
  if (res) {
    int32_t* g = res->grid;
    uint8_t* im = res->image;
    *res = d.res;
    res->grid = g;
    res->image = im;
  }
  if (latency_ms) *latency_ms = d.latency_ms;
  return d.status;
}

int mg_server_poll(mg_server* S, uint64_t ticket, mg_result* res, double* latency_ms) {
  if (!S) return fail(MG_ERR_ARG, "null server");
  std::lock_guard<std::mutex> lk(S->mu);
  if (!S->done.count(ticket)) return -1;  // still pending (or unknown)
  return take_done(S, ticket, res, latency_ms);
}

int mg_server_wait(mg_server* S, uint64_t ticket, mg_result* res, double* latency_ms) {
  if (!S) return fail(MG_ERR_ARG, "null server");
  std::unique_lock<std::mutex> lk(S->mu);
  if (ticket == 0 || ticket >= S->next_ticket) return fail(MG_ERR_ARG, "unknown ticket");
  S->cv_done.wait(lk, [&] { return S->done.count(ticket) > 0; });
  return take_done(S, ticket, res, latency_ms);
}

int mg_server_get_stats(mg_server* S, mg_server_stats* st) {
  if (!S || !st) return fail(MG_ERR_ARG, "null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  st->submitted = S->submitted;
  st->completed = S->completed;
  st->rejected = S->rejected;
  st->batches = S->batches;
  st->pending = (int64_t)S->pending.size();
  st->bytes_in_use = S->in_use;
  st->peak_bytes_in_use = S->peak_in_use;
  return MG_OK;
}

int64_t mg_server_request_bytes(mg_server* S, const mg_mosaic* m) {
  if (!S || !m) return -1;
  return server_request_bytes(S->pal, m);
}

int mg_server_destroy(mg_server* S) {
  if (!S) return MG_OK;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    // let queued and in-flight work finish
    S->cv_done.wait(lk, [&] { return S->pending.empty() && S->inflight.empty() && S->completed + S->rejected >= S->submitted; });
    S->stop = true;
  }
  S->cv_dispatch.notify_all();
  S->cv_complete.notify_all();
  if (S->dispatcher.joinable()) S->dispatcher.join();
  if (S->completer.joinable()) S->completer.join();
  for (auto& sl : S->slots) {
    if (sl.batch) batch_free(sl.batch);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.ctx) mg_ctx_destroy(sl.ctx);
  }
  delete S;
  return MG_OK;
}

}  // extern "C"
