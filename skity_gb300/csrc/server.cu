// Serving loop of the GB300 raster backend: requests (one canvas each, as a
// scene stream) are admitted against a device-memory budget and rendered in
// batches formed continuously -- whatever is queued when a worker frees up
// goes into its next batch -- by several workers, each with its own context
// and stream, so batches overlap on the device.
//
// No counterpart in the reference (its software canvas renders one canvas
// per host thread).  The pipeline per batch is the batch pipeline of
// pipeline.cu: parse + upload into the worker's resident buffers, a render
// planned on the device (one wait on the device per batch, at the end), the
// pixels of every request read back together.
//
// Admission: a request's footprint is estimated when it is submitted
// (RequestFootprint below); a batch takes requests in arrival order while
// the footprints of everything in flight stay within the budget.  A request
// whose footprint alone exceeds the budget is refused at submit.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "device.h"

namespace skc {
namespace {

double NowS() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t ticket = 0;
  std::vector<uint8_t> stream;
  uint32_t w = 0, h = 0;
  uint64_t footprint = 0;
  std::vector<uint8_t> pixels;
  int32_t status = SKITY_CUDA_NOT_READY;
  double t_submit = 0, t_start = 0, t_done = 0;
  uint32_t batch_size = 0;
};

// Device bytes a request may hold while in flight: its canvas (4 B/px),
// span-pool rows (a few 8-byte spans per row a draw covers: 32 B per draw
// and canvas row), geometry scratch and sweep state (bounded by 96 B per
// stream byte), plus 1 MiB of fixed buffers.
uint64_t RequestFootprint(uint32_t w, uint32_t h, uint32_t draws, size_t stream_bytes) {
  return 4ull * w * h + 32ull * draws * h + 96ull * stream_bytes + (1ull << 20);
}

}  // namespace
}  // namespace skc

struct skity_cuda_server_s {
  std::vector<skity_cuda_context> workers;
  std::vector<std::thread> threads;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<skc::Request>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<skc::Request>> table;
  uint64_t budget = 0, in_flight = 0;
  uint32_t max_batch = 64;
  uint64_t next_ticket = 1;
  bool stop = false;
  uint64_t batches = 0, completed = 0;  // totals since creation
};

namespace skc {
namespace {

void WorkerLoop(skity_cuda_server_s* sv, skity_cuda_context ctx) {
  // The worker's batch: rebuilt for every batch of requests, its device
  // buffers (paths, paints, geometry scratch, sweep memory, row tables,
  // bins, canvases) kept resident and reused, so a batch allocates only
  // when it outgrows every batch before it.
  DeviceBatch db;
  for (;;) {
    std::vector<std::shared_ptr<Request>> batch;
    uint64_t fp = 0;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] {
        return sv->stop ||
               (!sv->queue.empty() && sv->in_flight + sv->queue.front()->footprint <= sv->budget);
      });
      if (sv->stop) return;
      while (!sv->queue.empty() && batch.size() < sv->max_batch &&
             sv->in_flight + fp + sv->queue.front()->footprint <= sv->budget) {
        fp += sv->queue.front()->footprint;
        batch.push_back(sv->queue.front());
        sv->queue.pop_front();
      }
      sv->in_flight += fp;
    }
    const double t0 = NowS();
    int32_t rc = SKITY_CUDA_SUCCESS;
    {
      std::lock_guard<std::mutex> clk(ctx->mu);
      cudaSetDevice(ctx->device);
      db.Reset();
      std::vector<const uint8_t*> ptrs;
      std::vector<size_t> lens;
      std::vector<uint8_t*> outs;
      for (auto& r : batch) {
        ptrs.push_back(r->stream.data());
        lens.push_back(r->stream.size());
        r->pixels.resize((size_t)r->w * r->h * 4);
        outs.push_back(r->pixels.data());
      }
      rc = BuildFromStreams(db, (uint32_t)batch.size(), ptrs.data(), lens.data());
      if (!rc) rc = UploadBatch(ctx, db);
      if (!rc) rc = RenderBatch(ctx, db, true);
      if (!rc) rc = QueueReadCanvases(ctx, db, (uint32_t)batch.size(), outs.data());
      if (!rc && cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = SKITY_CUDA_ERROR_DEVICE;
      if (!rc) ctx->last = db.stats;
    }
    const double t1 = NowS();
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->in_flight -= fp;
      sv->batches++;
      for (auto& r : batch) {
        r->status = rc;
        r->t_start = t0;
        r->t_done = t1;
        r->batch_size = (uint32_t)batch.size();
        if (!rc) sv->completed++;
      }
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();
  }
}

}  // namespace
}  // namespace skc

extern "C" {

SKITY_CUDA_API int32_t skity_cuda_server_create(const skity_cuda_server_create_info* info,
                                                skity_cuda_server* out) {
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  skity_cuda_server_create_info ci{};
  ci.struct_size = sizeof ci;
  if (info) {
    if (info->struct_size < sizeof(skity_cuda_server_create_info))
      return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    ci = *info;
  }
  if (ci.memory_budget == 0) ci.memory_budget = 40ull << 30;
  if (ci.workers == 0) ci.workers = 2;
  if (ci.max_batch == 0) ci.max_batch = 64;
  if (ci.workers > 16) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  auto* sv = new (std::nothrow) skity_cuda_server_s();
  if (!sv) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  sv->budget = ci.memory_budget;
  sv->max_batch = ci.max_batch;
  for (uint32_t i = 0; i < ci.workers; ++i) {
    skity_cuda_context_create_info xi{};
    xi.struct_size = sizeof xi;
    xi.device = ci.device;
    xi.device_memory_budget = ci.memory_budget;
    skity_cuda_context c = nullptr;
    int32_t rc = skity_cuda_context_create(&xi, &c);
    if (rc) {
      for (auto w : sv->workers) skity_cuda_context_destroy(w);
      delete sv;
      return rc;
    }
    sv->workers.push_back(c);
  }
  for (auto w : sv->workers) sv->threads.emplace_back(skc::WorkerLoop, sv, w);
  *out = sv;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_server_submit(skity_cuda_server server, const uint8_t* stream,
                                                size_t stream_bytes, uint64_t* ticket) {
  if (!server) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!stream || !ticket) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  skc::StreamView sv;
  if (!skc::ParseStream(stream, stream_bytes, &sv)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  auto r = std::make_shared<skc::Request>();
  r->stream.assign(stream, stream + stream_bytes);
  r->w = sv.width;
  r->h = sv.height;
  r->footprint = skc::RequestFootprint(sv.width, sv.height, sv.nd, stream_bytes);
  r->t_submit = skc::NowS();
  {
    std::lock_guard<std::mutex> lk(server->mu);
    if (server->stop) return SKITY_CUDA_ERROR_INVALID_HANDLE;
    if (r->footprint > server->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
    r->ticket = server->next_ticket++;
    server->table[r->ticket] = r;
    server->queue.push_back(r);
    *ticket = r->ticket;
  }
  server->cv_work.notify_one();
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_server_wait(skity_cuda_server server, uint64_t ticket,
                                              uint32_t timeout_ms, uint8_t* out_pixels,
                                              skity_cuda_request_info* info) {
  if (!server) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  std::unique_lock<std::mutex> lk(server->mu);
  auto it = server->table.find(ticket);
  if (it == server->table.end()) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  std::shared_ptr<skc::Request> r = it->second;
  if (!server->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                [&] { return r->status != SKITY_CUDA_NOT_READY; }))
    return SKITY_CUDA_NOT_READY;
  server->table.erase(it);
  lk.unlock();
  if (info) {
    info->queue_ms = 1e3 * (r->t_start - r->t_submit);
    info->latency_ms = 1e3 * (r->t_done - r->t_submit);
    info->batch_size = r->batch_size;
    info->width = r->w;
    info->height = r->h;
  }
  if (r->status == SKITY_CUDA_SUCCESS && out_pixels)
    std::memcpy(out_pixels, r->pixels.data(), r->pixels.size());
  return r->status;
}

SKITY_CUDA_API void skity_cuda_server_destroy(skity_cuda_server server) {
  if (!server) return;
  {
    std::lock_guard<std::mutex> lk(server->mu);
    server->stop = true;
    for (auto& r : server->queue) r->status = SKITY_CUDA_ERROR_CANCELLED;
    server->queue.clear();
  }
  server->cv_work.notify_all();
  server->cv_done.notify_all();
  for (auto& t : server->threads) t.join();
  for (auto w : server->workers) skity_cuda_context_destroy(w);
  delete server;
}

}  // extern "C"
