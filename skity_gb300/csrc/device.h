// Device-side state of the raster pipeline shared by the batch / canvas C
// ABI (pipeline.cu) and the serving loop (server.cu): device buffers, a
// batch resident on the device, the context, and the pipeline entry points.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/skity_cuda.h"
#include "batch.h"

namespace skc {

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    release();
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    cap = want;
    return cudaSuccess;
  }
  template <typename T>
  T* as() const { return (T*)p; }
};

struct Context;

// Launch shape of the compositor and the granularity of its pass bins
// (skity_cuda_raster_config; chosen per batch, e.g. by the autotuner).
struct RasterConfig {
  uint32_t tile_w = 1024;    // row-tile width in pixels
  uint32_t ctas_per_sm = 6;  // persistent compositor CTAs per SM (0: one warp per tile)
  int32_t band_shift = 4;    // pass-bin bands of 1 << band_shift rows
  uint32_t sweep_warps = 2;  // warps per CTA of the register sweeps (1, 2 or 4)
};

// A batch resident on the device: inputs uploaded once, re-rendered on
// demand.
struct DeviceBatch {
  Context* ctx = nullptr;
  HostBatch hb;
  DevBuf verbs, pts, weights, draws, passes, canvases, brushes, stop_colors, stop_offsets;
  DevBuf conicals, cf_matrices, srgb_tables;
  DevBuf scratch, geom, sweep, sweepmem, rowspan, pass_spans, comp, pixels;
  DevBuf tasks_main, tasks_temp, temps, pass_list, roundtrip, pass_frags, err, pass_class;
  DevBuf band_off, bins, sweep_order;
  std::vector<RowTask> h_tasks_main, h_tasks_temp;
  std::vector<uint32_t> h_band_off, h_bins;
  uint32_t chunk = 1024;
  uint32_t n_bands = 0;
  RasterConfig cfg;
  DevBuf task_next;  // persistent compositor's counters
  DevBuf retry;      // DevBatch::sweep_retry
  DevBuf clip_states, clip_flags, clip_rows, clip_items;  // path clips
  // device planning (batches without path clips): status, per-pass scan
  // arrays and band ranges, bin segments, the tiles (main then temp) and
  // their sorted copy; capacities of the plan's buffers
  DevBuf plan_st, plan_a, plan_r, pband, segs, seg_cnt, tasks_in, tasks_sorted;
  DevBuf sort_keys, sort_hist;
  std::vector<BandSeg> h_segs;
  bool slices_dirty = true;   // pass capacities changed: slice offsets and passes re-uploaded
  uint64_t cap_sweep = 0, cap_rows = 0, cap_bins = 0;
  uint64_t cap_scratch = 0;
  // the launch parameters the replay graphs were recorded with
  DevBatch graph_b{};
  DevPlan graph_q{};
  int graph_launches = 0;
  // true when the caller has loaded the canvases' current pixels (a canvas
  // flush without a clear); otherwise a canvas without a clear colour starts
  // from transparent black, as a fresh Bitmap does
  bool keep_pixels = false;
  bool uploaded = false;
  // Replay of the planned render as one CUDA graph (device-resident
  // batches): the plan -- scratch capacities, sweep buffers, row tables,
  // bins -- depends only on the batch's inputs, so a re-render can run the
  // same launches on the same buffers without host round trips.
  bool want_graph = false;
  bool graph_ok = false;
  cudaGraphExec_t graphs[6] = {};
  DevBatch planned{};
  uint64_t planned_rows = 0;
  const void* planned_pool = nullptr;  // the context span pool the plan used
  skity_cuda_stats planned_stats{};
  ~DeviceBatch() {
    for (auto g : graphs)
      if (g) cudaGraphExecDestroy(g);
  }
  // Forgets the batch's canvases and draws but keeps its device buffers, so
  // the next batch built in it reuses their memory.
  void Reset() {
    for (auto& g : graphs) {
      if (g) cudaGraphExecDestroy(g);
      g = nullptr;
    }
    graph_ok = false;
    hb = HostBatch{};
    h_tasks_main.clear();
    h_tasks_temp.clear();
    h_band_off.clear();
    h_bins.clear();
    h_segs.clear();
    h_geom.clear();
    keep_pixels = false;
    uploaded = false;
    slices_dirty = true;
    cap_sweep = cap_rows = cap_bins = 0;
    stats = skity_cuda_stats{};
  }
  std::vector<PassGeom> h_geom;
  skity_cuda_stats stats{};
};

}  // namespace skc

struct skity_cuda_context_s {
  int device = 0;
  uint64_t budget = 0;
  // span pool shared by the context's renders (they are serialised), grown
  // to what the largest render so far needed
  skc::DevBuf span_pool, span_next;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t stage[12] = {};
  // largest plan needs seen by the context's device-planned renders (sweep
  // bytes, row entries, bin entries): first capacities of new batches
  uint64_t hint_sweep = 0, hint_rows = 0, hint_bins = 0;
  // the batch skity_cuda_render_streams builds each call in (its device
  // buffers are reused from call to call)
  skc::DeviceBatch* streams_batch = nullptr;
  ~skity_cuda_context_s() { delete streams_batch; }
  skc::RasterConfig cfg;  // default launch shape of new batches and canvases
  uint32_t num_sms = 0;
  skity_cuda_stats last{};
  std::mutex mu;
};

namespace skc {

int32_t CudaErr(cudaError_t e);
// Parses scene streams into the batch's host description.
int32_t BuildFromStreams(DeviceBatch& db, uint32_t count, const uint8_t* const* streams,
                         const size_t* bytes);
// Uploads the batch's inputs (once per batch).
int32_t UploadBatch(skity_cuda_context_s* ctx, DeviceBatch& db);
// Renders the batch on the context's stream (planned render, or the replay
// graphs when the batch has them); pixels stay on the device.
int32_t RenderBatch(skity_cuda_context_s* ctx, DeviceBatch& db, bool timed);
// Rebuilds the row tiles and bands of an uploaded batch for `cfg`; the next
// render plans again.
int32_t ApplyConfig(skity_cuda_context_s* ctx, DeviceBatch& db, const RasterConfig& cfg);
// Copies canvas `index` of the batch to host memory (row_bytes 0: packed).
int32_t ReadCanvas(skity_cuda_context_s* ctx, DeviceBatch& db, uint32_t index, uint8_t* out,
                   size_t row_bytes);
// Renders the batch's main canvases one DrawPath at a time (per_draw.cu);
// batches with blur mask filters or path clips are not taken.
int32_t RenderPerDraw(skity_cuda_context_s* ctx, DeviceBatch& db);
// Queues the copies of canvases [0, count) to out[i] (packed rows) on the
// context stream; the caller waits for the stream.
int32_t QueueReadCanvases(skity_cuda_context_s* ctx, DeviceBatch& db, uint32_t count,
                          uint8_t* const* out);

}  // namespace skc
