// Host side of the GB300 raster backend: batch building, the launch
// pipeline and the C ABI declared in include/skity_cuda.h.
//
// A batch is a set of canvases, each with its draws in order.  Every
// DrawPath becomes one or two rasterisation passes (fill / stroke, in
// Paint::Style order, src/render/paint_order.hpp:12-31).  A draw with a
// kNormal blur mask filter becomes a temp canvas holding the draw
// (SWCanvas::HandleFilter, src/render/sw/sw_canvas.cc:797-826) plus an image
// pass on the main canvas that samples the blurred temp
// (ImageFilterBase::BlurBitmapToCanvas, src/effect/image_filter.cc:184-194).
//
// Pipeline per render:
//   geometry (retry passes whose scratch overflowed) -> host sizes rows ->
//   sweep count -> host sizes spans -> sweep emit -> composite temp canvases
//   -> StackBlur -> composite main canvases
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "device.h"

namespace skc {

int32_t CudaErr(cudaError_t e) {
  if (e == cudaSuccess) return SKITY_CUDA_SUCCESS;
  if (e == cudaErrorMemoryAllocation) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
  return SKITY_CUDA_ERROR_DEVICE;
}
#define SKC_TRY(expr)                              \
  do {                                             \
    cudaError_t _e = (expr);                       \
    if (_e != cudaSuccess) return CudaErr(_e);     \
  } while (0)

template <typename T>
static cudaError_t Upload(DevBuf& d, const std::vector<T>& v, cudaStream_t s) {
  cudaError_t e = d.ensure(std::max<size_t>(v.size() * sizeof(T), 16));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

// Inputs of the device planner that depend only on the canvases, their
// passes and the raster config: the compositor's tiles (main canvases, then
// the temp canvases) and the pass-bin segments.
static int32_t UploadDevicePlanInputs(skity_cuda_context_s* ctx, DeviceBatch& db) {
  cudaStream_t s = ctx->stream;
  std::vector<RowTask> all(db.h_tasks_main);
  all.insert(all.end(), db.h_tasks_temp.begin(), db.h_tasks_temp.end());
  SKC_TRY(Upload(db.tasks_in, all, s));
  BuildBandSegs(db.hb, db.cfg.band_shift, db.h_segs);
  SKC_TRY(Upload(db.segs, db.h_segs, s));
  return SKITY_CUDA_SUCCESS;
}

int32_t UploadBatch(skity_cuda_context_s* ctx, DeviceBatch& db) {
  cudaStream_t s = ctx->stream;
  HostBatch& hb = db.hb;
  if (hb.verbs.empty()) hb.verbs.push_back(0);
  if (hb.pts.empty()) hb.pts.push_back(mkP(0, 0));
  if (hb.weights.empty()) hb.weights.push_back(0);
  if (hb.stop_colors.empty()) {
    hb.stop_colors.push_back(make_float4(0, 0, 0, 0));
    hb.stop_offsets.push_back(0);
  }
  SKC_TRY(Upload(db.verbs, hb.verbs, s));
  SKC_TRY(Upload(db.pts, hb.pts, s));
  SKC_TRY(Upload(db.weights, hb.weights, s));
  SKC_TRY(Upload(db.draws, hb.draws, s));
  db.cfg = ctx->cfg;
  db.n_bands = AssignBands(hb, db.cfg.band_shift);
  SKC_TRY(Upload(db.canvases, hb.canvases, s));
  SKC_TRY(Upload(db.brushes, hb.brushes, s));
  SKC_TRY(Upload(db.stop_colors, hb.stop_colors, s));
  SKC_TRY(Upload(db.stop_offsets, hb.stop_offsets, s));
  if (hb.conicals.empty()) hb.conicals.push_back(ConicalParams{});
  SKC_TRY(Upload(db.conicals, hb.conicals, s));
  if (hb.cf_matrices.empty()) hb.cf_matrices.push_back(0);
  SKC_TRY(Upload(db.cf_matrices, hb.cf_matrices, s));
  {
    std::vector<uint8_t> tables(512);
    SRGBTables(tables.data());
    SKC_TRY(Upload(db.srgb_tables, tables, s));
  }
  SKC_TRY(Upload(db.temps, hb.temp_canvases, s));
  uint32_t maxw = 1;
  for (uint32_t c : hb.main_canvases) maxw = std::max(maxw, hb.canvases[c].w);
  db.chunk = std::min<uint32_t>(maxw, std::max<uint32_t>(32, std::min<uint32_t>(db.cfg.tile_w, 2048)));
  BuildRowTasks(hb, hb.main_canvases, db.chunk, db.h_tasks_main);
  BuildRowTasks(hb, hb.temp_canvases, db.chunk, db.h_tasks_temp);
  SKC_TRY(Upload(db.tasks_main, db.h_tasks_main, s));
  SKC_TRY(Upload(db.tasks_temp, db.h_tasks_temp, s));
  if (int32_t rc = UploadDevicePlanInputs(ctx, db)) return rc;
  // PixmapBrush colour round trip per channel value (Color4fFromColor then
  // Color4fToColor, bitmap_sampler.cc:21-29, color.cc:44-59)
  std::vector<uint8_t> rtab(256);
  for (int v = 0; v < 256; ++v) rtab[v] = ChannelToByte(v / 255.f);
  SKC_TRY(Upload(db.roundtrip, rtab, s));
  SKC_TRY(db.pixels.ensure(std::max<uint64_t>(hb.pixel_bytes, 16)));
  for (const HostBatch::ImageUpload& u : hb.image_uploads)  // the draws' images
    SKC_TRY(cudaMemcpyAsync(db.pixels.as<uint8_t>() + u.off, u.bytes.data(), u.bytes.size(),
                            cudaMemcpyHostToDevice, s));
  SKC_TRY(db.task_next.ensure(32));
  db.uploaded = true;
  return SKITY_CUDA_SUCCESS;
}

int32_t ApplyConfig(skity_cuda_context_s* ctx, DeviceBatch& db, const RasterConfig& cfg) {
  cudaStream_t s = ctx->stream;
  HostBatch& hb = db.hb;
  db.cfg = cfg;
  db.n_bands = AssignBands(hb, cfg.band_shift);
  SKC_TRY(Upload(db.canvases, hb.canvases, s));
  uint32_t maxw = 1;
  for (uint32_t c : hb.main_canvases) maxw = std::max(maxw, hb.canvases[c].w);
  db.chunk = std::min<uint32_t>(maxw, std::max<uint32_t>(32, std::min<uint32_t>(cfg.tile_w, 2048)));
  BuildRowTasks(hb, hb.main_canvases, db.chunk, db.h_tasks_main);
  BuildRowTasks(hb, hb.temp_canvases, db.chunk, db.h_tasks_temp);
  if (int32_t rc = UploadDevicePlanInputs(ctx, db)) return rc;
  for (auto& g : db.graphs) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  db.graph_ok = false;
  SKC_TRY(cudaStreamSynchronize(s));
  return SKITY_CUDA_SUCCESS;
}

// The launches of a planned render, in five parts (so that the stages can
// be timed between graph launches): 0 canvases without a clear colour
// zeroed and the geometry of every pass; 1 sweep-state resets and the
// sweeps; 2 composite of the blur temp canvases; 3 StackBlur; 4 composite
// of the main canvases.  Returns the number of kernel launches.
static int EnqueuePlanned(skity_cuda_context_s* ctx, DeviceBatch& db, cudaStream_t s, int part) {
  HostBatch& hb = db.hb;
  DevBatch b = db.planned;
  const uint32_t np = b.n_passes;
  b.pass_list = nullptr;
  b.n_list = np;
  switch (part) {
    case 0:
      if (!db.keep_pixels) {
        for (uint32_t c : hb.main_canvases) {
          const CanvasDesc& cd = hb.canvases[c];
          if (!cd.has_clear)
            cudaMemsetAsync(db.pixels.as<uint8_t>() + cd.px_off, 0, (size_t)cd.w * cd.h * 4, s);
        }
      }
      return LaunchGeometry(b, s);
    case 1:
      cudaMemsetAsync(db.rowspan.p, 0, std::max<uint64_t>(db.planned_rows, 1) * sizeof(uint2), s);
      cudaMemsetAsync(db.err.p, 0, 16, s);
      cudaMemsetAsync(db.pass_class.p, 0, std::max<size_t>(np, 1), s);
      cudaMemsetAsync(ctx->span_next.p, 0, 8, s);
      cudaMemsetAsync(b.sweep_done, 0, 16, s);
      cudaMemsetAsync(b.sweep_retry, 0, 4, s);
      {
        int n = LaunchSweep(b, s);
        if (b.n_clip_states || b.n_clip_items) {
          cudaMemsetAsync(b.clip_flags, 0, 8 * (size_t)std::max<uint32_t>(b.n_clip_states, 1), s);
          n += LaunchPathClips(b, hb.clip_states.data(), b.n_clip_states, s);
        }
        return n;
      }
    case 2:
      if (db.h_tasks_temp.empty()) return 0;
      cudaMemsetAsync(b.task_next, 0, 4, s);
      return LaunchComposite(b, db.tasks_temp.as<RowTask>(), (uint32_t)db.h_tasks_temp.size(),
                             db.chunk, db.cfg.ctas_per_sm, ctx->num_sms, b.task_next, s);
    case 3:
      if (db.h_tasks_temp.empty()) return 0;
      return LaunchBlur(b, db.temps.as<uint32_t>(), (uint32_t)hb.temp_canvases.size(),
                        hb.max_temp_h, hb.max_temp_w, hb.max_temp_style, s);
    default:
      cudaMemsetAsync(b.task_next + 1, 0, 4, s);
      return LaunchComposite(b, db.tasks_main.as<RowTask>(), (uint32_t)db.h_tasks_main.size(),
                             db.chunk, db.cfg.ctas_per_sm, ctx->num_sms, b.task_next + 1, s);
  }
}

// Milliseconds between two recorded events (0 if the runtime cannot say;
// the error is cleared so it does not surface at a later call).
static double ElapsedMs(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0.0;
  }
  return (double)ms;
}
static double StageMs(skity_cuda_context_s* ctx, int a, int b) {
  return ElapsedMs(ctx->stage[a], ctx->stage[b]);
}

static void DropReplay(DeviceBatch& db) {
  for (auto& g : db.graphs) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  db.graph_ok = false;
}

// Records the replay graphs of a batch whose plan is current.
static void CaptureReplay(skity_cuda_context_s* ctx, DeviceBatch& db) {
  DropReplay(db);
  cudaStream_t s = ctx->stream;
  bool ok = true;
  for (int part = 0; part < 5 && ok; ++part) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      ok = false;
      break;
    }
    const int n = EnqueuePlanned(ctx, db, s, part);
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess || !g) {
      ok = false;
    } else if (n > 0 || part == 0 || part == 1) {
      if (cudaGraphInstantiate(&db.graphs[part], g, 0) != cudaSuccess) {
        db.graphs[part] = nullptr;
        ok = false;
      }
    }
    if (g) cudaGraphDestroy(g);
  }
  cudaGetLastError();
  if (!ok) {
    DropReplay(db);
    return;
  }
  db.graph_ok = true;
}

static int32_t PlanAndRender(skity_cuda_context_s* ctx, DeviceBatch& db, bool timed);

// ---------------------------------------------------------------------------
// Device-planned render (batches without path clips): geometry -> device
// plan -> sweeps -> composite of the temp canvases -> StackBlur -> composite
// of the main canvases, all queued on the stream with no host round trip;
// the host waits once, at the end, for the plan's status and the device
// self-checks.  A plan that fell short (geometry scratch, sweep memory, row
// table, pass bins, span pool) is rendered again with the buffers grown to
// what the status reports.
// ---------------------------------------------------------------------------
static uint64_t GuessSweepBytes(const HostBatch& hb) {
  uint64_t t = 0;
  for (const PassDesc& pd : hb.passes) {
    const uint32_t w = std::min<uint32_t>(hb.canvases[pd.canvas].w, 2048);
    t += (SweepMemBytes(pd.cap[12], (int)w + 2) + 255) & ~uint64_t(255);
  }
  return t;
}
static uint64_t GuessRows(const HostBatch& hb) {
  uint64_t t = 0;
  for (const PassDesc& pd : hb.passes) t += hb.canvases[pd.canvas].h;
  return std::min<uint64_t>(t, 64ull << 20);
}
static uint64_t GuessBins(const HostBatch& hb, int shift) {
  uint64_t t = 0;
  for (const CanvasDesc& cd : hb.canvases)
    t += (uint64_t)((cd.h + (1u << shift) - 1) >> shift) * (cd.pass1 - cd.pass0);
  return std::min<uint64_t>(std::max<uint64_t>(t, 1), 64ull << 20);
}

// Buffers of a device-planned render at the batch's current capacities, and
// the launch parameters over them.
static int32_t PrepareDevice(skity_cuda_context_s* ctx, DeviceBatch& db, DevBatch& b, DevPlan& q) {
  HostBatch& hb = db.hb;
  cudaStream_t s = ctx->stream;
  const uint32_t np = (uint32_t)hb.passes.size();
  const size_t npm = std::max<size_t>(np, 1);
  if (db.slices_dirty) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < np; ++i) {
      SliceLayout L;
      L.compute(hb.passes[i].cap, sizeof(Edge));
      hb.passes[i].slice_off = total;
      total += L.bytes;
    }
    if (ctx->budget && total > ctx->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
    SKC_TRY(db.scratch.ensure(std::max<uint64_t>(total, 16)));
    SKC_TRY(Upload(db.passes, hb.passes, s));
    db.slices_dirty = false;
  }
  SKC_TRY(db.geom.ensure(npm * sizeof(PassGeom)));
  SKC_TRY(db.sweep.ensure(npm * sizeof(PassSweep)));
  SKC_TRY(db.comp.ensure(npm * sizeof(PassComp)));
  SKC_TRY(db.pass_spans.ensure(npm * 4));
  SKC_TRY(db.pass_frags.ensure(npm * 8));
  SKC_TRY(db.pass_class.ensure(npm));
  SKC_TRY(db.retry.ensure((npm + 1) * 4));
  SKC_TRY(db.err.ensure(16));
  SKC_TRY(db.plan_st.ensure(sizeof(PlanStatus)));
  SKC_TRY(db.plan_a.ensure(npm * 8));
  SKC_TRY(db.plan_r.ensure(npm * 8));
  SKC_TRY(db.pband.ensure(npm * 8));
  SKC_TRY(db.sweep_order.ensure(npm * 4));
  SKC_TRY(db.seg_cnt.ensure(std::max<size_t>(db.h_segs.size(), 1) * 8));
  SKC_TRY(db.band_off.ensure(((size_t)db.n_bands + 1) * 4));
  const size_t nt = db.h_tasks_main.size() + db.h_tasks_temp.size();
  SKC_TRY(db.tasks_sorted.ensure(std::max<size_t>(nt, 1) * sizeof(RowTask)));
  SKC_TRY(db.task_next.ensure(32));
  SKC_TRY(ctx->span_next.ensure(8));
  {
    // bucket sorts: a key per item, 1024 counts per block of 2048 items
    const size_t items = std::max<size_t>(np, nt);
    SKC_TRY(db.sort_keys.ensure(std::max<size_t>(items, 1) * 2));
    SKC_TRY(db.sort_hist.ensure(((items + 2047) / 2048 + 1) * 1024 * 8));
  }
  if (!db.cap_sweep) db.cap_sweep = std::max(ctx->hint_sweep, GuessSweepBytes(hb));
  if (!db.cap_rows) db.cap_rows = std::max(ctx->hint_rows, GuessRows(hb));
  if (!db.cap_bins) db.cap_bins = std::max(ctx->hint_bins, GuessBins(hb, db.cfg.band_shift));
  if (ctx->budget && (db.cap_sweep > ctx->budget || db.cap_rows * 8 > ctx->budget ||
                      db.cap_bins * 4 > ctx->budget))
    return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
  SKC_TRY(db.sweepmem.ensure(std::max<uint64_t>(db.cap_sweep, 16)));
  SKC_TRY(db.rowspan.ensure(std::max<uint64_t>(db.cap_rows, 1) * sizeof(uint2)));
  SKC_TRY(db.bins.ensure(std::max<uint64_t>(db.cap_bins, 1) * 4));
  if (!ctx->span_pool.p) SKC_TRY(ctx->span_pool.ensure((uint64_t)(1 << 20) * sizeof(uint2)));

  // zeroed bytewise (padding included): the replay test compares the bytes
  std::memset(&b, 0, sizeof b);
  std::memset(&q, 0, sizeof q);
  b.verbs = db.verbs.as<uint8_t>();
  b.pts = db.pts.as<P>();
  b.weights = db.weights.as<float>();
  b.draws = db.draws.as<DrawDesc>();
  b.passes = db.passes.as<PassDesc>();
  b.n_passes = np;
  b.n_list = np;
  b.canvases = db.canvases.as<CanvasDesc>();
  b.scratch = db.scratch.as<uint8_t>();
  b.geom = db.geom.as<PassGeom>();
  b.sweep = db.sweep.as<PassSweep>();
  b.sweepmem = db.sweepmem.as<uint8_t>();
  b.rowspan = db.rowspan.as<uint2>();
  b.pass_spans = db.pass_spans.as<uint32_t>();
  b.pass_frags = db.pass_frags.as<unsigned long long>();
  b.err = db.err.as<uint32_t>();
  b.pass_class = db.pass_class.as<uint8_t>();
  uint32_t maxw = 1;
  for (const CanvasDesc& cd : hb.canvases) maxw = std::max(maxw, cd.w);
  // accumulator entries of a register-sweep warp in shared memory: a path
  // about as wide as its canvas fits (wider ones use their sweep memory)
  b.reg_diff_cap = std::max<int32_t>(4, std::min<int32_t>(((int32_t)maxw + 132 + 3) & ~3, kRegDiffMax));
  b.comp = db.comp.as<PassComp>();
  b.band_off = db.band_off.as<uint32_t>();
  b.bins = db.bins.as<uint32_t>();
  b.sweep_order = np ? db.sweep_order.as<uint32_t>() : nullptr;
  b.band_shift = db.cfg.band_shift;
  b.reg_warps = db.cfg.sweep_warps;
  b.sweep_retry = db.retry.as<uint32_t>();
  b.task_next = db.task_next.as<unsigned int>();
  b.sweep_done = db.task_next.as<unsigned int>() + 2;
  b.spans = ctx->span_pool.as<uint2>();
  b.span_cap = ctx->span_pool.cap / sizeof(uint2);
  b.span_next = ctx->span_next.as<unsigned long long>();
  b.any_general = 0;
  for (const CanvasDesc& cd : hb.canvases) b.any_general |= cd.general;
  b.brushes = db.brushes.as<Brush>();
  b.conicals = db.conicals.as<ConicalParams>();
  b.srgb_tables = db.srgb_tables.as<uint8_t>();
  b.cf_matrices = db.cf_matrices.as<int16_t>();
  b.stop_colors = db.stop_colors.as<float4>();
  b.stop_offsets = db.stop_offsets.as<float>();
  b.pixels = db.pixels.as<uint8_t>();
  b.roundtrip = db.roundtrip.as<uint8_t>();
  b.plan = db.plan_st.as<PlanStatus>();

  q.st = db.plan_st.as<PlanStatus>();
  q.a = db.plan_a.as<unsigned long long>();
  q.r = db.plan_r.as<unsigned long long>();
  q.pband = db.pband.as<uint2>();
  q.segs = db.segs.as<BandSeg>();
  q.n_segs = (uint32_t)db.h_segs.size();
  q.seg_cnt = db.seg_cnt.as<unsigned long long>();
  q.band_off = db.band_off.as<uint32_t>();
  q.n_bands = db.n_bands;
  q.bins = db.bins.as<uint32_t>();
  q.sweep_cap = db.cap_sweep;
  q.rows_cap = db.cap_rows;
  q.bins_cap = db.cap_bins;
  q.sweep_order = b.sweep_order ? db.sweep_order.as<uint32_t>() : nullptr;
  q.tasks_in = db.tasks_in.as<RowTask>();
  q.tasks_out = db.tasks_sorted.as<RowTask>();
  q.n_main = (uint32_t)db.h_tasks_main.size();
  q.n_temp = (uint32_t)db.h_tasks_temp.size();
  q.sort_keys = db.sort_keys.as<uint16_t>();
  q.sort_hist = db.sort_hist.as<unsigned long long>();
  return SKITY_CUDA_SUCCESS;
}

// The launches of one device-planned render, in six parts (timed apart):
// 0 clears, status reset and geometry; 1 the device plan; 2 the sweeps;
// 3 composite of the blur temp canvases; 4 StackBlur; 5 composite of the
// main canvases and the work totals.  Returns the number of kernel launches.
static int EnqueueDevice(DeviceBatch& db, const DevBatch& b, const DevPlan& q, uint32_t num_sms,
                         cudaStream_t s, int part) {
  HostBatch& hb = db.hb;
  switch (part) {
    case 0:
      if (!db.keep_pixels) {
        for (uint32_t c : hb.main_canvases) {
          const CanvasDesc& cd = hb.canvases[c];
          if (!cd.has_clear)
            cudaMemsetAsync(db.pixels.as<uint8_t>() + cd.px_off, 0, (size_t)cd.w * cd.h * 4, s);
        }
      }
      cudaMemsetAsync(q.st, 0, sizeof(PlanStatus), s);
      cudaMemsetAsync(b.err, 0, 16, s);
      return LaunchGeometry(b, s);
    case 1:
      return LaunchPlan(b, q, s);
    case 2:
      cudaMemsetAsync(b.span_next, 0, 8, s);
      cudaMemsetAsync(b.sweep_done, 0, 16, s);
      cudaMemsetAsync(b.sweep_retry, 0, 4, s);
      return LaunchSweep(b, s);
    case 3:
      if (!q.n_temp) return 0;
      cudaMemsetAsync(b.task_next, 0, 4, s);
      return LaunchComposite(b, q.tasks_out + q.n_main, q.n_temp, db.chunk, db.cfg.ctas_per_sm,
                             num_sms, b.task_next, s);
    case 4:
      if (!q.n_temp) return 0;
      return LaunchBlur(b, db.temps.as<uint32_t>(), (uint32_t)hb.temp_canvases.size(),
                        hb.max_temp_h, hb.max_temp_w, hb.max_temp_style, s);
    default: {
      cudaMemsetAsync(b.task_next + 1, 0, 4, s);
      int n = LaunchComposite(b, q.tasks_out, q.n_main, db.chunk, db.cfg.ctas_per_sm, num_sms,
                              b.task_next + 1, s);
      return n + LaunchPlanStats(b, q, s);
    }
  }
}

static void DropReplay(DeviceBatch& db);

// Records a device-planned render -- its six parts, every kernel of the
// batch -- as one replay graph.  The stage events are event-record nodes of
// the graph (recorded as the graph runs), so a replay keeps its per-stage
// timings.
static void CaptureDevice(skity_cuda_context_s* ctx, DeviceBatch& db, const DevBatch& b,
                          const DevPlan& q) {
  DropReplay(db);
  cudaStream_t s = ctx->stream;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  bool ok = true;
  int launches = 0;
  for (int part = 0; part < 6; ++part) {
    ok = ok && cudaEventRecordWithFlags(ctx->stage[2 * part], s, cudaEventRecordExternal) ==
                   cudaSuccess;
    launches += EnqueueDevice(db, b, q, ctx->num_sms, s, part);
    ok = ok && cudaEventRecordWithFlags(ctx->stage[2 * part + 1], s, cudaEventRecordExternal) ==
                   cudaSuccess;
  }
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s, &g);
  ok = ok && e == cudaSuccess && g && cudaGraphInstantiate(&db.graphs[0], g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();
  if (!ok) {
    DropReplay(db);
    return;
  }
  db.graph_ok = true;
  std::memcpy(&db.graph_b, &b, sizeof b);
  std::memcpy(&db.graph_q, &q, sizeof q);
  db.graph_launches = launches;
}

static double ElapsedMs(cudaEvent_t a, cudaEvent_t b);

static int32_t DeviceRender(skity_cuda_context_s* ctx, DeviceBatch& db, bool timed) {
  (void)timed;
  cudaStream_t s = ctx->stream;
  HostBatch& hb = db.hb;
  const uint32_t np = (uint32_t)hb.passes.size();
  skity_cuda_stats st{};
  st.draws = hb.draw_count;
  st.passes = np;
  const uint64_t kMaxPool = 0xFFFFFFFFull;  // span indices are 32-bit
  double discarded_ms = 0;
  for (int attempt = 0; attempt < 8; ++attempt) {
    DevBatch b;
    DevPlan q;
    int32_t rc = PrepareDevice(ctx, db, b, q);
    if (rc) return rc;
    const bool replay = db.graph_ok && std::memcmp(&b, &db.graph_b, sizeof b) == 0 &&
                        std::memcmp(&q, &db.graph_q, sizeof q) == 0;
    int launches = 0;
    SKC_TRY(cudaEventRecord(ctx->ev0, s));
    if (replay) {
      SKC_TRY(cudaGraphLaunch(db.graphs[0], s));  // the stage events are nodes of the graph
    } else {
      for (int part = 0; part < 6; ++part) {
        SKC_TRY(cudaEventRecord(ctx->stage[2 * part], s));
        launches += EnqueueDevice(db, b, q, ctx->num_sms, s, part);
        SKC_TRY(cudaEventRecord(ctx->stage[2 * part + 1], s));
      }
    }
    SKC_TRY(cudaEventRecord(ctx->ev1, s));
    SKC_TRY(cudaGetLastError());
    PlanStatus ps;
    uint32_t err = 0;
    unsigned long long used = 0;
    SKC_TRY(cudaMemcpyAsync(&ps, q.st, sizeof ps, cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaMemcpyAsync(&err, b.err, 4, cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaMemcpyAsync(&used, b.span_next, 8, cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaStreamSynchronize(s));
    st.host_syncs++;
    if (err) {
      std::fprintf(stderr, "skity_cuda: device self-check failed (code %u)\n", err);
      return SKITY_CUDA_ERROR_DEVICE;
    }
    if (ps.flags == 0 && used <= b.span_cap) {
      st.device_ms = ElapsedMs(ctx->ev0, ctx->ev1);
      st.geometry_ms = ElapsedMs(ctx->stage[0], ctx->stage[1]);
      st.plan_ms = ElapsedMs(ctx->stage[2], ctx->stage[3]);
      st.sweep_emit_ms = ElapsedMs(ctx->stage[4], ctx->stage[5]);
      st.composite_ms = ElapsedMs(ctx->stage[6], ctx->stage[7]) + ElapsedMs(ctx->stage[10], ctx->stage[11]);
      st.blur_ms = ElapsedMs(ctx->stage[8], ctx->stage[9]);
      st.sweep_count_ms = discarded_ms;
      st.edges = ps.edges;
      st.spans = ps.spans;
      st.fragments = 0;
      for (int k = 0; k < 4; ++k) {
        st.fragments_by_brush[k] = ps.frags_by_brush[k];
        st.fragments += ps.frags_by_brush[k];
      }
      for (uint32_t c : hb.main_canvases) st.pixels += (uint64_t)hb.canvases[c].w * hb.canvases[c].h;
      st.graph_replays = replay ? 1 : 0;
      st.kernel_launches = replay ? (uint64_t)db.graph_launches : (uint64_t)launches;
      ctx->hint_sweep = std::max<uint64_t>(ctx->hint_sweep, ps.sweep_need);
      ctx->hint_rows = std::max<uint64_t>(ctx->hint_rows, ps.rows_need);
      ctx->hint_bins = std::max<uint64_t>(ctx->hint_bins, ps.bins_need);
      db.stats = st;
      if (!replay && db.want_graph) CaptureDevice(ctx, db, b, q);
      return SKITY_CUDA_SUCCESS;
    }
    // grow what fell short and render again
    DropReplay(db);
    discarded_ms += ElapsedMs(ctx->ev0, ctx->ev1);
    st.retries++;
    if (ps.flags & kPlanGeomOverflow) {
      db.h_geom.resize(np);
      SKC_TRY(cudaMemcpy(db.h_geom.data(), db.geom.p, (size_t)np * sizeof(PassGeom),
                         cudaMemcpyDeviceToHost));
      for (uint32_t p = 0; p < np; ++p)
        if (db.h_geom[p].status) GrowCaps(hb.passes[p], db.h_geom[p]);
      db.slices_dirty = true;
    }
    if (ps.sweep_need > db.cap_sweep) db.cap_sweep = ps.sweep_need + ps.sweep_need / 8;
    if (ps.rows_need > db.cap_rows) db.cap_rows = ps.rows_need + ps.rows_need / 8;
    if (ps.bins_need > db.cap_bins) db.cap_bins = ps.bins_need + ps.bins_need / 8;
    if (used > b.span_cap) {
      if (used > kMaxPool) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
      const uint64_t grow = std::min<uint64_t>(used + used / 16, kMaxPool);
      if (ctx->budget && grow * sizeof(uint2) > ctx->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
      ctx->span_pool.release();
      SKC_TRY(ctx->span_pool.ensure(grow * sizeof(uint2)));
    }
  }
  return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
}

// Render of a resident batch; pixels stay on the device.  A batch whose
// replay graph is current re-renders with one graph launch; the graph's
// device self-checks (error word, span pool use) are read back, and any
// surprise falls back to a full planned render.
int32_t RenderBatch(skity_cuda_context_s* ctx, DeviceBatch& db, bool timed) {
  // batches without path clips are planned on the device
  if (db.hb.clip_states.empty()) return DeviceRender(ctx, db, timed);
  if (db.graph_ok && db.planned_pool == ctx->span_pool.p) {
    cudaStream_t s = ctx->stream;
    static const int kStageEv[5][2] = {{0, 1}, {4, 5}, {6, 7}, {7, 8}, {8, 9}};
    SKC_TRY(cudaEventRecord(ctx->ev0, s));
    for (int part = 0; part < 5; ++part) {
      if (part != 3) SKC_TRY(cudaEventRecord(ctx->stage[kStageEv[part][0]], s));
      if (db.graphs[part]) SKC_TRY(cudaGraphLaunch(db.graphs[part], s));
      SKC_TRY(cudaEventRecord(ctx->stage[kStageEv[part][1]], s));
    }
    SKC_TRY(cudaEventRecord(ctx->ev1, s));
    uint32_t err = 0;
    unsigned long long used = 0;
    SKC_TRY(cudaMemcpyAsync(&err, db.err.p, 4, cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaMemcpyAsync(&used, ctx->span_next.p, 8, cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaStreamSynchronize(s));
    if (err == 0 && used <= db.planned.span_cap) {
      skity_cuda_stats st = db.planned_stats;
      st.device_ms = ElapsedMs(ctx->ev0, ctx->ev1);
      st.geometry_ms = StageMs(ctx, 0, 1);
      st.sweep_count_ms = 0;
      st.sweep_emit_ms = StageMs(ctx, 4, 5);
      st.composite_ms = StageMs(ctx, 6, 7) + StageMs(ctx, 8, 9);
      st.blur_ms = StageMs(ctx, 7, 8);
      st.retries = 0;
      st.graph_replays = 1;
      db.stats = st;
      return SKITY_CUDA_SUCCESS;
    }
    DropReplay(db);
  }
  int32_t rc = PlanAndRender(ctx, db, timed);
  if (rc == SKITY_CUDA_SUCCESS && db.want_graph) {
    db.planned_pool = ctx->span_pool.p;
    CaptureReplay(ctx, db);
  }
  return rc;
}

// Full render of a resident batch with planning (geometry sizes read back,
// sweep buffers and bins built on the host); pixels stay on the device.
static int32_t PlanAndRender(skity_cuda_context_s* ctx, DeviceBatch& db, bool timed) {
  cudaStream_t s = ctx->stream;
  HostBatch& hb = db.hb;
  const uint32_t np = (uint32_t)hb.passes.size();
  skity_cuda_stats st{};
  st.draws = hb.draw_count;
  st.passes = np;
  if (timed) SKC_TRY(cudaEventRecord(ctx->ev0, s));
  if (!db.keep_pixels) {
    for (uint32_t c : hb.main_canvases) {
      const CanvasDesc& cd = hb.canvases[c];
      if (!cd.has_clear)
        SKC_TRY(cudaMemsetAsync(db.pixels.as<uint8_t>() + cd.px_off, 0, (size_t)cd.w * cd.h * 4, s));
    }
  }

  // ---- geometry with scratch-capacity retries
  std::vector<uint32_t> todo(np);
  for (uint32_t i = 0; i < np; ++i) todo[i] = i;
  db.h_geom.assign(np, PassGeom{});
  SKC_TRY(db.geom.ensure(std::max<size_t>(np, 1) * sizeof(PassGeom)));
  for (int attempt = 0; attempt < 8 && !todo.empty(); ++attempt) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < np; ++i) {
      SliceLayout L;
      L.compute(hb.passes[i].cap, sizeof(Edge));
      hb.passes[i].slice_off = total;
      total += L.bytes;
    }
    if (ctx->budget && total > ctx->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
    SKC_TRY(db.scratch.ensure(std::max<uint64_t>(total, 16)));
    SKC_TRY(Upload(db.passes, hb.passes, s));
    SKC_TRY(Upload(db.pass_list, todo, s));
    DevBatch b{};
    b.verbs = db.verbs.as<uint8_t>();
    b.pts = db.pts.as<P>();
    b.weights = db.weights.as<float>();
    b.draws = db.draws.as<DrawDesc>();
    b.passes = db.passes.as<PassDesc>();
    b.n_passes = np;
    b.canvases = db.canvases.as<CanvasDesc>();
    b.scratch = db.scratch.as<uint8_t>();
    b.geom = db.geom.as<PassGeom>();
    b.pass_list = db.pass_list.as<uint32_t>();
    b.n_list = (uint32_t)todo.size();
    SKC_TRY(cudaEventRecord(ctx->stage[0], s));
    st.kernel_launches += LaunchGeometry(b, s);
    SKC_TRY(cudaEventRecord(ctx->stage[1], s));
    SKC_TRY(cudaGetLastError());
    SKC_TRY(cudaMemcpyAsync(db.h_geom.data(), db.geom.p, np * sizeof(PassGeom),
                            cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaStreamSynchronize(s));
    // Passes whose scratch overflowed get bigger capacities; since every
    // slice offset then moves, the whole geometry stage is run again.
    uint32_t grown = 0;
    for (uint32_t p : todo) {
      const PassGeom& g = db.h_geom[p];
      if (g.status == 0) continue;
      GrowCaps(hb.passes[p], g);
      grown++;
    }
    st.retries += grown;
    if (grown == 0) todo.clear();
  }
  if (!todo.empty()) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;

  // ---- per-pass sweep buffers and row-span tables
  std::vector<PassSweep> sw;
  SweepPlan pl = PlanSweep(hb, db.h_geom, sw);
  const uint64_t rows = pl.rows;
  st.edges = pl.edges;
  if (rows >= 0xFFFFFFFFull) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
  SKC_TRY(Upload(db.sweep, sw, s));
  SKC_TRY(db.sweepmem.ensure(std::max<uint64_t>(pl.sweep_bytes, 16)));
  SKC_TRY(db.rowspan.ensure(std::max<uint64_t>(rows, 1) * sizeof(uint2)));
  SKC_TRY(db.pass_spans.ensure(std::max<size_t>(np, 1) * 4));
  SKC_TRY(db.pass_frags.ensure(std::max<size_t>(np, 1) * 8));
  SKC_TRY(db.err.ensure(16));
  SKC_TRY(db.pass_class.ensure(std::max<size_t>(np, 1)));
  SKC_TRY(db.retry.ensure((std::max<size_t>(np, 1) + 1) * 4));
  SKC_TRY(ctx->span_next.ensure(8));
  std::vector<PassComp> comp;
  PlanComp(hb, db.h_geom, sw, comp);
  SKC_TRY(Upload(db.comp, comp, s));
  BuildBins(hb, comp, db.n_bands, db.cfg.band_shift, db.h_band_off, db.h_bins);
  SKC_TRY(Upload(db.band_off, db.h_band_off, s));
  SKC_TRY(Upload(db.bins, db.h_bins, s));
  OrderRowTasks(hb, db.h_band_off, db.cfg.band_shift, db.h_tasks_main);
  OrderRowTasks(hb, db.h_band_off, db.cfg.band_shift, db.h_tasks_temp);
  SKC_TRY(Upload(db.tasks_main, db.h_tasks_main, s));
  SKC_TRY(Upload(db.tasks_temp, db.h_tasks_temp, s));
  std::vector<uint32_t> order;
  SweepOrder(db.h_geom, order);
  SKC_TRY(Upload(db.sweep_order, order, s));
  // path clips: the states' rows and the clipped draws' (pass, row) items
  std::vector<uint2> clip_items;
  const uint64_t clip_state_rows = PlanPathClips(hb, db.h_geom, clip_items);
  if (clip_state_rows >= 0xFFFFFFFFull || clip_items.size() >= 0xFFFFFFFFull)
    return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
  if (!hb.clip_states.empty()) SKC_TRY(Upload(db.clip_states, hb.clip_states, s));
  SKC_TRY(db.clip_flags.ensure(8 * std::max<size_t>(hb.clip_states.size(), 1)));
  SKC_TRY(db.clip_rows.ensure(8 * std::max<uint64_t>(clip_state_rows, 1)));
  if (!clip_items.empty()) SKC_TRY(Upload(db.clip_items, clip_items, s));
  // span indices are 32-bit
  const uint64_t kMaxPool = 0xFFFFFFFFull;
  uint64_t want = std::min<uint64_t>(std::max<uint64_t>(pl.span_estimate, 1 << 16), kMaxPool);
  if (ctx->span_pool.cap / sizeof(uint2) < want) {
    if (ctx->budget && want * sizeof(uint2) > ctx->budget) want = ctx->budget / sizeof(uint2);
    SKC_TRY(ctx->span_pool.ensure(want * sizeof(uint2)));
  }

  DevBatch b{};
  b.verbs = db.verbs.as<uint8_t>();
  b.pts = db.pts.as<P>();
  b.weights = db.weights.as<float>();
  b.draws = db.draws.as<DrawDesc>();
  b.passes = db.passes.as<PassDesc>();
  b.n_passes = np;
  b.canvases = db.canvases.as<CanvasDesc>();
  b.scratch = db.scratch.as<uint8_t>();
  b.geom = db.geom.as<PassGeom>();
  b.sweep = db.sweep.as<PassSweep>();
  b.sweepmem = db.sweepmem.as<uint8_t>();
  b.rowspan = db.rowspan.as<uint2>();
  b.pass_spans = db.pass_spans.as<uint32_t>();
  b.pass_frags = db.pass_frags.as<unsigned long long>();
  b.err = db.err.as<uint32_t>();
  b.pass_class = db.pass_class.as<uint8_t>();
  b.reg_diff_cap = RegDiffCap(pl);
  b.comp = db.comp.as<PassComp>();
  b.band_off = db.band_off.as<uint32_t>();
  b.bins = db.bins.as<uint32_t>();
  b.sweep_order = np ? db.sweep_order.as<uint32_t>() : nullptr;
  b.band_shift = db.cfg.band_shift;
  b.reg_warps = db.cfg.sweep_warps;
  b.sweep_retry = db.retry.as<uint32_t>();
  b.task_next = db.task_next.as<unsigned int>();
  b.sweep_done = db.task_next.as<unsigned int>() + 2;
  b.span_next = ctx->span_next.as<unsigned long long>();
  b.clip_states = db.clip_states.as<ClipStateDesc>();
  b.n_clip_states = (uint32_t)hb.clip_states.size();
  b.any_general = 0;
  for (const CanvasDesc& cd : hb.canvases) b.any_general |= cd.general;
  b.clip_flags = db.clip_flags.as<uint32_t>();
  b.clip_rows = db.clip_rows.as<uint2>();
  b.clip_items = db.clip_items.as<uint2>();
  b.n_clip_items = (uint32_t)clip_items.size();
  // The sweep; if the span pool ran out it is grown to the size the sweep
  // reported and the sweep runs again (first renders of a context only).
  double discarded_ms = 0;
  for (int attempt = 0;; ++attempt) {
    b.spans = ctx->span_pool.as<uint2>();
    b.span_cap = ctx->span_pool.cap / sizeof(uint2);
    SKC_TRY(cudaMemsetAsync(db.rowspan.p, 0, std::max<uint64_t>(rows, 1) * sizeof(uint2), s));
    SKC_TRY(cudaMemsetAsync(db.err.p, 0, 16, s));
    SKC_TRY(cudaMemsetAsync(db.pass_class.p, 0, std::max<size_t>(np, 1), s));
    SKC_TRY(cudaMemsetAsync(ctx->span_next.p, 0, 8, s));
    SKC_TRY(cudaMemsetAsync(b.sweep_done, 0, 16, s));
    SKC_TRY(cudaMemsetAsync(b.sweep_retry, 0, 4, s));
    SKC_TRY(cudaEventRecord(ctx->stage[4], s));
    st.kernel_launches += LaunchSweep(b, s);
    if (b.n_clip_states || b.n_clip_items) {  // the path-clip stages use the span pool too
      SKC_TRY(cudaMemsetAsync(b.clip_flags, 0, 8 * (size_t)std::max<uint32_t>(b.n_clip_states, 1), s));
      st.kernel_launches += LaunchPathClips(b, hb.clip_states.data(), b.n_clip_states, s);
    }
    SKC_TRY(cudaEventRecord(ctx->stage[5], s));
    SKC_TRY(cudaGetLastError());
    unsigned long long used = 0;
    SKC_TRY(cudaMemcpyAsync(&used, ctx->span_next.p, 8, cudaMemcpyDeviceToHost, s));
    SKC_TRY(cudaStreamSynchronize(s));
    if (used <= b.span_cap) break;
    // the path-clip stages read rows the sweep wrote: a row past the end of
    // a short pool reads as empty, so a chain of clip states can show more
    // need on each try; with clips the pool doubles
    const int attempts = 3 + (int)hb.clip_states.size();
    if (attempt == attempts - 1 || used > kMaxPool) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
    discarded_ms += StageMs(ctx, 4, 5);
    const uint64_t grow =
        std::min<uint64_t>(hb.clip_states.empty() ? used + used / 16 : 2 * used, kMaxPool);
    if (ctx->budget && grow * sizeof(uint2) > ctx->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
    ctx->span_pool.release();
    SKC_TRY(ctx->span_pool.ensure(grow * sizeof(uint2)));
    st.retries++;
  }
  st.sweep_count_ms = discarded_ms;

  // ---- composite temp canvases, blur, composite main canvases
  b.brushes = db.brushes.as<Brush>();
  b.conicals = db.conicals.as<ConicalParams>();
  b.srgb_tables = db.srgb_tables.as<uint8_t>();
  b.cf_matrices = db.cf_matrices.as<int16_t>();
  b.stop_colors = db.stop_colors.as<float4>();
  b.stop_offsets = db.stop_offsets.as<float>();
  b.pixels = db.pixels.as<uint8_t>();
  b.roundtrip = db.roundtrip.as<uint8_t>();
  SKC_TRY(cudaEventRecord(ctx->stage[6], s));
  SKC_TRY(cudaMemsetAsync(db.task_next.p, 0, 8, s));
  if (!db.h_tasks_temp.empty()) {
    st.kernel_launches += LaunchComposite(b, db.tasks_temp.as<RowTask>(),
                                          (uint32_t)db.h_tasks_temp.size(), db.chunk,
                                          db.cfg.ctas_per_sm, ctx->num_sms, b.task_next, s);
  }
  SKC_TRY(cudaEventRecord(ctx->stage[7], s));
  if (!db.h_tasks_temp.empty()) {
    st.kernel_launches += LaunchBlur(b, db.temps.as<uint32_t>(), (uint32_t)hb.temp_canvases.size(),
                                     hb.max_temp_h, hb.max_temp_w, hb.max_temp_style, s);
  }
  SKC_TRY(cudaEventRecord(ctx->stage[8], s));
  st.kernel_launches += LaunchComposite(b, db.tasks_main.as<RowTask>(),
                                        (uint32_t)db.h_tasks_main.size(), db.chunk,
                                        db.cfg.ctas_per_sm, ctx->num_sms, b.task_next + 1, s);
  SKC_TRY(cudaEventRecord(ctx->stage[9], s));
  SKC_TRY(cudaGetLastError());
  if (timed) SKC_TRY(cudaEventRecord(ctx->ev1, s));
  uint32_t err = 0;
  SKC_TRY(cudaMemcpyAsync(&err, db.err.p, 4, cudaMemcpyDeviceToHost, s));
  SKC_TRY(cudaStreamSynchronize(s));
  if (err) {
    std::fprintf(stderr, "skity_cuda: device self-check failed (code %u)\n", err);
    return SKITY_CUDA_ERROR_DEVICE;
  }
  if (timed) st.device_ms = ElapsedMs(ctx->ev0, ctx->ev1);
  st.geometry_ms = StageMs(ctx, 0, 1);
  st.sweep_emit_ms = StageMs(ctx, 4, 5);
  st.composite_ms = StageMs(ctx, 6, 7) + StageMs(ctx, 8, 9);
  st.blur_ms = StageMs(ctx, 7, 8);
  db.planned = b;
  db.planned_rows = rows;
  for (uint32_t c : hb.main_canvases) st.pixels += (uint64_t)hb.canvases[c].w * hb.canvases[c].h;
  if (np) {
    std::vector<uint32_t> pspans(np);
    std::vector<unsigned long long> pfrags(np);
    SKC_TRY(cudaMemcpy(pspans.data(), db.pass_spans.p, np * 4, cudaMemcpyDeviceToHost));
    SKC_TRY(cudaMemcpy(pfrags.data(), db.pass_frags.p, np * 8, cudaMemcpyDeviceToHost));
    for (uint32_t p = 0; p < np; ++p) {
      st.spans += pspans[p];
      st.fragments += pfrags[p];
      // sweep and two-point conical gradients count with the radial ones
      const uint32_t kind = hb.brushes[hb.passes[p].brush].kind;
      st.fragments_by_brush[kind >= 4 ? 2 : kind] += pfrags[p];
    }
  }
  db.stats = st;
  db.planned_stats = st;
  return SKITY_CUDA_SUCCESS;
}

// The streams are parsed on the host's threads (BuildStreams), at most 32.
int32_t BuildFromStreams(DeviceBatch& db, uint32_t count, const uint8_t* const* streams,
                                const size_t* bytes) {
  const unsigned hw = std::thread::hardware_concurrency();
  return BuildStreams(db.hb, count, streams, bytes, std::min(hw ? hw : 1u, 32u));
}

int32_t ReadCanvas(skity_cuda_context_s* ctx, DeviceBatch& db, uint32_t index, uint8_t* out,
                          size_t row_bytes) {
  if (index >= db.hb.main_canvases.size()) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  const CanvasDesc& cd = db.hb.canvases[db.hb.main_canvases[index]];
  size_t w4 = (size_t)cd.w * 4;
  if (row_bytes == 0) row_bytes = w4;
  SKC_TRY(cudaMemcpy2DAsync(out, row_bytes, db.pixels.as<uint8_t>() + cd.px_off, w4, w4, cd.h,
                            cudaMemcpyDeviceToHost, ctx->stream));
  SKC_TRY(cudaStreamSynchronize(ctx->stream));
  return SKITY_CUDA_SUCCESS;
}

int32_t QueueReadCanvases(skity_cuda_context_s* ctx, DeviceBatch& db, uint32_t count,
                          uint8_t* const* out) {
  if (count > db.hb.main_canvases.size()) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  for (uint32_t i = 0; i < count; ++i) {
    const CanvasDesc& cd = db.hb.canvases[db.hb.main_canvases[i]];
    SKC_TRY(cudaMemcpyAsync(out[i], db.pixels.as<uint8_t>() + cd.px_off, (size_t)cd.w * cd.h * 4,
                            cudaMemcpyDeviceToHost, ctx->stream));
  }
  return SKITY_CUDA_SUCCESS;
}

}  // namespace skc

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
struct skity_cuda_batch_s {
  skity_cuda_context ctx;
  skc::DeviceBatch db;
};

namespace skc {

// One recorded canvas call of a display list (the reference's RecordedOp,
// src/recorder/recorded_op.hpp): the call's arguments, with the path,
// paint, shader, colour filter and image copied so the list owns them.
struct RecordedOp {
  enum Type : uint32_t {
    kClear, kDrawPath, kDrawImageRect, kSave, kRestore, kSaveLayer, kTranslate, kClipRect,
    kClipPath, kScale, kRotate, kSkew, kConcat, kSetMatrix, kConcat44, kSetMatrix44
  };
  Type type = kSave;
  float f[16] = {};  // colour / bounds / translation / rect / src + dst / matrix
  uint32_t u = 0;   // ClipOp / image filter
  bool has_path = false;
  std::vector<uint8_t> verbs;
  std::vector<float> pts, wts;
  uint32_t fill_type = 0;
  bool has_paint = false;
  skity_cuda_paint paint{};
  bool has_grad = false;
  skity_cuda_gradient grad{};
  std::vector<float> grad_colors, grad_offsets;
  bool has_cf = false;
  skity_cuda_color_filter cf{};
  bool has_ish = false;
  skity_cuda_image_shader ish{};
  bool has_img = false;  // the image of the image shader or of DrawImageRect
  skity_cuda_image img{};
  std::vector<uint8_t> img_px;

  void CopyPath(const skity_cuda_path* p) {
    has_path = true;
    verbs.assign(p->verbs, p->verbs + p->verb_count);
    pts.assign(p->points, p->points + 2 * (size_t)p->point_count);
    wts.assign(p->conic_weights, p->conic_weights + p->conic_weight_count);
    fill_type = p->fill_type;
  }
  void CopyImage(const skity_cuda_image* im) {
    has_img = true;
    img = *im;
    const uint8_t* px = (const uint8_t*)im->pixels;
    img_px.assign(px, px + (size_t)im->width * im->height * 4);
  }
  void CopyPaint(const skity_cuda_paint* q) {
    if (!q) return;
    has_paint = true;
    paint = *q;
    if (q->shader) {
      has_grad = true;
      grad = *q->shader;
      grad_colors.assign(q->shader->colors, q->shader->colors + 4 * (size_t)q->shader->stop_count);
      if (q->shader->has_offsets && q->shader->offsets)
        grad_offsets.assign(q->shader->offsets, q->shader->offsets + q->shader->stop_count);
    }
    if (q->color_filter) {
      has_cf = true;
      cf = *q->color_filter;
    }
    if (q->image_shader) {
      has_ish = true;
      ish = *q->image_shader;
      if (q->image_shader->image) CopyImage(q->image_shader->image);
    }
  }
  // views of the copies (valid while the op is not moved)
  skity_cuda_path PathView() const {
    skity_cuda_path p{};
    p.verbs = verbs.data();
    p.verb_count = (uint32_t)verbs.size();
    p.points = pts.data();
    p.point_count = (uint32_t)(pts.size() / 2);
    p.conic_weights = wts.data();
    p.conic_weight_count = (uint32_t)wts.size();
    p.fill_type = fill_type;
    return p;
  }
  skity_cuda_image ImageView() const {
    skity_cuda_image im = img;
    im.pixels = img_px.data();
    return im;
  }
  // q (and the shader records it points to) over the copies
  void PaintView(skity_cuda_paint* q, skity_cuda_gradient* g, skity_cuda_image_shader* is,
                 skity_cuda_image* im) const {
    *q = paint;
    q->shader = nullptr;
    q->color_filter = has_cf ? &cf : nullptr;
    q->image_shader = nullptr;
    if (has_grad) {
      *g = grad;
      g->colors = grad_colors.data();
      g->offsets = grad_offsets.empty() ? nullptr : grad_offsets.data();
      q->shader = g;
    }
    if (has_ish) {
      *is = ish;
      *im = ImageView();
      is->image = has_img ? im : nullptr;
      q->image_shader = is;
    }
  }
};

}  // namespace skc

struct skity_cuda_display_list_s {
  uint32_t width = 0, height = 0;
  std::vector<skc::RecordedOp> ops;
};

struct skity_cuda_canvas_s {
  skity_cuda_context ctx;
  // a recorder's canvas (skity_cuda_recorder_begin): calls are recorded as
  // ops of a display list instead of being drawn
  bool recording = false;
  std::vector<skc::RecordedOp> ops;
  uint32_t width, height;
  uint8_t* pixels;
  size_t row_bytes;
  // recorded scene (same records as the stream layout)
  bool has_clear = false;
  float clear[4] = {0, 0, 0, 0};
  bool dirty = false;   // draws recorded since the last flush
  std::vector<uint8_t> verbs;
  std::vector<float> pts, wts;
  std::vector<uint32_t> vo{0}, po{0}, wo{0};
  std::vector<skc::PaintRec> paints;
  std::vector<skc::GradRec> grads;
  std::vector<float> stop_colors, stop_offsets;
  // canvas matrix, global clip bounds and their save stack
  struct State {
    // the canvas matrix as the reference's CanvasState keeps it (canvas_state
    // .hpp:41,55,89-95): a SaveLayer starts a layer state whose world matrix
    // is the total matrix at the call and whose own matrix starts at the
    // identity; the calls after it multiply the layer's own matrix, and the
    // total is world * own (Matrix::operator*).  Column-major.
    skc::Mat4 m;      // the total matrix (GetTotalMatrix)
    skc::Mat4 world;  // the layer state's world matrix (the identity outside layers)
    skc::Mat4 own;    // the layer state's CurrentMatrix
    void set_own(const skc::Mat4& o) {
      own = o;
      m = skc::MatMul(world, own);
    }
    float clip[4] = {-1e9f, -1e9f, 1e9f, 1e9f};  // kMaxCullRect
    uint32_t path_clip = 0;  // the path-clip state (1-based in clip_states; 0: none)
    State() {
      m.identity();
      world.identity();
      own.identity();
    }
    float tx() const { return m.e[3][0]; }
    float ty() const { return m.e[3][1]; }
    // no perspective: CopyWithMatrix and MapRect then map points by
    // (sx, kx, tx, ky, sy, ty) alone (the z terms meet z = 0)
    bool affine() const { return m.e[0][3] == 0.f && m.e[1][3] == 0.f && m.e[3][3] == 1.f; }
    void six(float out[6]) const {
      out[0] = m.e[0][0];
      out[1] = m.e[1][0];
      out[2] = m.e[3][0];
      out[3] = m.e[0][1];
      out[4] = m.e[1][1];
      out[5] = m.e[3][1];
    }
    bool translation() const {
      return affine() && m.e[0][0] == 1.f && m.e[1][0] == 0.f && m.e[0][1] == 0.f &&
             m.e[1][1] == 1.f;
    }
    // Matrix::OnlyScaleAndTranslate (matrix.cc:171-187), every term checked
    bool scale_translate() const {
      return affine() && m.e[0][2] == 0.f && m.e[1][2] == 0.f && m.e[2][2] == 1.f &&
             m.e[3][2] == 0.f && m.e[2][0] == 0.f && m.e[2][1] == 0.f && m.e[2][3] == 0.f &&
             m.e[1][0] == 0.f && m.e[0][1] == 0.f;
    }
  };
  State st;
  std::vector<State> saved;
  // per saved level: the layer its Restore composites (1-based in `layers`; 0: none)
  std::vector<uint32_t> saved_layer;
  std::vector<skc::LayerRec> layers;
  std::vector<float> clips;  // per recorded draw: its clip bounds
  bool any_clip = false;
  std::vector<skc::ColorFilterRec> filters;  // per recorded draw: its colour filter
  bool any_filter = false;
  // path clips: the ClipPath calls (with their paths) and each draw's state
  std::vector<skc::ClipStateRec> clip_states;
  std::vector<uint8_t> clip_verbs;
  std::vector<float> clip_pts, clip_wts;
  std::vector<uint32_t> draw_clip_state;
  // per clip state: the canvas matrix of the call (sx, kx, tx, ky, sy, ty);
  // written to the scene when one of them is more than a translation
  std::vector<float> clip_matrices;
  bool any_clip_matrix = false;
  // images of the recorded draws (copied) and the per-draw image shaders
  std::vector<skc::ImageRec> images;
  std::vector<uint8_t> image_blob;
  std::vector<skc::ImageShaderRec> image_shaders;
  // per recorded draw: its canvas matrix (sx, kx, tx, ky, sy, ty); written
  // to the scene when a draw's matrix is more than a translation
  std::vector<float> matrices;
  bool any_matrix = false;
  skc::DeviceBatch db;
};

namespace {

// Canvas::CalculateGlobalClipBounds for kIntersect (canvas.cc:463-476): the
// rect mapped by the canvas matrix (Matrix::MapRect, matrix.cc:306-337: the
// corners mapped, w = 1, their min and max), intersected with the bounds
// (Rect::Intersect, rect.cc:160-172), or the empty rect.
void NarrowClipBounds(skity_cuda_canvas_s* canvas, float left, float top, float right,
                      float bottom) {
  float m6[6];
  canvas->st.six(m6);
  skc::Xform xf;
  xf.sx = m6[0];
  xf.kx = m6[1];
  xf.tx = m6[2];
  xf.ky = m6[3];
  xf.sy = m6[4];
  xf.ty = m6[5];
  xf.lin = !canvas->st.translation();
  const skc::P q[4] = {xf.map(skc::mkP(left, top)), xf.map(skc::mkP(right, top)),
                       xf.map(skc::mkP(right, bottom)), xf.map(skc::mkP(left, bottom))};
  float ml = q[0].x, mr = q[0].x, mt = q[0].y, mb = q[0].y;
  for (int i = 1; i < 4; ++i) {
    ml = std::min(q[i].x, ml);
    mr = std::max(q[i].x, mr);
    mt = std::min(q[i].y, mt);
    mb = std::max(q[i].y, mb);
  }
  float* c = canvas->st.clip;
  const float l = std::max(c[0], ml), r = std::min(c[2], mr);
  const float t = std::max(c[1], mt), b = std::min(c[3], mb);
  if (!(l < r && t < b)) {
    c[0] = c[1] = c[2] = c[3] = 0.f;
  } else {
    c[0] = l;
    c[1] = t;
    c[2] = r;
    c[3] = b;
  }
}

// SWCanvas::OnClipPath (sw_canvas.cc:317-335): a new clip state over the
// current one, with the canvas matrix and global clip bounds of the call.
void AddClipState(skity_cuda_canvas_s* canvas, const uint8_t* verbs, uint32_t nv,
                  const float* pts, uint32_t np, const float* wts, uint32_t nw, uint32_t op,
                  uint32_t fill_type) {
  skc::ClipStateRec c;
  std::memset(&c, 0, sizeof c);
  c.parent = canvas->st.path_clip;
  c.op = op;
  c.fill_type = fill_type;
  c.nv = nv;
  c.np = np;
  c.nw = nw;
  c.translate[0] = canvas->st.tx();
  c.translate[1] = canvas->st.ty();
  std::memcpy(c.bounds, canvas->st.clip, sizeof c.bounds);
  canvas->clip_states.push_back(c);
  canvas->clip_verbs.insert(canvas->clip_verbs.end(), verbs, verbs + nv);
  canvas->clip_pts.insert(canvas->clip_pts.end(), pts, pts + 2 * (size_t)np);
  if (nw) canvas->clip_wts.insert(canvas->clip_wts.end(), wts, wts + nw);
  float m6[6];
  canvas->st.six(m6);
  canvas->clip_matrices.insert(canvas->clip_matrices.end(), m6, m6 + 6);
  canvas->any_clip_matrix = canvas->any_clip_matrix || !canvas->st.translation();
  canvas->st.path_clip = (uint32_t)canvas->clip_states.size();
  canvas->dirty = true;
}

}  // namespace

extern "C" {

SKITY_CUDA_API const char* skity_cuda_version(void) { return "skity-gb300 0.1.0 (sm_103a)"; }

SKITY_CUDA_API int32_t skity_cuda_context_create(const skity_cuda_context_create_info* info,
                                                 skity_cuda_context* out) {
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  int device = 0;
  uint64_t budget = 16ull << 30;
  if (info) {
    if (info->struct_size < sizeof(skity_cuda_context_create_info))
      return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    device = info->device;
    if (info->device_memory_budget) budget = info->device_memory_budget;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || device < 0 || device >= n)
    return SKITY_CUDA_ERROR_INITIALIZATION_FAILED;
  auto* c = new (std::nothrow) skity_cuda_context_s();
  if (!c) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  c->device = device;
  c->budget = budget;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) == cudaSuccess)
    c->num_sms = (uint32_t)sms;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    delete c;
    return SKITY_CUDA_ERROR_INITIALIZATION_FAILED;
  }
  for (auto& e : c->stage) {
    if (cudaEventCreate(&e) != cudaSuccess) {
      delete c;
      return SKITY_CUDA_ERROR_INITIALIZATION_FAILED;
    }
  }
  *out = c;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API void skity_cuda_context_destroy(skity_cuda_context ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  for (auto& e : ctx->stage) cudaEventDestroy(e);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

// A config of the first layout (no sweep_warps) keeps the default of 2.
static bool ToConfig(const skity_cuda_raster_config* c, skc::RasterConfig* out) {
  const size_t v1 = offsetof(skity_cuda_raster_config, sweep_warps);
  if (!c || c->struct_size < v1) return false;
  if (c->tile_width < 32 || c->tile_width > 2048 || c->ctas_per_sm > 64) return false;
  int shift = -1;
  for (int k = 3; k <= 6; ++k)
    if (c->band_rows == (1u << k)) shift = k;
  if (shift < 0) return false;
  uint32_t warps = 2;
  if (c->struct_size >= sizeof(skity_cuda_raster_config)) {
    warps = c->sweep_warps;
    if (warps != 1 && warps != 2 && warps != 4) return false;
  }
  out->tile_w = c->tile_width;
  out->ctas_per_sm = c->ctas_per_sm;
  out->band_shift = shift;
  out->sweep_warps = warps;
  return true;
}

SKITY_CUDA_API int32_t skity_cuda_context_set_config(skity_cuda_context ctx,
                                                     const skity_cuda_raster_config* cfg) {
  if (!ctx) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  skc::RasterConfig rc;
  if (!ToConfig(cfg, &rc)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->cfg = rc;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_context_get_stats(skity_cuda_context ctx, skity_cuda_stats* out) {
  if (!ctx) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  *out = ctx->last;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_render_streams(skity_cuda_context ctx, uint32_t count,
                                                 const uint8_t* const* streams,
                                                 const size_t* stream_bytes,
                                                 uint8_t* const* out_pixels) {
  if (!ctx) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!streams || !stream_bytes || !out_pixels) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  if (!ctx->streams_batch) ctx->streams_batch = new (std::nothrow) skc::DeviceBatch();
  if (!ctx->streams_batch) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  skc::DeviceBatch& db = *ctx->streams_batch;
  db.Reset();
  auto ms_since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
  };
  int32_t rc = skc::BuildFromStreams(db, count, streams, stream_bytes);
  if (rc) return rc;
  const double parse_ms = ms_since(t0);
  auto t1 = std::chrono::steady_clock::now();
  rc = skc::UploadBatch(ctx, db);
  if (rc) return rc;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return SKITY_CUDA_ERROR_DEVICE;
  const double upload_ms = ms_since(t1);
  rc = skc::RenderBatch(ctx, db, true);
  if (rc) return rc;
  auto t2 = std::chrono::steady_clock::now();
  rc = skc::QueueReadCanvases(ctx, db, count, out_pixels);
  if (rc) return rc;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return SKITY_CUDA_ERROR_DEVICE;
  db.stats.host_syncs += 2;
  db.stats.parse_ms = parse_ms;
  db.stats.upload_ms = upload_ms;
  db.stats.readback_ms = ms_since(t2);
  db.stats.total_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  ctx->last = db.stats;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_batch_create(skity_cuda_context ctx, uint32_t count,
                                               const uint8_t* const* streams,
                                               const size_t* stream_bytes, skity_cuda_batch* out) {
  if (!ctx) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!streams || !stream_bytes || !out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  auto* b = new (std::nothrow) skity_cuda_batch_s();
  if (!b) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  b->ctx = ctx;
  int32_t rc = skc::BuildFromStreams(b->db, count, streams, stream_bytes);
  if (!rc) rc = skc::UploadBatch(ctx, b->db);
  b->db.want_graph = true;
  if (rc) {
    delete b;
    return rc;
  }
  *out = b;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_batch_render(skity_cuda_batch batch) {
  if (!batch) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  std::lock_guard<std::mutex> lock(batch->ctx->mu);
  cudaSetDevice(batch->ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  int32_t rc = skc::RenderBatch(batch->ctx, batch->db, true);
  batch->db.stats.total_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  batch->ctx->last = batch->db.stats;
  return rc;
}

SKITY_CUDA_API int32_t skity_cuda_batch_render_per_draw(skity_cuda_batch batch) {
  if (!batch) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  std::lock_guard<std::mutex> lock(batch->ctx->mu);
  cudaSetDevice(batch->ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  int32_t rc = skc::RenderPerDraw(batch->ctx, batch->db);
  batch->db.stats.total_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  batch->ctx->last = batch->db.stats;
  return rc;
}

SKITY_CUDA_API int32_t skity_cuda_batch_read(skity_cuda_batch batch, uint32_t index,
                                             uint8_t* out_pixels) {
  if (!batch) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!out_pixels) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(batch->ctx->mu);
  cudaSetDevice(batch->ctx->device);
  return skc::ReadCanvas(batch->ctx, batch->db, index, out_pixels, 0);
}

SKITY_CUDA_API int32_t skity_cuda_batch_set_config(skity_cuda_batch batch,
                                                   const skity_cuda_raster_config* cfg) {
  if (!batch) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  skc::RasterConfig rc;
  if (!ToConfig(cfg, &rc)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(batch->ctx->mu);
  cudaSetDevice(batch->ctx->device);
  return skc::ApplyConfig(batch->ctx, batch->db, rc);
}

SKITY_CUDA_API int32_t skity_cuda_batch_get_config(skity_cuda_batch batch,
                                                   skity_cuda_raster_config* out) {
  if (!batch) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  out->struct_size = sizeof(skity_cuda_raster_config);
  out->tile_width = batch->db.cfg.tile_w;
  out->ctas_per_sm = batch->db.cfg.ctas_per_sm;
  out->band_rows = 1u << batch->db.cfg.band_shift;
  out->sweep_warps = batch->db.cfg.sweep_warps;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API void skity_cuda_batch_destroy(skity_cuda_batch batch) {
  if (!batch) return;
  {
    std::lock_guard<std::mutex> lock(batch->ctx->mu);
    cudaSetDevice(batch->ctx->device);
    cudaStreamSynchronize(batch->ctx->stream);
  }
  delete batch;
}

// ---- canvas ----------------------------------------------------------------
SKITY_CUDA_API int32_t skity_cuda_canvas_create(skity_cuda_context ctx, uint32_t width,
                                                uint32_t height, void* pixels, size_t row_bytes,
                                                skity_cuda_canvas* out) {
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!ctx) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  // MakeSoftwareCanvas: null bitmap or zero size -> no canvas
  if (!pixels || width == 0 || height == 0) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (width > 65535 || height > 65535) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  if (row_bytes == 0) row_bytes = (size_t)width * 4;
  if (row_bytes < (size_t)width * 4) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  auto* c = new (std::nothrow) skity_cuda_canvas_s();
  if (!c) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  c->ctx = ctx;
  c->width = width;
  c->height = height;
  c->pixels = (uint8_t*)pixels;
  c->row_bytes = row_bytes;
  *out = c;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API void skity_cuda_canvas_destroy(skity_cuda_canvas canvas) { delete canvas; }

SKITY_CUDA_API int32_t skity_cuda_canvas_clear(skity_cuda_canvas canvas, const float color[4]) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!color) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kClear;
    std::memcpy(op.f, color, 16);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  if (canvas->st.path_clip) {
    // SWCanvas::OnDrawPaint under a path clip (sw_canvas.cc:413-439): the
    // canvas rect, rasterised with no matrix and no clip bounds, clipped by
    // the state, brushed with kSrc
    const float w = (float)canvas->width, h = (float)canvas->height;
    const uint8_t verbs[5] = {SKITY_CUDA_VERB_MOVE, SKITY_CUDA_VERB_LINE, SKITY_CUDA_VERB_LINE,
                              SKITY_CUDA_VERB_LINE, SKITY_CUDA_VERB_CLOSE};
    const float pts[8] = {0.f, 0.f, w, 0.f, w, h, 0.f, h};
    skity_cuda_path path{};
    path.verbs = verbs;
    path.verb_count = 5;
    path.points = pts;
    path.point_count = 4;
    skity_cuda_paint paint{};
    paint.blend_mode = 1;  // kSrc
    std::memcpy(paint.fill_color, color, 16);
    std::memcpy(paint.stroke_color, color, 16);
    paint.stroke_width = 1.f;
    paint.miter_limit = 4.f;
    const skity_cuda_canvas_s::State keep = canvas->st;
    canvas->st.m.identity();
    canvas->st.world.identity();
    canvas->st.own.identity();
    canvas->st.clip[0] = canvas->st.clip[1] = -1e9f;
    canvas->st.clip[2] = canvas->st.clip[3] = 1e9f;
    const int32_t rc = skity_cuda_canvas_draw_path(canvas, &path, &paint);
    canvas->st = keep;
    return rc;
  }
  // a Clear inside a layer clears the layer's bitmap in the reference (the
  // sub-canvas takes the DrawPaint); not taken here
  for (uint32_t l : canvas->saved_layer)
    if (l) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  // a kSrc fill of the whole canvas overwrites everything drawn before
  canvas->layers.clear();
  canvas->has_clear = true;
  std::memcpy(canvas->clear, color, 16);
  canvas->verbs.clear();
  canvas->pts.clear();
  canvas->wts.clear();
  canvas->vo.assign(1, 0);
  canvas->po.assign(1, 0);
  canvas->wo.assign(1, 0);
  canvas->paints.clear();
  canvas->grads.clear();
  canvas->stop_colors.clear();
  canvas->stop_offsets.clear();
  canvas->clips.clear();
  canvas->any_clip = false;
  canvas->filters.clear();
  canvas->any_filter = false;
  canvas->matrices.clear();
  canvas->any_matrix = false;
  canvas->draw_clip_state.clear();
  canvas->images.clear();
  canvas->image_blob.clear();
  canvas->image_shaders.clear();
  canvas->dirty = true;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_draw_path(skity_cuda_canvas canvas,
                                                   const skity_cuda_path* path,
                                                   const skity_cuda_paint* paint) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!path || !paint) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if ((path->verb_count && !path->verbs) || (path->point_count && !path->points) ||
      (path->conic_weight_count && !path->conic_weights))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  // verb/point/weight counts must agree (Path storage invariant)
  uint64_t need_p = 0, need_w = 0;
  for (uint32_t i = 0; i < path->verb_count; ++i) {
    switch (path->verbs[i]) {
      case SKITY_CUDA_VERB_MOVE: case SKITY_CUDA_VERB_LINE: need_p += 1; break;
      case SKITY_CUDA_VERB_QUAD: need_p += 2; break;
      case SKITY_CUDA_VERB_CONIC: need_p += 2; need_w += 1; break;
      case SKITY_CUDA_VERB_CUBIC: need_p += 3; break;
      case SKITY_CUDA_VERB_CLOSE: break;
      default: return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    }
  }
  if (need_p != path->point_count || need_w != path->conic_weight_count)
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (paint->blend_mode > 28) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;  // past kLuminosity
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kDrawPath;
    op.CopyPath(path);
    op.CopyPaint(paint);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  const skity_cuda_image_shader* is = paint->image_shader;
  if (is) {
    const skity_cuda_image* im = is->image;
    if (!im || !im->pixels || im->width == 0 || im->height == 0 || im->width > 16384 ||
        im->height > 16384 || (im->alpha_type != 2 && im->alpha_type != 3) || is->filter > 2 ||
        is->tile_x > 3 || is->tile_y > 3 || paint->shader)
      return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    const float* m = is->local_matrix;
    for (int i : {0, 2, 4, 5})
      if (!(std::fabs(m[i]) <= 1e30f)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    if (!(std::fabs(m[0]) >= 1e-30f) || !(std::fabs(m[4]) >= 1e-30f))
      return SKITY_CUDA_ERROR_INVALID_ARGUMENT;  // not invertible
    if (m[1] != 0.f || m[3] != 0.f) return SKITY_CUDA_ERROR_NOT_SUPPORTED;  // rotated / skewed
  }
  if (paint->color_filter) {
    skc::ColorFilterRec fr;
    std::memset(&fr, 0, sizeof fr);
    fr.type = paint->color_filter->type;
    fr.mode = paint->color_filter->blend_mode;
    std::memcpy(fr.matrix, paint->color_filter->matrix, sizeof fr.matrix);
    if (fr.type == 0 || !skc::ValidColorFilter(fr)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  }
  if (paint->blur_style > 4) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;  // past BlurStyle::kInner
  if (!skc::ValidPaint(paint->style, paint->cap, paint->join, paint->stroke_width,
                       paint->miter_limit, paint->blur_style ? paint->blur_radius : 0.f))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (!skc::ValidPath(path->verbs, path->verb_count, path->points, path->point_count,
                      path->conic_weights, path->conic_weight_count))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (paint->shader && (paint->shader->stop_count > 4096 || paint->shader->tile_mode > 3))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  skc::PaintRec pr;
  std::memset(&pr, 0, sizeof pr);
  pr.style = paint->style;
  pr.cap = paint->cap;
  pr.join = paint->join;
  pr.blend = paint->blend_mode;
  pr.fill_type = path->fill_type ? 1 : 0;
  pr.gradient = -1;
  pr.blur_style = paint->blur_style;
  pr.blur_radius = paint->blur_radius;
  std::memcpy(pr.fill_color, paint->fill_color, 16);
  std::memcpy(pr.stroke_color, paint->stroke_color, 16);
  pr.stroke_width = paint->stroke_width;
  pr.miter = paint->miter_limit;
  // the canvas matrix: a translation goes in the paint record; anything
  // more in the draw's matrix record
  if (!canvas->st.affine()) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  float ctm[6];
  canvas->st.six(ctm);
  const bool lin = !canvas->st.translation();
  pr.translate[0] = lin ? 0.f : ctm[2];
  pr.translate[1] = lin ? 0.f : ctm[5];
  if (lin ? !skc::ValidMatrix(ctm, path->points, path->point_count)
          : !skc::ValidTranslate(pr.translate, path->points, path->point_count))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  // shaders under scale and translation only (their device_to_local is
  // then the short inverse), a blur's filtered bitmap included; no layers
  // under more than a translation
  if ((paint->shader || paint->image_shader ||
       (paint->blur_style != 0 && paint->blur_radius > 0.f)) &&
      !canvas->st.scale_translate())
    return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  if (lin) {
    for (uint32_t l : canvas->saved_layer)
      if (l) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  }
  if (paint->shader) {
    const skity_cuda_gradient* g = paint->shader;
    if (!g->colors || (g->has_offsets && !g->offsets)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    skc::GradRec gr;
    std::memset(&gr, 0, sizeof gr);
    gr.type = g->type;
    gr.tile_mode = g->tile_mode;
    gr.stop_count = g->stop_count;
    gr.stop_start = (uint32_t)canvas->stop_offsets.size();
    gr.has_offsets = g->has_offsets;
    std::memcpy(gr.p0, g->p0, 8);
    std::memcpy(gr.p1, g->p1, 8);
    std::memcpy(gr.radius, g->radius, 8);
    for (uint32_t i = 0; i < g->stop_count; ++i) {
      canvas->stop_colors.insert(canvas->stop_colors.end(), g->colors + 4 * i, g->colors + 4 * i + 4);
      canvas->stop_offsets.push_back(g->has_offsets ? g->offsets[i] : 0.f);
    }
    pr.gradient = (int32_t)canvas->grads.size();
    canvas->grads.push_back(gr);
  }
  canvas->verbs.insert(canvas->verbs.end(), path->verbs, path->verbs + path->verb_count);
  canvas->pts.insert(canvas->pts.end(), path->points, path->points + 2 * (size_t)path->point_count);
  canvas->wts.insert(canvas->wts.end(), path->conic_weights,
                     path->conic_weights + path->conic_weight_count);
  canvas->vo.push_back((uint32_t)canvas->verbs.size());
  canvas->po.push_back((uint32_t)(canvas->pts.size() / 2));
  canvas->wo.push_back((uint32_t)canvas->wts.size());
  canvas->paints.push_back(pr);
  canvas->matrices.insert(canvas->matrices.end(), ctm, ctm + 6);
  canvas->any_matrix = canvas->any_matrix || lin;
  canvas->clips.insert(canvas->clips.end(), canvas->st.clip, canvas->st.clip + 4);
  canvas->any_clip = canvas->any_clip || !skc::IsNoClip(canvas->st.clip);
  skc::ColorFilterRec fr;
  std::memset(&fr, 0, sizeof fr);
  if (paint->color_filter) {
    fr.type = paint->color_filter->type;
    fr.mode = paint->color_filter->blend_mode;
    fr.color = paint->color_filter->color;
    std::memcpy(fr.matrix, paint->color_filter->matrix, sizeof fr.matrix);
    canvas->any_filter = true;
  }
  canvas->filters.push_back(fr);
  canvas->draw_clip_state.push_back(canvas->st.path_clip);
  skc::ImageShaderRec ir;
  std::memset(&ir, 0, sizeof ir);
  if (is) {
    const skity_cuda_image* im = is->image;
    const uint64_t bytes = (uint64_t)im->width * im->height * 4;
    skc::ImageRec rec;
    std::memset(&rec, 0, sizeof rec);
    rec.width = im->width;
    rec.height = im->height;
    rec.alpha_type = im->alpha_type;
    rec.offset = canvas->image_blob.size();
    const uint8_t* px = (const uint8_t*)im->pixels;
    canvas->image_blob.insert(canvas->image_blob.end(), px, px + bytes);
    canvas->images.push_back(rec);
    ir.image = (uint32_t)canvas->images.size();
    ir.filter = is->filter;
    ir.tile_x = is->tile_x;
    ir.tile_y = is->tile_y;
    std::memcpy(ir.local, is->local_matrix, sizeof ir.local);
  }
  canvas->image_shaders.push_back(ir);
  canvas->dirty = true;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_draw_image_rect(skity_cuda_canvas canvas,
                                                         const skity_cuda_image* image,
                                                         const float src[4], const float dst[4],
                                                         uint32_t filter,
                                                         const skity_cuda_paint* paint) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!image) return SKITY_CUDA_SUCCESS;
  if (!src || !dst || filter > 2) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kDrawImageRect;
    std::memcpy(op.f, src, 16);
    std::memcpy(op.f + 4, dst, 16);
    op.u = filter;
    op.CopyImage(image);
    op.CopyPaint(paint);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  // Rect::Width / Height; an empty src or dst draws nothing
  const float sw = src[2] - src[0], sh = src[3] - src[1];
  const float dw = dst[2] - dst[0], dh = dst[3] - dst[1];
  if (sw == 0 || sh == 0 || dw == 0 || dh == 0) return SKITY_CUDA_SUCCESS;
  // Translate(dst.L, dst.T) * Scale(dw / sw, dh / sh) * Translate(-src.L, -src.T)
  const skc::Mat4 local = skc::MatMul(
      skc::MatMul(skc::MatTranslate(dst[0], dst[1]), skc::MatScale(dw / sw, dh / sh)),
      skc::MatTranslate(-src[0], -src[1]));
  skity_cuda_image_shader is;
  std::memset(&is, 0, sizeof is);
  is.image = image;
  is.filter = filter;
  is.tile_x = is.tile_y = 3;  // TileMode::kDecal
  is.local_matrix[0] = local.e[0][0];
  is.local_matrix[1] = local.e[1][0];
  is.local_matrix[2] = local.e[3][0];
  is.local_matrix[3] = local.e[0][1];
  is.local_matrix[4] = local.e[1][1];
  is.local_matrix[5] = local.e[3][1];
  skity_cuda_paint p;
  if (paint) {
    p = *paint;
  } else {  // Paint()
    std::memset(&p, 0, sizeof p);
    p.blend_mode = 3;
    p.fill_color[3] = p.stroke_color[3] = 1.f;
    p.stroke_width = 1.f;
    p.miter_limit = 4.f;
  }
  p.style = 0;  // work_paint.SetStyle(kFill_Style)
  p.shader = nullptr;
  p.image_shader = &is;
  const uint8_t verbs[5] = {SKITY_CUDA_VERB_MOVE, SKITY_CUDA_VERB_LINE, SKITY_CUDA_VERB_LINE,
                            SKITY_CUDA_VERB_LINE, SKITY_CUDA_VERB_CLOSE};
  const float pts[8] = {dst[0], dst[1], dst[2], dst[1], dst[2], dst[3], dst[0], dst[3]};
  skity_cuda_path path;
  std::memset(&path, 0, sizeof path);
  path.verbs = verbs;
  path.verb_count = 5;
  path.points = pts;
  path.point_count = 4;
  const int32_t rc = skity_cuda_canvas_draw_path(canvas, &path, &p);
  if (rc) return rc;
  skc::ImageShaderRec& ir = canvas->image_shaders.back();
  ir.rect = 1;
  std::memcpy(ir.src, src, 16);
  std::memcpy(ir.dst, dst, 16);
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_save(skity_cuda_canvas canvas) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kSave;
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  canvas->saved.push_back(canvas->st);
  canvas->saved_layer.push_back(0);
  return SKITY_CUDA_SUCCESS;
}

// Canvas::Restore with nothing saved leaves the matrix as it is.  Restoring
// the level a SaveLayer made composites the layer before the next draw.
SKITY_CUDA_API int32_t skity_cuda_canvas_restore(skity_cuda_canvas canvas) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kRestore;
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  if (!canvas->saved.empty()) {
    canvas->st = canvas->saved.back();
    canvas->saved.pop_back();
    const uint32_t layer = canvas->saved_layer.back();
    canvas->saved_layer.pop_back();
    if (layer) {
      canvas->layers[layer - 1].restore = (uint32_t)canvas->paints.size();
      canvas->dirty = true;
    }
  }
  return SKITY_CUDA_SUCCESS;
}

// Canvas::SaveLayer(bounds, paint) (canvas.cc:255-276): empty bounds, or
// bounds the global clip bounds reject (QuickReject, canvas.cc:478-486),
// save no layer -- a Save and an empty clip instead; otherwise a Save, the
// global clip bounds narrowed by the bounds, and a layer whose draws are
// composited at the matching Restore (SWCanvas::OnSaveLayer / OnLayerRestore,
// sw_canvas.cc:441-484, 891-902).
SKITY_CUDA_API int32_t skity_cuda_canvas_save_layer(skity_cuda_canvas canvas, const float bounds[4],
                                                    const skity_cuda_paint* paint) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!bounds || !std::isfinite(bounds[0]) || !std::isfinite(bounds[1]) ||
      !std::isfinite(bounds[2]) || !std::isfinite(bounds[3]))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (paint && paint->blend_mode > 28) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kSaveLayer;
    std::memcpy(op.f, bounds, 16);
    op.CopyPaint(paint);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  // one level of layers; no mask or colour filter on the layer paint
  for (uint32_t l : canvas->saved_layer)
    if (l) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  if (paint && ((paint->blur_style != 0 && paint->blur_radius > 0.f) || paint->color_filter))
    return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  if (!canvas->st.translation()) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  const bool empty = !(bounds[0] < bounds[2] && bounds[1] < bounds[3]);
  bool reject = empty;
  if (!empty) {  // QuickReject: the mapped bounds against the global clip bounds
    const float x0 = bounds[0] + canvas->st.tx(), x1 = bounds[2] + canvas->st.tx();
    const float y0 = bounds[1] + canvas->st.ty(), y1 = bounds[3] + canvas->st.ty();
    const float* c = canvas->st.clip;
    const float l = std::max(c[0], std::min(x0, x1)), r = std::min(c[2], std::max(x0, x1));
    const float t = std::max(c[1], std::min(y0, y1)), b = std::min(c[3], std::max(y0, y1));
    reject = !(l < r && t < b);
  }
  canvas->saved.push_back(canvas->st);
  if (reject) {
    canvas->saved_layer.push_back(0);
    float* c = canvas->st.clip;
    c[0] = c[1] = c[2] = c[3] = 0.f;
    return SKITY_CUDA_SUCCESS;
  }
  skc::LayerRec L;
  std::memset(&L, 0, sizeof L);
  std::memcpy(L.bounds, bounds, sizeof L.bounds);
  L.translate[0] = canvas->st.tx();
  L.translate[1] = canvas->st.ty();
  std::memcpy(L.clip, canvas->st.clip, sizeof L.clip);
  L.start = (uint32_t)canvas->paints.size();
  L.restore = skc::kLayerOpen;
  // the image draw's alpha: Paint::GetAlphaF (paint.cc:96-98)
  L.alpha = paint ? (paint->style == 1 ? paint->stroke_color[3] : paint->fill_color[3]) : 1.f;
  L.alpha = std::min(std::max(L.alpha, 0.f), 1.f);
  L.blend = paint ? paint->blend_mode : 3u;
  canvas->layers.push_back(L);
  canvas->saved_layer.push_back((uint32_t)canvas->layers.size());
  canvas->dirty = true;
  const int32_t rc = skity_cuda_canvas_clip_rect(canvas, bounds[0], bounds[1], bounds[2], bounds[3]);
  // CanvasState::SaveLayer -> PushLayer: a layer state over the total matrix
  canvas->st.world = canvas->st.m;
  canvas->st.own.identity();
  canvas->st.m = skc::MatMul(canvas->st.world, canvas->st.own);
  return rc;
}

// The canvas matrix times another (LayerState::Translate / Scale / Rotate
// / Skew / Concat, canvas_state.cc:18-42: CurrentMatrix() * m through
// Matrix::operator*, matrix.cc:452-460), or recorded as an op of a display
// list.
static int32_t CanvasConcat(skity_cuda_canvas canvas, skc::RecordedOp::Type type,
                            const float* args, int nargs, const skc::Mat4& m) {
  for (int i = 0; i < nargs; ++i)
    if (!std::isfinite(args[i])) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = type;
    std::memcpy(op.f, args, sizeof(float) * nargs);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  canvas->st.set_own(skc::MatMul(canvas->st.own, m));
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_translate(skity_cuda_canvas canvas, float dx, float dy) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  const float a[2] = {dx, dy};
  return CanvasConcat(canvas, skc::RecordedOp::kTranslate, a, 2, skc::MatTranslate(dx, dy));
}

SKITY_CUDA_API int32_t skity_cuda_canvas_scale(skity_cuda_canvas canvas, float sx, float sy) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  const float a[2] = {sx, sy};
  return CanvasConcat(canvas, skc::RecordedOp::kScale, a, 2, skc::MatScale(sx, sy));
}

SKITY_CUDA_API int32_t skity_cuda_canvas_rotate(skity_cuda_canvas canvas, float degrees, float px,
                                                float py) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  const float a[3] = {degrees, px, py};
  for (float v : a)
    if (!std::isfinite(v)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  return CanvasConcat(canvas, skc::RecordedOp::kRotate, a, 3, skc::MatRotateDeg(degrees, px, py));
}

SKITY_CUDA_API int32_t skity_cuda_canvas_skew(skity_cuda_canvas canvas, float sx, float sy) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  const float a[2] = {sx, sy};
  return CanvasConcat(canvas, skc::RecordedOp::kSkew, a, 2, skc::MatSkew(sx, sy));
}

SKITY_CUDA_API int32_t skity_cuda_canvas_concat(skity_cuda_canvas canvas, const float m[9]) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!m) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  for (int i = 0; i < 9; ++i)
    if (!std::isfinite(m[i])) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  return CanvasConcat(canvas, skc::RecordedOp::kConcat, m, 9, skc::MatFrom9(m));
}

// Canvas::SetMatrix (LayerState::SetMatrix: the matrix replaces the current one).
SKITY_CUDA_API int32_t skity_cuda_canvas_set_matrix(skity_cuda_canvas canvas, const float m[9]) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!m) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  for (int i = 0; i < 9; ++i)
    if (!std::isfinite(m[i])) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kSetMatrix;
    std::memcpy(op.f, m, sizeof(float) * 9);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  canvas->st.set_own(skc::MatFrom9(m));
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_concat44(skity_cuda_canvas canvas, const float m[16]) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!m) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(m[i])) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  return CanvasConcat(canvas, skc::RecordedOp::kConcat44, m, 16, skc::MatFrom16(m));
}

SKITY_CUDA_API int32_t skity_cuda_canvas_set_matrix44(skity_cuda_canvas canvas, const float m[16]) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!m) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  for (int i = 0; i < 16; ++i)
    if (!std::isfinite(m[i])) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kSetMatrix44;
    std::memcpy(op.f, m, sizeof(float) * 16);
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  canvas->st.set_own(skc::MatFrom16(m));
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_get_matrix(skity_cuda_canvas canvas, float m[9]) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!m) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  const skc::Mat4& a = canvas->st.m;  // Matrix::Get9 (matrix.cc:106-116)
  const float v[9] = {a.e[0][0], a.e[1][0], a.e[3][0], a.e[0][1], a.e[1][1],
                      a.e[3][1], a.e[0][3], a.e[1][3], a.e[3][3]};
  std::memcpy(m, v, sizeof v);
  return SKITY_CUDA_SUCCESS;
}

// Canvas::ClipPath(path, op) (canvas.cc:157-162; SWCanvas::OnClipPath,
// sw_canvas.cc:317-336): a new path-clip state on top of the current one,
// recorded with the canvas translation and the global clip bounds, which a
// kIntersect clip first narrows by the path's bounds (Path::GetBounds,
// path.cc:1341-1360).
SKITY_CUDA_API int32_t skity_cuda_canvas_clip_path(skity_cuda_canvas canvas,
                                                   const skity_cuda_path* path, uint32_t op) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!path || op > 1 || (path->verb_count && !path->verbs) ||
      (path->point_count && !path->points) || (path->conic_weight_count && !path->conic_weights))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  uint32_t need_p = 0, need_w = 0;
  for (uint32_t i = 0; i < path->verb_count; ++i) {
    switch (path->verbs[i]) {
      case SKITY_CUDA_VERB_MOVE: case SKITY_CUDA_VERB_LINE: need_p += 1; break;
      case SKITY_CUDA_VERB_QUAD: need_p += 2; break;
      case SKITY_CUDA_VERB_CONIC: need_p += 2; need_w += 1; break;
      case SKITY_CUDA_VERB_CUBIC: need_p += 3; break;
      case SKITY_CUDA_VERB_CLOSE: break;
      default: return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
    }
  }
  if (need_p != path->point_count || need_w != path->conic_weight_count)
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (!skc::ValidPath(path->verbs, path->verb_count, path->points, path->point_count,
                      path->conic_weights, path->conic_weight_count))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp rop;
    rop.type = skc::RecordedOp::kClipPath;
    rop.CopyPath(path);
    rop.u = op;
    canvas->ops.push_back(std::move(rop));
    return SKITY_CUDA_SUCCESS;
  }
  // the path under the canvas matrix (any affine map), as RastePath takes
  // CurrentTransform() (sw_canvas.cc:317-324)
  if (!canvas->st.affine()) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  float m6[6];
  canvas->st.six(m6);
  if (!canvas->st.translation()) {
    if (!skc::ValidMatrix(m6, path->points, path->point_count))
      return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  } else {
    float t[2] = {m6[2], m6[5]};
    if (!skc::ValidTranslate(t, path->points, path->point_count))
      return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  }
  if (op == 1) {
    // Canvas::ClipPath narrows the global clip bounds by the path's bounds
    // (canvas.cc:159-164): its points but a trailing move
    uint32_t n = path->point_count;
    if (path->verb_count > 1 && path->verbs[path->verb_count - 1] == SKITY_CUDA_VERB_MOVE) n--;
    float l = 0.f, tp = 0.f, r = 0.f, b = 0.f;
    for (uint32_t i = 0; i < n; ++i) {
      const float x = path->points[2 * i], y = path->points[2 * i + 1];
      if (i == 0) {
        l = r = x;
        tp = b = y;
      } else {
        l = std::min(l, x);
        r = std::max(r, x);
        tp = std::min(tp, y);
        b = std::max(b, y);
      }
    }
    NarrowClipBounds(canvas, l, tp, r, b);
  }
  AddClipState(canvas, path->verbs, path->verb_count, path->points, path->point_count,
               path->conic_weights, path->conic_weight_count, op, path->fill_type ? 1u : 0u);
  return SKITY_CUDA_SUCCESS;
}

// Canvas::ClipRect (canvas.cc:130-150): the global clip bounds narrowed by
// the mapped rect (Canvas::CalculateGlobalClipBounds, canvas.cc:463-476;
// Matrix::MapRect, matrix.cc:306-337: the corners mapped, w = 1, their min
// and max); under a rotation or skew SWCanvas::OnClipRect then clips by the
// rect as a path (Path::AddRect, sw_canvas.cc:297-313, canvas.cc:144-150).
SKITY_CUDA_API int32_t skity_cuda_canvas_clip_rect(skity_cuda_canvas canvas, float left, float top,
                                                   float right, float bottom) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!std::isfinite(left) || !std::isfinite(top) || !std::isfinite(right) ||
      !std::isfinite(bottom))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (canvas->recording) {
    skc::RecordedOp op;
    op.type = skc::RecordedOp::kClipRect;
    op.f[0] = left;
    op.f[1] = top;
    op.f[2] = right;
    op.f[3] = bottom;
    canvas->ops.push_back(std::move(op));
    return SKITY_CUDA_SUCCESS;
  }
  if (!canvas->st.affine()) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  const float pts[8] = {left, top, right, top, right, bottom, left, bottom};
  if (!canvas->st.scale_translate()) {
    float m6[6];
    canvas->st.six(m6);
    if (!skc::ValidMatrix(m6, pts, 4)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  }
  NarrowClipBounds(canvas, left, top, right, bottom);
  if (!canvas->st.scale_translate()) {
    static const uint8_t kRectVerbs[5] = {SKITY_CUDA_VERB_MOVE, SKITY_CUDA_VERB_LINE,
                                          SKITY_CUDA_VERB_LINE, SKITY_CUDA_VERB_LINE,
                                          SKITY_CUDA_VERB_CLOSE};
    AddClipState(canvas, kRectVerbs, 5, pts, 4, nullptr, 0, 1u /* kIntersect */, 0u);
  }
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_canvas_flush(skity_cuda_canvas canvas) {
  if (!canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (canvas->recording || !canvas->ctx) return SKITY_CUDA_SUCCESS;  // a recorder draws nothing
  if (!canvas->dirty) return SKITY_CUDA_SUCCESS;  // OnFlush with nothing recorded
  // a layer still open holds draws the bitmap does not show yet; this
  // canvas does not carry them across a flush
  for (uint32_t l : canvas->saved_layer)
    if (l) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  skity_cuda_context ctx = canvas->ctx;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->device);
  auto t0 = std::chrono::steady_clock::now();
  // the recorded draws as one stream view
  skc::StreamView sv;
  std::memset(&sv, 0, sizeof sv);
  sv.width = canvas->width;
  sv.height = canvas->height;
  sv.has_clear = canvas->has_clear ? 1 : 0;
  std::memcpy(sv.clear, canvas->clear, 16);
  sv.nd = (uint32_t)canvas->paints.size();
  sv.vo = canvas->vo.data();
  sv.po = canvas->po.data();
  sv.wo = canvas->wo.data();
  sv.verbs = canvas->verbs.data();
  sv.pts = canvas->pts.data();
  sv.wts = canvas->wts.data();
  sv.paints = canvas->paints.data();
  sv.grads = canvas->grads.data();
  sv.stop_colors = canvas->stop_colors.data();
  sv.stop_offsets = canvas->stop_offsets.data();
  sv.clips = canvas->any_clip ? canvas->clips.data() : nullptr;
  sv.filters = canvas->any_filter ? canvas->filters.data() : nullptr;
  if (!canvas->clip_states.empty()) {
    sv.n_clip_states = (uint32_t)canvas->clip_states.size();
    sv.clip_states = canvas->clip_states.data();
    sv.clip_verbs = canvas->clip_verbs.data();
    sv.clip_pts = canvas->clip_pts.data();
    sv.clip_wts = canvas->clip_wts.data();
    sv.draw_clip_state = canvas->draw_clip_state.data();
    if (canvas->any_clip_matrix) sv.clip_matrices = canvas->clip_matrices.data();
  }
  if (!canvas->images.empty()) {
    sv.n_images = (uint32_t)canvas->images.size();
    sv.images = canvas->images.data();
    sv.image_pixels = canvas->image_blob.data();
    sv.image_bytes = canvas->image_blob.size();
    sv.image_shaders = canvas->image_shaders.data();
  }
  if (!canvas->layers.empty()) {
    sv.n_layers = (uint32_t)canvas->layers.size();
    sv.layers = canvas->layers.data();
  }
  sv.matrices = canvas->any_matrix ? canvas->matrices.data() : nullptr;
  skc::DeviceBatch& db = canvas->db;
  db.hb = skc::HostBatch();
  int32_t rc = skc::AddStreamCanvas(db.hb, sv);
  if (rc) return rc;
  rc = skc::UploadBatch(ctx, db);
  if (rc) return rc;
  const skc::CanvasDesc& cd = db.hb.canvases[db.hb.main_canvases[0]];
  db.keep_pixels = !canvas->has_clear;
  if (!canvas->has_clear) {
    // draws blend over the bitmap's current pixels
    cudaError_t e = cudaMemcpy2DAsync(db.pixels.as<uint8_t>() + cd.px_off, (size_t)cd.w * 4,
                                      canvas->pixels, canvas->row_bytes, (size_t)cd.w * 4, cd.h,
                                      cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return skc::CudaErr(e);
  }
  rc = skc::RenderBatch(ctx, db, true);
  if (rc) return rc;
  rc = skc::ReadCanvas(ctx, db, 0, canvas->pixels, canvas->row_bytes);
  if (rc) return rc;
  db.stats.total_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  ctx->last = db.stats;
  // the bitmap now holds the result; later draws blend over it
  canvas->has_clear = false;
  canvas->verbs.clear();
  canvas->pts.clear();
  canvas->wts.clear();
  canvas->vo.assign(1, 0);
  canvas->po.assign(1, 0);
  canvas->wo.assign(1, 0);
  canvas->paints.clear();
  canvas->grads.clear();
  canvas->stop_colors.clear();
  canvas->stop_offsets.clear();
  canvas->clips.clear();
  canvas->any_clip = false;
  canvas->filters.clear();
  canvas->any_filter = false;
  canvas->matrices.clear();
  canvas->any_matrix = false;
  canvas->draw_clip_state.clear();
  canvas->images.clear();
  canvas->image_blob.clear();
  canvas->image_shaders.clear();
  canvas->layers.clear();
  canvas->dirty = false;
  return SKITY_CUDA_SUCCESS;
}


// ---------------------------------------------------------------------------
// PictureRecorder / DisplayList (src/recorder/picture_recorder.cc,
// display_list.cc; C API module/capi/include/skity_c/skity_recorder.h)
// ---------------------------------------------------------------------------
SKITY_CUDA_API int32_t skity_cuda_recorder_begin(uint32_t width, uint32_t height,
                                                 skity_cuda_canvas* out) {
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  *out = nullptr;
  if (width == 0 || height == 0) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (width > 65535 || height > 65535) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  auto* c = new (std::nothrow) skity_cuda_canvas_s();
  if (!c) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  c->ctx = nullptr;
  c->recording = true;
  c->width = width;
  c->height = height;
  c->pixels = nullptr;
  c->row_bytes = (size_t)width * 4;
  *out = c;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API int32_t skity_cuda_recorder_finish(skity_cuda_canvas recorder,
                                                  skity_cuda_display_list* out) {
  if (!recorder || !recorder->recording) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!out) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  auto* dl = new (std::nothrow) skity_cuda_display_list_s();
  if (!dl) return SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY;
  dl->width = recorder->width;
  dl->height = recorder->height;
  dl->ops.swap(recorder->ops);
  *out = dl;
  return SKITY_CUDA_SUCCESS;
}

SKITY_CUDA_API void skity_cuda_display_list_destroy(skity_cuda_display_list list) { delete list; }

SKITY_CUDA_API uint32_t skity_cuda_display_list_op_count(skity_cuda_display_list list) {
  return list ? (uint32_t)list->ops.size() : 0u;
}

// DisplayList::Draw (display_list.cc:330-343, ReplayRecordedOp :69-): every
// op replayed, in order, through the canvas's own calls -- so the canvas's
// current matrix and clips apply, and a recorder's canvas records them again.
SKITY_CUDA_API int32_t skity_cuda_display_list_draw(skity_cuda_display_list list,
                                                    skity_cuda_canvas canvas) {
  if (!list || !canvas) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  int32_t first_error = SKITY_CUDA_SUCCESS;
  for (const skc::RecordedOp& op : list->ops) {
    int32_t rc = SKITY_CUDA_SUCCESS;
    skity_cuda_paint q{};
    skity_cuda_gradient g{};
    skity_cuda_image_shader is{};
    skity_cuda_image im{};
    if (op.has_paint) op.PaintView(&q, &g, &is, &im);
    switch (op.type) {
      case skc::RecordedOp::kClear:
        rc = skity_cuda_canvas_clear(canvas, op.f);
        break;
      case skc::RecordedOp::kDrawPath: {
        const skity_cuda_path p = op.PathView();
        rc = skity_cuda_canvas_draw_path(canvas, &p, &q);
      } break;
      case skc::RecordedOp::kDrawImageRect: {
        const skity_cuda_image img = op.ImageView();
        rc = skity_cuda_canvas_draw_image_rect(canvas, &img, op.f, op.f + 4, op.u,
                                               op.has_paint ? &q : nullptr);
      } break;
      case skc::RecordedOp::kSave:
        rc = skity_cuda_canvas_save(canvas);
        break;
      case skc::RecordedOp::kRestore:
        rc = skity_cuda_canvas_restore(canvas);
        break;
      case skc::RecordedOp::kSaveLayer:
        rc = skity_cuda_canvas_save_layer(canvas, op.f, op.has_paint ? &q : nullptr);
        break;
      case skc::RecordedOp::kTranslate:
        rc = skity_cuda_canvas_translate(canvas, op.f[0], op.f[1]);
        break;
      case skc::RecordedOp::kScale:
        rc = skity_cuda_canvas_scale(canvas, op.f[0], op.f[1]);
        break;
      case skc::RecordedOp::kRotate:
        rc = skity_cuda_canvas_rotate(canvas, op.f[0], op.f[1], op.f[2]);
        break;
      case skc::RecordedOp::kSkew:
        rc = skity_cuda_canvas_skew(canvas, op.f[0], op.f[1]);
        break;
      case skc::RecordedOp::kConcat:
        rc = skity_cuda_canvas_concat(canvas, op.f);
        break;
      case skc::RecordedOp::kSetMatrix:
        rc = skity_cuda_canvas_set_matrix(canvas, op.f);
        break;
      case skc::RecordedOp::kConcat44:
        rc = skity_cuda_canvas_concat44(canvas, op.f);
        break;
      case skc::RecordedOp::kSetMatrix44:
        rc = skity_cuda_canvas_set_matrix44(canvas, op.f);
        break;
      case skc::RecordedOp::kClipRect:
        rc = skity_cuda_canvas_clip_rect(canvas, op.f[0], op.f[1], op.f[2], op.f[3]);
        break;
      case skc::RecordedOp::kClipPath: {
        const skity_cuda_path p = op.PathView();
        rc = skity_cuda_canvas_clip_path(canvas, &p, op.u);
      } break;
    }
    if (rc != SKITY_CUDA_SUCCESS && first_error == SKITY_CUDA_SUCCESS) first_error = rc;
  }
  return first_error;
}

}  // extern "C"

namespace {

template <typename T>
void Put(std::vector<uint8_t>& out, const T* p, size_t n) {
  const uint8_t* b = (const uint8_t*)p;
  out.insert(out.end(), b, b + n * sizeof(T));
}
void Pad4(std::vector<uint8_t>& out, size_t n) { out.insert(out.end(), (4 - n % 4) % 4, 0); }

// The recorded scene of a canvas as a scene stream (the layout ParseStream
// reads; skity_gb300/scene.py writes the same).
void SerializeCanvas(const skity_cuda_canvas_s& c, std::vector<uint8_t>& out) {
  const uint32_t nd = (uint32_t)c.paints.size();
  const uint32_t flags = (c.any_clip ? 1u : 0u) | (c.any_filter ? 2u : 0u) |
                         (!c.clip_states.empty() ? 4u : 0u) | (!c.images.empty() ? 8u : 0u) |
                         (!c.layers.empty() ? 16u : 0u) | (c.any_matrix ? 32u : 0u) |
                         (!c.clip_states.empty() && c.any_clip_matrix ? 64u : 0u);
  out.clear();
  out.insert(out.end(), {'S', 'K', 'S', 'C'});
  const uint32_t hdr[7] = {1u, c.width, c.height, c.has_clear ? 1u : 0u, flags, 0u, 0u};
  Put(out, hdr, 7);
  Put(out, c.clear, 4);
  const uint32_t cnt[6] = {nd, (uint32_t)c.verbs.size(), (uint32_t)(c.pts.size() / 2),
                           (uint32_t)c.wts.size(), (uint32_t)c.grads.size(),
                           (uint32_t)c.stop_offsets.size()};
  Put(out, cnt, 6);
  Put(out, c.vo.data(), c.vo.size());
  Put(out, c.po.data(), c.po.size());
  Put(out, c.wo.data(), c.wo.size());
  Put(out, c.verbs.data(), c.verbs.size());
  Pad4(out, c.verbs.size());
  Put(out, c.pts.data(), c.pts.size());
  Put(out, c.wts.data(), c.wts.size());
  if (flags & 32) {  // the translations are in the matrix records
    for (skc::PaintRec pr : c.paints) {
      pr.translate[0] = pr.translate[1] = 0.f;
      Put(out, &pr, 1);
    }
  } else {
    Put(out, c.paints.data(), c.paints.size());
  }
  Put(out, c.grads.data(), c.grads.size());
  Put(out, c.stop_colors.data(), c.stop_colors.size());
  Put(out, c.stop_offsets.data(), c.stop_offsets.size());
  if (flags & 1) Put(out, c.clips.data(), c.clips.size());
  if (flags & 2) Put(out, c.filters.data(), c.filters.size());
  if (flags & 4) {
    const uint32_t n = (uint32_t)c.clip_states.size();
    Put(out, &n, 1);
    if (flags & 64) {  // the translations are in the matrix records
      for (skc::ClipStateRec r : c.clip_states) {
        r.translate[0] = r.translate[1] = 0.f;
        Put(out, &r, 1);
      }
    } else {
      Put(out, c.clip_states.data(), c.clip_states.size());
    }
    Put(out, c.clip_verbs.data(), c.clip_verbs.size());
    Pad4(out, c.clip_verbs.size());
    Put(out, c.clip_pts.data(), c.clip_pts.size());
    Put(out, c.clip_wts.data(), c.clip_wts.size());
    Put(out, c.draw_clip_state.data(), c.draw_clip_state.size());
  }
  if (flags & 8) {
    const uint32_t n = (uint32_t)c.images.size();
    Put(out, &n, 1);
    Put(out, c.images.data(), c.images.size());
    const uint64_t nb = c.image_blob.size();
    Put(out, &nb, 1);
    Put(out, c.image_blob.data(), c.image_blob.size());
    Pad4(out, c.image_blob.size());
    Put(out, c.image_shaders.data(), c.image_shaders.size());
  }
  if (flags & 16) {
    const uint32_t n = (uint32_t)c.layers.size();
    Put(out, &n, 1);
    Put(out, c.layers.data(), c.layers.size());
  }
  if (flags & 32) Put(out, c.matrices.data(), c.matrices.size());
  if (flags & 64) Put(out, c.clip_matrices.data(), c.clip_matrices.size());
}

}  // namespace

extern "C" {

// The display list as a scene stream: its ops replayed onto a fresh canvas
// of the recording's size, whose recorded scene is written out -- the input
// of skity_cuda_render_streams, skity_cuda_batch_create and
// skity_cuda_server_submit.  out NULL: *size receives the byte count.
SKITY_CUDA_API int32_t skity_cuda_display_list_to_stream(skity_cuda_display_list list, uint8_t* out,
                                                         size_t* size) {
  if (!list) return SKITY_CUDA_ERROR_INVALID_HANDLE;
  if (!size) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  skity_cuda_canvas_s c;
  c.ctx = nullptr;
  c.width = list->width;
  c.height = list->height;
  c.pixels = nullptr;
  c.row_bytes = (size_t)list->width * 4;
  int32_t rc = skity_cuda_display_list_draw(list, &c);
  if (rc) return rc;
  for (uint32_t l : c.saved_layer)
    if (l) return SKITY_CUDA_ERROR_NOT_SUPPORTED;  // a layer left open
  std::vector<uint8_t> bytes;
  SerializeCanvas(c, bytes);
  if (!out) {
    *size = bytes.size();
    return SKITY_CUDA_SUCCESS;
  }
  if (*size < bytes.size()) {
    *size = bytes.size();
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  }
  std::memcpy(out, bytes.data(), bytes.size());
  *size = bytes.size();
  return SKITY_CUDA_SUCCESS;
}

}  // extern "C"
