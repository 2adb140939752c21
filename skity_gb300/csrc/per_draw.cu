// The plain per-draw form of the pipeline: a resident batch rendered one
// DrawPath at a time, as the reference's software canvas works (each
// SWCanvas::OnDrawPath rasterises and blends its path before the next draw,
// src/render/sw/sw_canvas.cc:357-411).  Per draw, on one stream and with no
// host round trip:
//
//   k_geometry        the draw's passes (fill and / or stroke)
//   k_draw_plan       1 thread: the passes' sweep memory, row tables and
//                     sweep form, the span pool reset
//   k_sweep_*         the sweep forms (each takes the passes of its form)
//   k_draw_composite  1 warp / canvas row: the passes' spans blended in
//                     paint order straight into the canvas
//
// Every draw reuses the same sweep memory, row table and span pool (the
// stream orders the draws).  Capacities come from the host; a draw that
// does not fit is skipped and flagged in the status, and the host grows the
// buffers and renders the batch again -- the only wait on the device is at
// the end.  It is the comparison point of the batched form: the same
// kernels, without batching.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>

#include "device.h"

namespace skc {

#define SKC_TRY_RC(expr)                       \
  do {                                         \
    cudaError_t _e = (expr);                   \
    if (_e != cudaSuccess) return CudaErr(_e); \
  } while (0)

namespace {

struct DrawStatus {  // zeroed before a per-draw render, read back after it
  uint32_t flags;            // kPlanGeomOverflow | kPlanSweepMem | kPlanRows
  uint32_t span_short;       // a draw's spans outgrew the pool
  unsigned long long sweep_need, rows_need, span_need;  // largest draw
  unsigned long long spans, frags;
};

__global__ void k_draw_plan(DevBatch b, uint32_t npass, uint64_t sweep_cap, uint64_t rows_cap,
                            DrawStatus* st) {
  if (threadIdx.x != 0) return;
  unsigned long long off = 0, rb = 0;
  for (uint32_t i = 0; i < npass; ++i) {
    const PassGeom g = b.geom[i];
    const CanvasDesc& cd = b.canvases[b.passes[i].canvas];
    const int nr = g.row1 - g.row0;
    if (g.status) atomicOr(&st->flags, kPlanGeomOverflow);
    bool has = g.status == 0 && g.n_edges > 0 && nr > 0;
    unsigned long long bytes = 0;
    if (has) {
      bytes = (SweepMemBytes(g.n_edges, g.acc_width > 0 ? g.acc_width : 0) + 255ull) & ~255ull;
      if (off + bytes > sweep_cap || rb + (unsigned long long)nr > rows_cap) {
        atomicOr(&st->flags, (off + bytes > sweep_cap ? kPlanSweepMem : 0u) |
                                 (rb + (unsigned long long)nr > rows_cap ? kPlanRows : 0u));
        has = false;
      }
    }
    PassSweep sw;
    sw.work_off = off;
    sw.bytes = has ? bytes : 0ull;
    sw.rbase = (uint32_t)rb;
    sw.chunk = SpanChunk(cd.w, g.n_edges);
    ((PassSweep*)b.sweep)[i] = sw;
    PassComp pc;
    pc.row0 = has ? g.row0 : 0;
    pc.row1 = has ? g.row1 : 0;
    pc.rbase = (uint32_t)rb;
    pc.brush = b.passes[i].brush;
    ((PassComp*)b.comp)[i] = pc;
    b.pass_class[i] = has ? (uint8_t)0 : kSweepSkip;
    if (g.status == 0 && g.n_edges > 0 && nr > 0) {
      off += bytes;
      rb += (unsigned long long)nr;
    }
  }
  atomicMax(&st->sweep_need, off);
  atomicMax(&st->rows_need, rb);
  *b.span_next = 0;
  b.sweep_retry[0] = 0;
}

// One warp per canvas row: the spans of the draw's passes on that row,
// pass after pass (paint order), each span's pixels spread over the lanes
// (x = lane mod 32), so every pixel sees its blends in the reference's order.
constexpr int kDrawCompWarps = 4;
__global__ void __launch_bounds__(32 * kDrawCompWarps)
    k_draw_composite(DevBatch b, uint32_t npass, uint32_t canvas, DrawStatus* st) {
  const int lane = threadIdx.x & 31;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const unsigned long long used = *b.span_next;
    atomicMax(&st->span_need, used);
    if (used > b.span_cap) atomicOr(&st->span_short, 1u);
  }
  if (*b.span_next > b.span_cap) return;  // spans dropped: the host renders again
  const CanvasDesc cd = b.canvases[canvas];
  const int y = (int)(blockIdx.x * kDrawCompWarps + (threadIdx.x >> 5));
  if (y >= (int)cd.h) return;
  uint32_t* row = (uint32_t*)(b.pixels + cd.px_off) + (size_t)y * cd.w;
  for (uint32_t i = 0; i < npass; ++i) {
    const PassComp pc = b.comp[i];
    if (y < pc.row0 || y >= pc.row1) continue;
    const uint2 rs = b.rowspan[pc.rbase + (y - pc.row0)];
    if (!rs.y) continue;
    const Brush br = b.brushes[pc.brush];
    const uint32_t s0 = rs.x, s1 = rs.x + rs.y;
    for (uint32_t sb = s0; sb < s1; sb += 32) {
      uint2 mine = make_uint2(0, 0);
      if (sb + lane < s1) mine = b.spans[sb + lane];
      const int cnt = (int)min(32u, s1 - sb);
      for (int j = 0; j < cnt; ++j) {
        const uint32_t xs_len = __shfl_sync(0xffffffffu, mine.x, j);
        const uint32_t cover = __shfl_sync(0xffffffffu, mine.y, j);
        const int xs = (int)(xs_len & 0xFFFF);
        const int xe = xs + (int)(xs_len >> 16);
        const uint32_t alpha = cover & br.global_alpha;
        for (int x = xs + ((lane - xs) & 31); x < xe; x += 32) {
          uint32_t c = BrushColor(br, x, y, b.stop_colors, b.stop_offsets, b.pixels, b.roundtrip,
                                  b.conicals);
          if (alpha != 255) c = AlphaMulQ(c, alpha);
          if (br.cf_type) c = FilterColor(br, c, b.srgb_tables, b.cf_matrices);
          row[x] = ARGBtoRGBA(BlendPixel(RGBAtoARGB(row[x]), c, br.blend));
        }
      }
      __syncwarp();
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long sp = 0, fr = 0;
    for (uint32_t i = 0; i < npass; ++i)
      if (b.sweep[i].bytes) {
        sp += b.pass_spans[i];
        fr += b.pass_frags[i];
      }
    atomicAdd(&st->spans, sp);
    atomicAdd(&st->frags, fr);
  }
}

__global__ void k_clear_canvas(uint8_t* pixels, uint64_t px_off, uint64_t n, uint32_t value) {
  uint32_t* p = (uint32_t*)(pixels + px_off);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = value;
}

}  // namespace

// Renders every main canvas of the batch one draw at a time (see above);
// pixels stay on the device.
int32_t RenderPerDraw(skity_cuda_context_s* ctx, DeviceBatch& db) {
  HostBatch& hb = db.hb;
  if (!hb.clip_states.empty() || !hb.temp_canvases.empty()) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  cudaStream_t s = ctx->stream;
  const uint32_t np = (uint32_t)hb.passes.size();
  const size_t npm = std::max<size_t>(np, 1);
  skity_cuda_stats st{};
  st.draws = hb.draw_count;
  st.passes = np;
  uint32_t maxw = 1, maxh = 1;
  for (const CanvasDesc& cd : hb.canvases) {
    maxw = std::max(maxw, cd.w);
    maxh = std::max(maxh, cd.h);
  }
  // first capacities: the largest draw's sweep memory estimate, two passes'
  // rows, the context's span pool
  uint64_t cap_sweep = 0;
  for (const PassDesc& pd : hb.passes)
    cap_sweep = std::max<uint64_t>(
        cap_sweep, 2 * ((SweepMemBytes(pd.cap[12], (int)std::min<uint32_t>(hb.canvases[pd.canvas].w, 2048) + 2) + 255) & ~uint64_t(255)));
  uint64_t cap_rows = 2ull * maxh;
  DevBuf status, sweepmem, rowspan;
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (db.slices_dirty) {
      uint64_t total = 0;
      for (uint32_t i = 0; i < np; ++i) {
        SliceLayout L;
        L.compute(hb.passes[i].cap, sizeof(Edge));
        hb.passes[i].slice_off = total;
        total += L.bytes;
      }
      if (ctx->budget && total > ctx->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
      SKC_TRY_RC(db.scratch.ensure(std::max<uint64_t>(total, 16)));
      SKC_TRY_RC(db.passes.ensure(npm * sizeof(PassDesc)));
      if (np)
        SKC_TRY_RC(cudaMemcpyAsync(db.passes.p, hb.passes.data(), np * sizeof(PassDesc),
                                   cudaMemcpyHostToDevice, s));
      db.slices_dirty = false;
    }
    SKC_TRY_RC(db.geom.ensure(npm * sizeof(PassGeom)));
    SKC_TRY_RC(db.sweep.ensure(npm * sizeof(PassSweep)));
    SKC_TRY_RC(db.comp.ensure(npm * sizeof(PassComp)));
    SKC_TRY_RC(db.pass_spans.ensure(npm * 4));
    SKC_TRY_RC(db.pass_frags.ensure(npm * 8));
    SKC_TRY_RC(db.pass_class.ensure(npm));
    SKC_TRY_RC(db.retry.ensure((npm + 1) * 4));
    SKC_TRY_RC(db.err.ensure(16));
    SKC_TRY_RC(status.ensure(sizeof(DrawStatus)));
    SKC_TRY_RC(sweepmem.ensure(std::max<uint64_t>(cap_sweep, 16)));
    SKC_TRY_RC(rowspan.ensure(std::max<uint64_t>(cap_rows, 1) * sizeof(uint2)));
    SKC_TRY_RC(ctx->span_next.ensure(8));
    if (!ctx->span_pool.p) SKC_TRY_RC(ctx->span_pool.ensure((uint64_t)(1 << 20) * sizeof(uint2)));

    DevBatch b;
    std::memset(&b, 0, sizeof b);
    b.verbs = db.verbs.as<uint8_t>();
    b.pts = db.pts.as<P>();
    b.weights = db.weights.as<float>();
    b.draws = db.draws.as<DrawDesc>();
    b.canvases = db.canvases.as<CanvasDesc>();
    b.scratch = db.scratch.as<uint8_t>();
    b.sweepmem = sweepmem.as<uint8_t>();
    b.rowspan = rowspan.as<uint2>();
    b.err = db.err.as<uint32_t>();
    b.sweep_retry = db.retry.as<uint32_t>();  // zeroed by each draw's k_draw_plan
    b.reg_diff_cap = std::max<int32_t>(4, std::min<int32_t>(((int32_t)maxw + 132 + 3) & ~3, kRegDiffMax));
    b.spans = ctx->span_pool.as<uint2>();
    b.span_cap = ctx->span_pool.cap / sizeof(uint2);
    b.span_next = ctx->span_next.as<unsigned long long>();
    b.brushes = db.brushes.as<Brush>();
    b.conicals = db.conicals.as<ConicalParams>();
    b.srgb_tables = db.srgb_tables.as<uint8_t>();
    b.cf_matrices = db.cf_matrices.as<int16_t>();
    b.stop_colors = db.stop_colors.as<float4>();
    b.stop_offsets = db.stop_offsets.as<float>();
    b.pixels = db.pixels.as<uint8_t>();
    b.roundtrip = db.roundtrip.as<uint8_t>();
    DrawStatus* dst = status.as<DrawStatus>();

    uint64_t launches = 0;
    SKC_TRY_RC(cudaEventRecord(ctx->ev0, s));
    SKC_TRY_RC(cudaMemsetAsync(dst, 0, sizeof(DrawStatus), s));
    SKC_TRY_RC(cudaMemsetAsync(b.err, 0, 16, s));
    for (uint32_t c : hb.main_canvases) {
      const CanvasDesc& cd = hb.canvases[c];
      const uint64_t n = (uint64_t)cd.w * cd.h;
      k_clear_canvas<<<(unsigned)std::min<uint64_t>((n + 255) / 256, 4096), 256, 0, s>>>(
          b.pixels, cd.px_off, n, cd.has_clear ? ARGBtoRGBA(cd.clear_pm) : 0u);
      launches++;
      const unsigned rows_grid = (cd.h + kDrawCompWarps - 1) / kDrawCompWarps;
      for (uint32_t p0 = cd.pass0; p0 < cd.pass1;) {
        uint32_t p1 = p0 + 1;
        while (p1 < cd.pass1 && hb.passes[p1].draw == hb.passes[p0].draw) ++p1;
        const uint32_t k = p1 - p0;
        // the draw's passes as a batch of their own
        DevBatch v = b;
        v.passes = db.passes.as<PassDesc>() + p0;
        v.n_passes = k;
        v.n_list = k;
        v.geom = db.geom.as<PassGeom>() + p0;
        v.sweep = db.sweep.as<PassSweep>() + p0;
        v.comp = db.comp.as<PassComp>() + p0;
        v.pass_spans = db.pass_spans.as<uint32_t>() + p0;
        v.pass_frags = db.pass_frags.as<unsigned long long>() + p0;
        v.pass_class = db.pass_class.as<uint8_t>() + p0;
        launches += LaunchGeometry(v, s);
        k_draw_plan<<<1, 32, 0, s>>>(v, k, cap_sweep, cap_rows, dst);
        launches += 1 + LaunchSweep(v, s);
        k_draw_composite<<<rows_grid, 32 * kDrawCompWarps, 0, s>>>(v, k, c, dst);
        launches++;
        p0 = p1;
      }
    }
    SKC_TRY_RC(cudaEventRecord(ctx->ev1, s));
    SKC_TRY_RC(cudaGetLastError());
    DrawStatus hs;
    uint32_t err = 0;
    SKC_TRY_RC(cudaMemcpyAsync(&hs, dst, sizeof hs, cudaMemcpyDeviceToHost, s));
    SKC_TRY_RC(cudaMemcpyAsync(&err, b.err, 4, cudaMemcpyDeviceToHost, s));
    SKC_TRY_RC(cudaStreamSynchronize(s));
    st.host_syncs++;
    if (err) return SKITY_CUDA_ERROR_DEVICE;
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    if (hs.flags == 0 && !hs.span_short) {
      st.device_ms = ms;
      st.spans = hs.spans;
      st.fragments = hs.frags;
      st.kernel_launches = launches;
      for (uint32_t c : hb.main_canvases) st.pixels += (uint64_t)hb.canvases[c].w * hb.canvases[c].h;
      db.stats = st;
      return SKITY_CUDA_SUCCESS;
    }
    st.retries++;
    st.sweep_count_ms += ms;
    if (hs.flags & kPlanGeomOverflow) {
      db.h_geom.resize(np);
      SKC_TRY_RC(cudaMemcpy(db.h_geom.data(), db.geom.p, (size_t)np * sizeof(PassGeom),
                            cudaMemcpyDeviceToHost));
      for (uint32_t p = 0; p < np; ++p)
        if (db.h_geom[p].status) GrowCaps(hb.passes[p], db.h_geom[p]);
      db.slices_dirty = true;
    }
    if (hs.sweep_need > cap_sweep) cap_sweep = hs.sweep_need + hs.sweep_need / 8;
    if (hs.rows_need > cap_rows) cap_rows = hs.rows_need;
    if (hs.span_short) {
      const uint64_t grow = std::min<uint64_t>(hs.span_need + hs.span_need / 16, 0xFFFFFFFFull);
      if (ctx->budget && grow * sizeof(uint2) > ctx->budget) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
      ctx->span_pool.release();
      SKC_TRY_RC(ctx->span_pool.ensure(grow * sizeof(uint2)));
    }
  }
  return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
}

}  // namespace skc
