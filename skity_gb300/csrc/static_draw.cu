// skity_cuda_draw_path_static: one DrawPath with a solid-colour paint onto a
// canvas that already lives in device memory, with every intermediate buffer
// carved out of one fixed, file-scope device array instead of allocations.
//
// Who it is for: callers that must not allocate while they draw -- a render
// loop held to a fixed memory footprint, or a host that cannot afford the
// device-wide synchronisation that freeing device memory implies.  The call
// makes no cudaMalloc / cudaFree and no host heap allocation; the price is a
// hard size limit (kStaticScratchBytes per device), beyond which inputs are
// rejected with SKITY_CUDA_ERROR_SCRATCH_LIMIT.
//
// The work is the batch pipeline's, on the draw's one or two passes:
// k_geometry (path -> quads -> stroke -> edges -> introsort), the sweep
// kernels, then k_static_composite below, which blends each pass's spans
// straight into the caller's canvas rows, in paint order.  Layout of the static scratch:
//
//   [0, 4 KiB)     descriptors: per pass (at most two: fill and stroke)
//                  PassDesc, Brush, PassGeom, PassSweep, PassComp; the
//                  DrawDesc, CanvasDesc, self-check flag, span counts and
//                  span-pool allocator
//   path copy      verbs, points, conic weights of the caller's path
//   geometry       one SliceLayout per pass (capacities grown on overflow)
//   sweep memory   SweepMemLayout(edges, accumulator width) per pass
//   row tables     (first span, count) per row of each pass
//   span pool      whatever is left, shared by the passes
//
// Every pass of the draw is sized and swept before the first one is
// composited: a draw that does not fit, or whose sweep trips a device
// self-check, returns before any pixel of the caller's canvas is written.
//
// One scratch per device, not per call: calls that overlap on one device
// race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include "../../include/skity_cuda.h"
#include "batch.h"

namespace skc {

constexpr uint64_t kStaticScratchBytes = SKITY_CUDA_STATIC_SCRATCH_BYTES;  // 16 MiB
constexpr uint64_t kDescBytes = 4096;
constexpr int kMaxStaticDevices = 64;

static __device__ __align__(256) uint8_t g_static_scratch[kStaticScratchBytes];

namespace {

struct StaticDesc {  // the descriptor block at the start of the scratch
  // a DrawPath makes at most two passes (fill and stroke, in paint order)
  PassDesc pass[2];
  DrawDesc draw;
  CanvasDesc canvas;
  Brush brush[2];
  PassGeom geom[2];
  PassSweep sweep[2];
  PassComp comp[2];
  uint32_t err;
  uint32_t pass_spans[2];
  uint8_t pass_class[8];
  unsigned long long pass_frags[2];
  unsigned long long span_next;
  uint32_t sweep_retry[3];  // DevBatch::sweep_retry: a count, then at most two passes
};
static_assert(sizeof(StaticDesc) <= kDescBytes, "descriptor block");
static_assert(sizeof(P) == 8, "points are copied as float pairs");

// Device address of the scratch, looked up once per device.
std::atomic<uint8_t*> g_scratch_addr[kMaxStaticDevices];
std::mutex g_setup_mu;

int32_t ScratchFor(int device, uint8_t** out) {
  uint8_t* p = g_scratch_addr[device].load(std::memory_order_acquire);
  if (p) {
    *out = p;
    return SKITY_CUDA_SUCCESS;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  p = g_scratch_addr[device].load(std::memory_order_relaxed);
  if (!p) {
    // the caller has made `device` current
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_static_scratch);
    if (e != cudaSuccess || !p) return SKITY_CUDA_ERROR_INITIALIZATION_FAILED;
    g_scratch_addr[device].store(p, std::memory_order_release);
  }
  *out = p;
  return SKITY_CUDA_SUCCESS;
}

inline uint64_t Align256(uint64_t v) { return (v + 255) & ~uint64_t(255); }

// Blends the spans of pass `p` row by row into the caller's canvas: one warp
// per canvas row, spans replayed in emission order, each lane owning the
// pixel columns x = lane (mod 32), so every pixel sees its spans in the
// reference's order (the same rule as the batch compositor).
constexpr int kStaticCompWarps = 4;
__global__ void __launch_bounds__(32 * kStaticCompWarps)
    k_static_composite(DevBatch b, uint32_t p, uint8_t* pixels, size_t row_bytes) {
  const int lane = threadIdx.x & 31;
  const PassComp pc = b.comp[p];
  const int y = pc.row0 + (int)(blockIdx.x * kStaticCompWarps + (threadIdx.x >> 5));
  if (y >= pc.row1) return;
  const uint2 rs = b.rowspan[pc.rbase + (y - pc.row0)];
  const uint32_t s0 = rs.x, s1 = rs.x + rs.y;
  if (s0 >= s1) return;
  const Brush br = b.brushes[pc.brush];
  uint32_t* row = (uint32_t*)(pixels + (size_t)y * row_bytes);
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
      uint32_t c = br.solid;
      if (alpha != 255) c = AlphaMulQ(c, alpha);
      for (int x = xs + ((lane - xs) & 31); x < xe; x += 32) {
        row[x] = ARGBtoRGBA(BlendPixel(RGBAtoARGB(row[x]), c, br.blend));
      }
    }
  }
}

int32_t Err(cudaError_t e) {
  if (e == cudaSuccess) return SKITY_CUDA_SUCCESS;
  if (e == cudaErrorMemoryAllocation) return SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
  return SKITY_CUDA_ERROR_DEVICE;
}

// The passes of one DrawPath (one or two, in paint order).  Every pass is
// sized and swept before any of them is composited, so a draw that does not
// fit the scratch, or whose sweep fails its device self-check, leaves the
// caller's canvas untouched.  `pd[i]` arrive with their initial capacities;
// the path copy already sits at `path_off`.
int32_t StaticDraw(uint8_t* base, uint64_t path_off, uint64_t slice_off0, PassDesc* pd,
                   const Brush* br, uint32_t npass, const DrawDesc& dd, const CanvasDesc& cd,
                   uint8_t* pixels, size_t row_bytes, cudaStream_t st) {
  StaticDesc* dev = (StaticDesc*)base;
  DevBatch b;
  std::memset(&b, 0, sizeof b);
  b.verbs = base + path_off;
  b.draws = &dev->draw;
  b.passes = dev->pass;
  b.n_passes = npass;
  b.canvases = &dev->canvas;
  b.geom = dev->geom;
  b.sweep = dev->sweep;
  b.pass_spans = dev->pass_spans;
  b.pass_frags = dev->pass_frags;
  b.err = &dev->err;
  b.comp = dev->comp;
  b.brushes = dev->brush;
  b.pass_class = dev->pass_class;
  b.sweep_retry = dev->sweep_retry;
  b.pixels = pixels;
  b.n_list = npass;
  {
    uint64_t o = path_off + Align256(dd.nv);
    b.pts = (const P*)(base + o);
    o += Align256(8ull * dd.np);
    b.weights = (const float*)(base + o);
  }
  b.scratch = base + slice_off0;

  // geometry of every pass, each in its own slice, growing the capacities
  // while the slices still fit
  PassGeom g[2];
  uint64_t slices_end = slice_off0;
  for (int attempt = 0;; ++attempt) {
    StaticDesc h;
    std::memset(&h, 0, sizeof h);
    uint64_t o = 0;
    for (uint32_t i = 0; i < npass; ++i) {
      SliceLayout L;
      L.compute(pd[i].cap, sizeof(Edge));
      pd[i].slice_off = o;
      o = Align256(o + L.bytes);
      h.pass[i] = pd[i];
      h.brush[i] = br[i];
    }
    slices_end = slice_off0 + o;
    if (slices_end > kStaticScratchBytes) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
    h.draw = dd;
    h.canvas = cd;
    cudaError_t e = cudaMemcpyAsync(dev, &h, sizeof h, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return Err(e);
    LaunchGeometry(b, st);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(g, dev->geom, sizeof(PassGeom) * npass, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return Err(e);
    bool grown = false;
    for (uint32_t i = 0; i < npass; ++i) {
      if (!g[i].status) continue;
      GrowCaps(pd[i], g[i]);
      grown = true;
    }
    if (!grown) break;
    if (attempt == 7) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  }

  // sweep memory and row tables of every pass after the slices, then one
  // span pool (the rest of the scratch) shared by the passes
  PassSweep sw[2];
  PassComp pc[2];
  std::memset(sw, 0, sizeof sw);
  std::memset(pc, 0, sizeof pc);
  uint64_t sweep_total = 0, rows_total = 0;
  uint32_t chunk_max = 0;
  bool any = false;
  for (uint32_t i = 0; i < npass; ++i) {
    const int nrows = g[i].row1 - g[i].row0;
    pc[i].brush = i;
    if (g[i].n_edges <= 0 || nrows <= 0) continue;  // nothing to sweep or composite
    any = true;
    sw[i].work_off = sweep_total;
    sw[i].bytes = Align256(SweepMemBytes(g[i].n_edges, g[i].acc_width > 0 ? g[i].acc_width : 0));
    sw[i].rbase = (uint32_t)rows_total;
    sw[i].chunk = SpanChunk(cd.w, g[i].n_edges);
    chunk_max = std::max(chunk_max, sw[i].chunk);
    sweep_total += sw[i].bytes;
    rows_total += (uint64_t)nrows;
    pc[i].row0 = g[i].row0;
    pc[i].row1 = g[i].row1;
    pc[i].rbase = sw[i].rbase;
  }
  if (!any) return SKITY_CUDA_SUCCESS;
  const uint64_t sweep_off = Align256(slices_end);
  const uint64_t rows_off = Align256(sweep_off + sweep_total);
  const uint64_t spans_off = Align256(rows_off + sizeof(uint2) * rows_total);
  if (spans_off > kStaticScratchBytes) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  const uint64_t span_cap = (kStaticScratchBytes - spans_off) / sizeof(uint2);
  if (chunk_max > span_cap) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  int32_t max_acc = 0;
  for (uint32_t i = 0; i < npass; ++i) max_acc = std::max(max_acc, g[i].acc_width > 0 ? g[i].acc_width : 0);
  b.sweepmem = base + sweep_off;
  b.reg_diff_cap = std::max<int32_t>(4, std::min<int32_t>((max_acc + 1 + 3) & ~3, kRegDiffMax));
  b.rowspan = (uint2*)(base + rows_off);
  b.spans = (uint2*)(base + spans_off);
  b.span_cap = span_cap;
  b.span_next = &dev->span_next;

  cudaError_t e = cudaMemcpyAsync(dev->sweep, sw, sizeof(PassSweep) * npass,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dev->comp, pc, sizeof(PassComp) * npass, cudaMemcpyHostToDevice, st);
  // empty rows read as (0, 0); the flag, the sweep forms and the pool
  // allocator start clear
  if (e == cudaSuccess) e = cudaMemsetAsync(b.rowspan, 0, sizeof(uint2) * rows_total, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(&dev->err, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dev->pass_class, 0, sizeof dev->pass_class, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(&dev->span_next, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(dev->sweep_retry, 0, sizeof dev->sweep_retry, st);
  if (e != cudaSuccess) return Err(e);
  LaunchSweep(b, st);
  // the sweeps' self-check word and pool use, both read before any pixel is
  // written
  struct {
    uint32_t err;
    unsigned long long used;
  } chk = {0, 0};
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&chk.used, &dev->span_next, sizeof chk.used, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&chk.err, &dev->err, sizeof chk.err, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return Err(e);
  if (chk.err) return SKITY_CUDA_ERROR_DEVICE;
  if (chk.used > span_cap) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  for (uint32_t i = 0; i < npass; ++i) {
    const int nrows = pc[i].row1 - pc[i].row0;
    if (nrows <= 0) continue;
    const unsigned grid = (unsigned)((nrows + kStaticCompWarps - 1) / kStaticCompWarps);
    k_static_composite<<<grid, 32 * kStaticCompWarps, 0, st>>>(b, i, pixels, row_bytes);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return Err(e);
}

int32_t DrawStatic(uint8_t* base, uint8_t* pixels, uint32_t width, uint32_t height,
                   size_t row_bytes, const skity_cuda_path* path, const skity_cuda_paint* paint,
                   cudaStream_t st) {
  const uint32_t nv = path->verb_count, np = path->point_count, nw = path->conic_weight_count;
  if (nv == 0) return SKITY_CUDA_SUCCESS;
  // path copy
  const uint64_t path_off = kDescBytes;
  const uint64_t path_bytes = Align256(nv) + Align256(8ull * np) + Align256(4ull * nw);
  const uint64_t slice_off0 = Align256(path_off + path_bytes);
  if (slice_off0 > kStaticScratchBytes) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  cudaError_t e = cudaMemcpyAsync(base + path_off, path->verbs, nv, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && np)
    e = cudaMemcpyAsync(base + path_off + Align256(nv), path->points, 8ull * np,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && nw)
    e = cudaMemcpyAsync(base + path_off + Align256(nv) + Align256(8ull * np), path->conic_weights,
                        4ull * nw, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return Err(e);

  DrawDesc dd;
  dd.v0 = 0;
  dd.nv = nv;
  dd.p0 = 0;
  dd.np = np;
  dd.w0 = 0;
  dd.nw = nw;
  CanvasDesc cd;
  std::memset(&cd, 0, sizeof cd);
  cd.w = width;
  cd.h = height;
  // The passes of one DrawPath in Paint::Style order with solid brushes, as
  // the batch builder makes them (AddDrawPasses; paint_order.hpp:12-31,
  // SWCanvas::GenerateBrush sw_canvas.cc:727-795 for a paint without shader).
  PassDesc pd[2];
  Brush br[2];
  uint32_t npass = 0;
  auto pass = [&](bool stroke) {
    PassDesc& q = pd[npass];
    std::memset(&q, 0, sizeof q);
    q.flags = (stroke ? kPassStroke : 0) | ((!stroke && path->fill_type != 0) ? kPassEvenOdd : 0) |
              (paint->blend_mode == 3 ? kPassSrcOver : 0);
    q.cap_join = (paint->cap & 0xFF) | ((paint->join & 0xFF) << 8);
    q.stroke_width = paint->stroke_width;
    q.miter = paint->miter_limit;
    q.brush = npass;
    InitialCaps(path->verbs, nv, path->points, stroke, q.cap);
    DerivedCaps(q.cap, stroke);
    Brush& r = br[npass];
    std::memset(&r, 0, sizeof r);
    r.kind = 0;
    r.blend = paint->blend_mode;
    r.global_alpha = 255;
    r.solid = SolidPM(stroke ? paint->stroke_color : paint->fill_color);
    q.ga = r.global_alpha;
    npass++;
  };
  const uint32_t style = paint->style;
  const bool need_fill = style != 1, need_stroke = style != 0;
  if (style == 3) {
    if (need_stroke) pass(true);
    if (need_fill) pass(false);
  } else {
    if (need_fill) pass(false);
    if (need_stroke) pass(true);
  }
  return StaticDraw(base, path_off, slice_off0, pd, br, npass, dd, cd, pixels, row_bytes, st);
}

}  // namespace
}  // namespace skc

extern "C" SKITY_CUDA_API int32_t skity_cuda_draw_path_static(
    int32_t device, uint8_t* device_pixels, uint32_t width, uint32_t height, size_t row_bytes,
    const skity_cuda_path* path, const skity_cuda_paint* paint, void* stream) {
  using namespace skc;
  if (device < 0 || device >= kMaxStaticDevices) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (!device_pixels || !path || !paint || width == 0 || height == 0)
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (width > 65535 || height > 65535) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  if (row_bytes == 0) row_bytes = (size_t)width * 4;
  if (row_bytes < (size_t)width * 4 || (row_bytes & 3) || ((uintptr_t)device_pixels & 3))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if ((path->verb_count && !path->verbs) || (path->point_count && !path->points) ||
      (path->conic_weight_count && !path->conic_weights))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (!ValidPath(path->verbs, path->verb_count, path->points, path->point_count,
                 path->conic_weights, path->conic_weight_count))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (!ValidPaint(paint->style, paint->cap, paint->join, paint->stroke_width,
                  paint->miter_limit, 0.f))
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  if (paint->blend_mode > 28) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  // solid colours only: no shader, no mask filter (MakeBlur(r <= 0) is null)
  if (paint->shader || paint->color_filter || paint->image_shader ||
      (paint->blur_style != 0 && paint->blur_radius > 0.f))
    return SKITY_CUDA_ERROR_NOT_SUPPORTED;

  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess) return SKITY_CUDA_ERROR_DEVICE;
  if (prev != device && cudaSetDevice(device) != cudaSuccess)
    return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
  uint8_t* base = nullptr;
  int32_t rc = ScratchFor(device, &base);
  if (rc == SKITY_CUDA_SUCCESS)
    rc = DrawStatic(base, device_pixels, width, height, row_bytes, path, paint,
                    (cudaStream_t)stream);
  if (prev != device) cudaSetDevice(prev);
  return rc;
}
