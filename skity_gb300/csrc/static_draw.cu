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
// The work per rasterisation pass is the batch pipeline's, on one pass:
// k_geometry (path -> quads -> stroke -> edges -> introsort), the sweep
// kernels, then k_static_composite below, which blends the pass's spans
// straight into the caller's canvas rows.  Layout of the static scratch:
//
//   [0, 4 KiB)     descriptors: PassDesc, DrawDesc, CanvasDesc, Brush,
//                  PassGeom, PassSweep, PassComp, self-check flag, span
//                  count, span-pool allocator
//   path copy      verbs, points, conic weights of the caller's path
//   geometry       SliceLayout of the pass (capacities grown on overflow)
//   sweep memory   SweepMemLayout(edges, accumulator width)
//   row table      (first span, count) per row
//   span pool      whatever is left
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
  PassDesc pass;
  DrawDesc draw;
  CanvasDesc canvas;
  Brush brush;
  PassGeom geom;
  PassSweep sweep;
  PassComp comp;
  uint32_t err;
  uint32_t pass_spans[2];
  uint32_t pass_class;
  uint32_t pad;
  unsigned long long span_next;
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

// Blends the spans of the pass row by row into the caller's canvas: one warp
// per canvas row, spans replayed in emission order, each lane owning the
// pixel columns x = lane (mod 32), so every pixel sees its spans in the
// reference's order (the same rule as the batch compositor).
constexpr int kStaticCompWarps = 4;
__global__ void __launch_bounds__(32 * kStaticCompWarps)
    k_static_composite(DevBatch b, uint8_t* pixels, size_t row_bytes) {
  const int lane = threadIdx.x & 31;
  const PassComp pc = b.comp[0];
  const int y = pc.row0 + (int)(blockIdx.x * kStaticCompWarps + (threadIdx.x >> 5));
  if (y >= pc.row1) return;
  const uint2 rs = b.rowspan[y - pc.row0];
  const uint32_t s0 = rs.x, s1 = rs.x + rs.y;
  if (s0 >= s1) return;
  const Brush br = b.brushes[0];
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

// One fill or stroke pass.  `pd` arrives with its initial capacities; the
// path copy already sits at `path_off`.
int32_t StaticPass(uint8_t* base, uint64_t path_off, uint64_t slice_off0, PassDesc pd,
                   const DrawDesc& dd, const CanvasDesc& cd, const Brush& br,
                   uint8_t* pixels, size_t row_bytes, cudaStream_t st) {
  StaticDesc* dev = (StaticDesc*)base;
  DevBatch b;
  std::memset(&b, 0, sizeof b);
  b.verbs = base + path_off;
  b.draws = &dev->draw;
  b.passes = &dev->pass;
  b.n_passes = 1;
  b.canvases = &dev->canvas;
  b.geom = &dev->geom;
  b.sweep = &dev->sweep;
  b.pass_spans = dev->pass_spans;
  b.err = &dev->err;
  b.comp = &dev->comp;
  b.brushes = &dev->brush;
  b.pass_class = (uint8_t*)&dev->pass_class;
  b.pixels = pixels;
  b.n_list = 1;
  {
    uint64_t o = path_off + Align256(dd.nv);
    b.pts = (const P*)(base + o);
    o += Align256(8ull * dd.np);
    b.weights = (const float*)(base + o);
  }
  b.scratch = base + slice_off0;

  // geometry, growing the capacities while the slice still fits
  PassGeom g;
  for (int attempt = 0;; ++attempt) {
    SliceLayout L;
    L.compute(pd.cap, sizeof(Edge));
    if (slice_off0 + L.bytes > kStaticScratchBytes) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
    pd.slice_off = 0;
    StaticDesc h;
    std::memset(&h, 0, sizeof h);
    h.pass = pd;
    h.draw = dd;
    h.canvas = cd;
    h.brush = br;
    cudaError_t e = cudaMemcpyAsync(dev, &h, sizeof h, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return Err(e);
    LaunchGeometry(b, st);
    e = cudaMemcpyAsync(&g, &dev->geom, sizeof g, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return Err(e);
    if (!g.status) break;
    if (attempt == 7) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
    GrowCaps(pd, g);
  }
  const int nrows = g.row1 - g.row0;
  if (g.n_edges <= 0 || nrows <= 0) return SKITY_CUDA_SUCCESS;

  // sweep memory, row table and span pool after the slice
  SliceLayout L;
  L.compute(pd.cap, sizeof(Edge));
  const uint64_t sweep_off = Align256(slice_off0 + L.bytes);
  const uint64_t sweep_bytes = SweepMemBytes(g.n_edges, g.acc_width > 0 ? g.acc_width : 0);
  const uint64_t rows_off = Align256(sweep_off + sweep_bytes);
  const uint64_t spans_off = Align256(rows_off + sizeof(uint2) * (uint64_t)nrows);
  if (spans_off > kStaticScratchBytes) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  const uint64_t span_cap = (kStaticScratchBytes - spans_off) / sizeof(uint2);
  const uint32_t chunk = SpanChunk(cd.w, g.n_edges);
  if (chunk > span_cap) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  b.sweepmem = base + sweep_off;
  b.reg_diff_cap = std::max<int32_t>(
      4, std::min<int32_t>(((g.acc_width > 0 ? g.acc_width : 0) + 1 + 3) & ~3, kRegDiffMax));
  b.rowspan = (uint2*)(base + rows_off);
  b.spans = (uint2*)(base + spans_off);
  b.span_cap = span_cap;
  b.span_next = &dev->span_next;

  PassSweep sw;
  std::memset(&sw, 0, sizeof sw);
  sw.work_off = 0;
  sw.bytes = sweep_bytes;
  sw.rbase = 0;
  sw.chunk = chunk;
  PassComp pc;
  std::memset(&pc, 0, sizeof pc);
  pc.row0 = g.row0;
  pc.row1 = g.row1;
  pc.rbase = 0;
  pc.brush = 0;
  cudaError_t e = cudaMemcpyAsync(&dev->sweep, &sw, sizeof sw, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&dev->comp, &pc, sizeof pc, cudaMemcpyHostToDevice, st);
  // empty rows read as (0, 0); the flag, the sweep form and the pool
  // allocator start clear
  if (e == cudaSuccess) e = cudaMemsetAsync(b.rowspan, 0, sizeof(uint2) * (uint64_t)nrows, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(&dev->err, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(&dev->pass_class, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(&dev->span_next, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return Err(e);
  LaunchSweep(b, st);
  unsigned long long used = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&used, &dev->span_next, sizeof used, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return Err(e);
  if (used > span_cap) return SKITY_CUDA_ERROR_SCRATCH_LIMIT;
  unsigned grid = (unsigned)((nrows + kStaticCompWarps - 1) / kStaticCompWarps);
  k_static_composite<<<grid, 32 * kStaticCompWarps, 0, st>>>(b, pixels, row_bytes);
  uint32_t err = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, &dev->err, sizeof err, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return Err(e);
  return err ? SKITY_CUDA_ERROR_DEVICE : SKITY_CUDA_SUCCESS;
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
  auto pass = [&](bool stroke) -> int32_t {
    PassDesc pd;
    std::memset(&pd, 0, sizeof pd);
    pd.flags = (stroke ? kPassStroke : 0) | ((!stroke && path->fill_type != 0) ? kPassEvenOdd : 0) |
               (paint->blend_mode == 3 ? kPassSrcOver : 0);
    pd.cap_join = (paint->cap & 0xFF) | ((paint->join & 0xFF) << 8);
    pd.stroke_width = paint->stroke_width;
    pd.miter = paint->miter_limit;
    InitialCaps(path->verbs, nv, path->points, stroke, pd.cap);
    DerivedCaps(pd.cap, stroke);
    Brush br;
    std::memset(&br, 0, sizeof br);
    br.kind = 0;
    br.blend = paint->blend_mode;
    br.global_alpha = 255;
    br.solid = SolidPM(stroke ? paint->stroke_color : paint->fill_color);
    pd.ga = br.global_alpha;
    return StaticPass(base, path_off, slice_off0, pd, dd, cd, br, pixels, row_bytes, st);
  };
  const uint32_t style = paint->style;
  const bool need_fill = style != 1, need_stroke = style != 0;
  int32_t rc = SKITY_CUDA_SUCCESS;
  if (style == 3) {
    if (need_stroke) rc = pass(true);
    if (rc == SKITY_CUDA_SUCCESS && need_fill) rc = pass(false);
  } else {
    if (need_fill) rc = pass(false);
    if (rc == SKITY_CUDA_SUCCESS && need_stroke) rc = pass(true);
  }
  return rc;
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
  // solid colours only: no shader, no mask filter (MakeBlur(r <= 0) is null)
  if (paint->blend_mode > 28 || paint->shader || paint->color_filter || paint->image_shader ||
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
