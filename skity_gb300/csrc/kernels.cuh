// Device-side data layout shared by the kernels (kernels.cu) and the host
// pipeline (pipeline.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "composite.cuh"
#include "raster.cuh"

namespace skc {

// One rasterisation pass (the fill or the stroke of one DrawPath call),
// in draw order within its canvas.
struct PassDesc {
  uint32_t draw;        // index into DrawDesc
  uint32_t canvas;      // index into CanvasDesc
  uint32_t flags;       // kPassStroke | kPassEvenOdd | kPassSrcOver
  uint32_t cap_join;    // Paint::Cap | Paint::Join << 8
  float tx, ty;         // translation of the canvas matrix the path is mapped by
  float stroke_width, miter;
  uint32_t ga;          // brush global alpha (spans with cover & ga == 0 are dropped)
  uint32_t brush;       // index into Brush
  uint64_t slice_off;   // byte offset of this pass's geometry scratch
  int32_t cap[13];      // scratch capacities, see SliceLayout
  uint32_t clipped;     // 1: clip (device-space LTRB) bounds the scan; 0: kMaxCullRect
  float clip[4];
  uint32_t path_clip;   // the path-clip state the draw is under (1-based; 0: none)
  uint32_t pad2;
  float lin[4];         // kPassMatrix: sx, kx, ky, sy of the canvas matrix (tx, ty above)
};
// kPassRawSpans: the sweep stores the raster's spans as they are (any x,
// zero coverage kept; ClipSpanRaw format) for the path-clip stages;
// kPassClipPath: the pass rasterises a ClipPath path (never composited, all
// of its rows kept, on the canvas or not)
enum : uint32_t {
  kPassStroke = 1,
  kPassEvenOdd = 2,
  kPassSrcOver = 4,
  kPassRawSpans = 8,
  kPassClipPath = 16,
  kPassMatrix = 32  // the canvas matrix has a linear part (PassDesc::lin)
};

// The canvas matrix a pass's path is mapped by.
SKC_HD Xform PassXform(const PassDesc& pd) {
  Xform x;
  x.tx = pd.tx;
  x.ty = pd.ty;
  x.lin = (pd.flags & kPassMatrix) != 0;
  x.sx = pd.lin[0];
  x.kx = pd.lin[1];
  x.ky = pd.lin[2];
  x.sy = pd.lin[3];
  return x;
}

// One Canvas::ClipPath call (SWCanvas::OnClipPath, sw_canvas.cc:317-336) on
// top of its parent state; its span rows are computed on the device.
struct ClipStateDesc {
  uint32_t parent;      // 1-based index of the parent state in the batch (0: none)
  uint32_t op;          // Canvas::ClipOp: 0 kDifference, 1 kIntersect
  uint32_t pass;        // the pass rasterising the clip path
  int32_t y0, y1;       // rows of this state's span list (its path's and its parent's)
  uint32_t rbase;       // first entry of its rows in DevBatch::clip_rows
};

struct DrawDesc {  // a Path inside the batch's verb/point/weight arrays
  uint32_t v0, nv, p0, np, w0, nw;
};

struct CanvasDesc {
  uint32_t w, h;
  uint64_t px_off;     // byte offset of RGBA8 rows in the canvas buffer
  uint64_t blur_off;   // temp canvases: byte offset of the blurred copy
  uint32_t has_clear;
  uint32_t clear_pm;   // premultiplied ARGB of the clear colour
  uint32_t pass0, pass1;
  int32_t blur_radius; // temp canvases: StackBlur radius (0 = not a temp)
  uint32_t band0;      // first entry of the canvas's row bands in band_off
  uint32_t blur_style; // temp canvases: BlurStyle (1 normal, 2 solid, 3 outer, 4 inner)
  uint32_t general;    // 1: a pass has a sweep / conical brush, a colour filter or a blend
                       // mode past the Porter-Duff src-over family
  uint64_t out_off;    // temp canvases: the filtered image the draw samples (px_off for
                       // kNormal, which blurs back in place; a third buffer otherwise)
};

// Rows of a canvas are grouped in bands of 1 << DevBatch::band_shift rows;
// each band lists, in draw order, the passes whose rows meet it (the
// compositor's pass bins).

// Geometry scratch layout of one pass: capacities in elements.
//   cap[0..2]  quad path (verbs, points, weights)
//   cap[3..5]  stroke outline
//   cap[6..8]  stroker inner path
//   cap[9..11] quad path of the outline
//   cap[12]    edges
struct SliceLayout {
  uint64_t off[16];
  uint64_t bytes;
  SKC_HD static uint64_t al(uint64_t v) { return (v + 15) & ~uint64_t(15); }
  SKC_HD void compute(const int32_t* cap, uint32_t edge_bytes) {
    uint64_t o = 0;
    for (int k = 0; k < 4; ++k) {
      off[3 * k + 0] = o; o = al(o + (uint64_t)cap[3 * k + 0]);
      off[3 * k + 1] = o; o = al(o + 8 * (uint64_t)cap[3 * k + 1]);
      off[3 * k + 2] = o; o = al(o + 4 * (uint64_t)cap[3 * k + 2]);
    }
    off[12] = o; o = al(o + (uint64_t)edge_bytes * cap[12]);        // built edges
    off[13] = o; o = al(o + (uint64_t)edge_bytes * (cap[12] + 2));  // sorted + sentinels
    off[14] = o; o = al(o + 4 * (uint64_t)cap[12]);                 // sort indices
    bytes = o;
  }
};

struct PassGeom {
  int32_t status;       // 0 ok, 1 scratch overflow (retry with bigger caps)
  int32_t n_edges;
  int32_t start_y, stop_y;
  int32_t left_bound, right_bound;
  int32_t acc_left, acc_width;
  float scan_top;
  int32_t row0, row1;   // canvas rows that can receive spans
  int32_t need[13];     // sizes seen (exact up to the failing stage)
  int32_t max_active;   // bound of the sweep's active-list length
  int32_t raw_spans;    // the pass keeps raw spans (kPassRawSpans): swept by the generic form
};

struct PassSweep {      // per-pass sweep buffers, set after geometry
  uint64_t work_off;    // byte offset of the pass's sweep memory
  uint64_t bytes;       // its size
  uint32_t rbase;       // first entry of the pass's rows in the row-span table
  uint32_t chunk;       // spans per span-pool chunk (any row of the pass fits)
};

struct PassComp {       // per-pass data the compositor reads
  int32_t row0, row1;   // canvas rows with row-span entries
  uint32_t rbase;
  uint32_t brush;
};

struct RowTask {
  uint32_t canvas, y, x0, x1;
};

// Batch device pointers handed to every kernel.
struct DevBatch {
  const uint8_t* verbs;
  const P* pts;
  const float* weights;
  const DrawDesc* draws;
  const PassDesc* passes;
  uint32_t n_passes;
  const CanvasDesc* canvases;
  uint8_t* scratch;
  PassGeom* geom;
  const PassSweep* sweep;
  uint8_t* sweepmem;   // per-pass sweep memory (SweepMemAt)
  uint2* rowspan;      // (first span, count) per pass row, zero when empty
  uint32_t* pass_spans;
  uint32_t* err;       // nonzero: a device self-check tripped (see pipeline)
  unsigned long long* pass_frags;  // fragments (clipped span pixels) per pass
  const PassComp* comp;
  uint2* spans;        // span pool: x | len << 16, alpha
  uint64_t span_cap;   // its capacity in spans
  unsigned long long* span_next;  // pool chunk allocator
  const Brush* brushes;
  const ConicalParams* conicals;  // per conical-gradient brush (Brush::conical)
  const uint8_t* srgb_tables;     // colour filters: linear->sRGB, sRGB->linear (256 each)
  const int16_t* cf_matrices;     // colour filters: matrix terms (Brush::cf_index)
  const float4* stop_colors;
  const float* stop_offsets;
  uint8_t* pixels;
  const uint8_t* roundtrip;
  const uint32_t* pass_list;  // passes to (re)run in the geometry kernel
  uint32_t n_list;
  uint8_t* pass_class;  // sweep form per pass: 0 register sweep, 1 generic
  int32_t reg_diff_cap; // accumulator entries per warp in shared memory
  const uint32_t* band_off;  // per band: first entry in bins (one past the end follows)
  const uint32_t* bins;      // pass indices, per band in draw order
  const uint32_t* sweep_order;  // passes in the order the sweeps take them (null: index order)
  int32_t band_shift;        // rows per pass-bin band: 1 << band_shift
  uint32_t reg_warps;        // warps per CTA of the register sweeps (1, 2 or 4)
  uint32_t* sweep_retry;     // [0]: passes the register sweeps gave up on (zeroed before the
                             // sweeps), [1, n_passes]: their indices
  unsigned int* task_next;   // persistent compositor's work counters (temp, main)
  unsigned int* sweep_done;  // per sweep form, CTAs finished (zeroed before the sweeps);
                             // null: the forms' launches do not overlap
  // path clips
  const ClipStateDesc* clip_states;  // [n_clip_states]
  uint32_t n_clip_states;
  uint32_t* clip_flags;       // per state: [0] its span list is not empty, [1] its op
  uint2* clip_rows;           // per state row: (first span, count) in the span pool
  const uint2* clip_items;    // (pass, canvas row) of the draws under a path clip
  uint32_t n_clip_items;
  // a canvas is general (CanvasDesc::general): the compositor's general
  // form runs for the whole batch
  uint32_t any_general;
  // device-planned renders: the plan's status (null for host-planned
  // ones); the compositor writes nothing when a plan buffer fell short
  const struct PlanStatus* plan;
};

// Spans per pool chunk for a pass: a power of two holding any one row of it.
// A row has at most one direct span per pixel plus one per interval end and
// one accumulated run per pixel: 2 * width + 2 * edges + 64 bounds it.
SKC_HD uint32_t SpanChunk(uint32_t width, int32_t edges) {
  uint64_t need = 2ull * width + 2ull * (uint64_t)(edges > 0 ? edges : 0) + 64;
  uint64_t c = 4096;
  while (c < need) c <<= 1;
  return (uint32_t)(c < (1ull << 31) ? c : (1ull << 31));
}

// ---------------------------------------------------------------------------
// Device planning (plan.cu): after the geometry stage, the per-pass sweep
// buffers, row tables, pass bins, sweep order and compositor tile order are
// computed on the device from the passes' geometry -- prefix sums over the
// passes, bins by warp-ballot compaction -- so a render needs no host round
// trip between its stages.  Buffers have host-chosen capacities; a plan that
// does not fit flags what fell short (and by how much) in its PlanStatus,
// the stages after it skip the work that would not fit, and the host grows
// the buffers and renders again.
// ---------------------------------------------------------------------------
enum : uint32_t {
  kPlanGeomOverflow = 1,  // a pass's geometry scratch overflowed (PassGeom::status)
  kPlanSweepMem = 2,      // sweep memory short
  kPlanRows = 4,          // row-span table short
  kPlanBins = 8,          // pass bins short
};
// pass_class of a pass no sweep form takes (nothing to sweep, or no room)
constexpr uint8_t kSweepSkip = 4;

struct PlanStatus {  // zeroed before each render, read back after it
  uint32_t flags;
  uint32_t geom_overflows;
  unsigned long long sweep_need;  // sweep-memory bytes the passes need
  unsigned long long rows_need;   // row-span entries
  unsigned long long bins_need;   // pass-bin entries
  // work of the render
  unsigned long long spans, edges;
  unsigned long long frags_by_brush[4];
  unsigned long long sort_total[2];  // items of the sweep and tile sorts
};

struct BandSeg {   // a pass-bin segment: the passes [p0, p1) of the band's canvas
  uint32_t band;   // global band index
  uint32_t p0, p1;
  uint32_t first;  // 1: the first segment of its band
};

struct DevPlan {
  PlanStatus* st;
  unsigned long long* a;  // per pass: sweep bytes, then their exclusive prefix sums
  unsigned long long* r;  // per pass: rows, then their exclusive prefix sums
  uint2* pband;           // per pass: first and last global band (x > y: none)
  const BandSeg* segs;
  uint32_t n_segs;
  unsigned long long* seg_cnt;  // per segment: bin entries, then their prefix sums
  uint32_t* band_off;
  uint32_t n_bands;
  uint32_t* bins;
  uint64_t sweep_cap, rows_cap, bins_cap;  // capacities: bytes, entries, entries
  uint32_t* sweep_order;
  const RowTask* tasks_in;  // main canvases' tiles, then the temp canvases'
  RowTask* tasks_out;       // the same, each list most work first
  uint32_t n_main, n_temp;
  // bucket-sort scratch: per item its key; per (key, block) counts, then
  // their prefix sums
  uint16_t* sort_keys;
  unsigned long long* sort_hist;
};
int LaunchPlan(const DevBatch& b, const DevPlan& q, cudaStream_t stream);
// Work totals of the render into the plan status.
int LaunchPlanStats(const DevBatch& b, const DevPlan& q, cudaStream_t stream);

// Shared memory of one register-sweep warp: its RegSharedT block, then an
// accumulator of reg_diff_cap entries (passes with wider accumulators keep
// theirs in the pass's sweep memory).
constexpr int32_t kRegDiffMax = 3072;

// kernel launchers (kernels.cu); all launch on `stream` and return the
// number of launches made
int LaunchGeometry(const DevBatch& b, cudaStream_t stream);
int LaunchSweep(const DevBatch& b, cudaStream_t stream);
// the path-clip stages after the sweeps; states: the host copy of b.clip_states
int LaunchPathClips(const DevBatch& b, const ClipStateDesc* states, uint32_t n_states,
                    cudaStream_t stream);
// ctas_per_sm > 0: a persistent grid of ctas_per_sm CTAs per SM taking row
// tiles from `counter` (zeroed before the launch); 0: one warp per tile.
int LaunchComposite(const DevBatch& b, const RowTask* tasks, uint32_t n_tasks, uint32_t chunk,
                    uint32_t ctas_per_sm, uint32_t num_sms, unsigned int* counter,
                    cudaStream_t stream);
// max_style: the largest BlurStyle of the temp canvases (the style pass
// runs only when one is not kNormal)
int LaunchBlur(const DevBatch& b, const uint32_t* temp_canvases, uint32_t n_temp,
               uint32_t max_h, uint32_t max_w, uint32_t max_style, cudaStream_t stream);
int LaunchClearCanvases(const DevBatch& b, const uint32_t* canvases, uint32_t n, cudaStream_t stream);

}  // namespace skc
