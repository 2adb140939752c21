/*
 * skity_cuda.h -- C ABI of the GB300 raster backend for Skity.
 *
 * This is the drop-in boundary for the reference's CPU software raster path:
 *
 *   Canvas::MakeSoftwareCanvas(Bitmap*)   include/skity/render/canvas.hpp:359,
 *                                         src/render/sw/sw_canvas.cc:146-156
 *   Canvas::Clear / DrawPath / Flush      include/skity/render/canvas.hpp:237-279
 *
 * It follows the conventions of the reference's C API (module/capi):
 * opaque handles (module/capi/include/skity_c/skity_base.h:34), result codes
 * (skity_base.h:48-56, extended here with device errors), extern "C"
 * entry points that never throw.  Plain pointers and sizes only.
 *
 * Pixels are premultiplied RGBA8 rows (Bitmap(w, h, kPremul_AlphaType) with
 * the default kRGBA colour type, include/skity/graphic/bitmap.hpp:28-30).
 * Draw semantics are those of SWCanvas: results agree with the reference
 * software backend (the oracle in oracle/ checks them).  The only observable
 * difference is timing: the software canvas writes pixels during each draw,
 * this canvas writes them back to the caller's bitmap at flush.
 */
#ifndef SKITY_CUDA_H
#define SKITY_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define SKITY_CUDA_API __declspec(dllexport)
#else
#define SKITY_CUDA_API __attribute__((visibility("default")))
#endif

/* Result codes: 0 and -1..-5 mean what skity_result means
 * (module/capi/include/skity_c/skity_base.h:48-56). */
typedef enum skity_cuda_result {
  SKITY_CUDA_NOT_READY = 1,                     /* skity_cuda_server_wait: not done yet */
  SKITY_CUDA_SUCCESS = 0,
  SKITY_CUDA_ERROR_INVALID_HANDLE = -1,
  SKITY_CUDA_ERROR_INVALID_ARGUMENT = -2,
  SKITY_CUDA_ERROR_INITIALIZATION_FAILED = -3,
  SKITY_CUDA_ERROR_OUT_OF_HOST_MEMORY = -4,
  SKITY_CUDA_ERROR_NOT_SUPPORTED = -5,
  SKITY_CUDA_ERROR_DEVICE = -6,                 /* a CUDA call failed */
  SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY = -7,   /* device budget exceeded */
  SKITY_CUDA_ERROR_DEVICE_TIMEOUT = -8,         /* a bounded device wait expired */
  SKITY_CUDA_ERROR_SCRATCH_LIMIT = -9,          /* input too large for the fixed
                                                   scratch of skity_cuda_draw_path_static */
  SKITY_CUDA_ERROR_CANCELLED = -10,             /* request dropped by skity_cuda_server_destroy */
} skity_cuda_result;

typedef struct skity_cuda_context_s* skity_cuda_context;
typedef struct skity_cuda_canvas_s* skity_cuda_canvas;
typedef struct skity_cuda_batch_s* skity_cuda_batch;

/* Path::Verb (include/skity/graphic/path.hpp:45-60). */
enum {
  SKITY_CUDA_VERB_MOVE = 0,
  SKITY_CUDA_VERB_LINE = 1,
  SKITY_CUDA_VERB_QUAD = 2,
  SKITY_CUDA_VERB_CONIC = 3,
  SKITY_CUDA_VERB_CUBIC = 4,
  SKITY_CUDA_VERB_CLOSE = 5,
};

/* A skity::Path as its storage holds it (path.hpp:590-596): verbs, points
 * (x, y pairs) and conic weights, plus Path::PathFillType (0 kWinding,
 * 1 kEvenOdd). */
typedef struct skity_cuda_path {
  const uint8_t* verbs;
  uint32_t verb_count;
  const float* points; /* 2 * point_count floats */
  uint32_t point_count;
  const float* conic_weights;
  uint32_t conic_weight_count;
  uint32_t fill_type;
} skity_cuda_path;

/* A gradient shader as Shader::AsGradient describes it (GradientInfo,
 * include/skity/effect/shader.hpp:48-70): Shader::MakeLinear, MakeRadial,
 * MakeSweep (radius = bias, scale of the angle: -start/360 and
 * 1 / ((end - start) / 360), shader.cc:88-104) and MakeTwoPointConical
 * (the degenerate concentric cases are radial gradients, shader.cc:50-86). */
typedef struct skity_cuda_gradient {
  uint32_t type;      /* 1 linear (p0 -> p1), 2 radial (centre p0, radius[0]),
                         3 sweep (centre p0, radius = bias, scale),
                         4 two-point conical (p0, radius[0] -> p1, radius[1]) */
  uint32_t tile_mode; /* TileMode: 0 clamp, 1 repeat, 2 mirror, 3 decal */
  uint32_t stop_count;
  uint32_t has_offsets; /* 0: stops evenly spaced (pos == nullptr) */
  float p0[2];
  float p1[2];
  float radius[2];
  const float* colors;  /* 4 * stop_count floats, unpremultiplied RGBA */
  const float* offsets; /* stop_count floats when has_offsets */
} skity_cuda_gradient;

/* A colour filter (include/skity/effect/color_filter.hpp, ColorFilters::*):
 * the fields of the filter ColorFilterBase describes (src/effect/
 * color_filter_base.hpp). */
typedef struct skity_cuda_color_filter {
  uint32_t type;       /* 1 Blend, 2 Matrix, 3 LinearToSRGBGamma, 4 SRGBToLinearGamma,
                          5 Compose (the identity on the software path) */
  uint32_t blend_mode; /* Blend: BlendMode */
  uint32_t color;      /* Blend: Color, ARGB */
  float matrix[20];    /* Matrix: row-major 4 x 5 */
} skity_cuda_color_filter;

/* An image (include/skity/graphic/image.hpp Image::MakeImage over an RGBA
 * Pixmap, include/skity/io/pixmap.hpp). */
typedef struct skity_cuda_image {
  uint32_t width, height;
  uint32_t alpha_type;  /* AlphaType: 2 kPremul_AlphaType, 3 kUnpremul_AlphaType */
  uint32_t reserved;
  const void* pixels;   /* RGBA8 rows, width * 4 bytes each; copied when recorded */
} skity_cuda_image;

/* Shader::MakeShader(image, sampling, x_tile_mode, y_tile_mode,
 * local_matrix) (include/skity/effect/shader.hpp:148-153). */
typedef struct skity_cuda_image_shader {
  const skity_cuda_image* image;
  uint32_t filter;          /* FilterMode: 0 kNearest, 1 kLinear; 2: a cubic resampler
                               (sampled bilinearly, as the software backend does) */
  uint32_t tile_x, tile_y;  /* TileMode: 0 kClamp, 1 kRepeat, 2 kMirror, 3 kDecal */
  float local_matrix[6];    /* sx, kx, tx, ky, sy, ty: scale and translate only (kx = ky = 0) */
} skity_cuda_image_shader;

/* The skity::Paint state the raster path reads (paint.hpp:46-285).
 * Colours are Color4f (unpremultiplied RGBA floats). */
typedef struct skity_cuda_paint {
  uint32_t style;      /* Paint::Style: fill, stroke, stroke-and-fill, stroke-then-fill */
  uint32_t cap;        /* Paint::Cap: butt, round, square */
  uint32_t join;       /* Paint::Join: miter, round, bevel */
  uint32_t blend_mode; /* BlendMode, kClear = 0 .. kLuminosity = 28 (kSrcOver = 3) */
  float fill_color[4];
  float stroke_color[4];
  float stroke_width;
  float miter_limit;
  const skity_cuda_gradient* shader; /* NULL: solid colour */
  uint32_t blur_style;  /* 0: no mask filter; BlurStyle: 1 kNormal, 2 kSolid, 3 kOuter, 4 kInner */
  float blur_radius;    /* MaskFilter::MakeBlur radius */
  const skity_cuda_color_filter* color_filter; /* NULL: none */
  const skity_cuda_image_shader* image_shader; /* NULL: none; not together with shader */
} skity_cuda_paint;

typedef struct skity_cuda_context_create_info {
  uint32_t struct_size;       /* sizeof(skity_cuda_context_create_info) */
  int32_t device;             /* CUDA device ordinal */
  uint64_t device_memory_budget; /* bytes the context may hold; 0 = 16 GiB */
} skity_cuda_context_create_info;

/* Timings and work counts of the last flush / batch render. */
typedef struct skity_cuda_stats {
  double device_ms;       /* kernel time, CUDA events on the context stream */
  double total_ms;        /* wall time of the call, uploads and readback included */
  uint64_t draws;         /* DrawPath calls rendered */
  uint64_t passes;        /* fill/stroke rasterisation passes */
  uint64_t edges;         /* fixed-point edges built */
  uint64_t spans;         /* coverage spans emitted inside the canvases */
  uint64_t pixels;        /* canvas pixels written back */
  uint64_t kernel_launches;
  uint64_t retries;       /* scratch-capacity and span-pool retries */
  /* per-stage device time of the last render (CUDA events around each
   * stage's launches on the context stream) */
  double geometry_ms;     /* path -> quads -> stroke -> edges -> sort */
  double sweep_count_ms;  /* AAA sweeps discarded because the context's span
                             pool had to grow (0 once it has grown) */
  double sweep_emit_ms;   /* AAA sweep writing the spans */
  double composite_ms;    /* span replay, shading, blending */
  double blur_ms;         /* StackBlur of blur mask filter temp canvases */
  uint64_t fragments;     /* sum of span lengths inside the canvases */
  uint64_t graph_replays; /* 1: the render replayed the batch's CUDA graph */
  uint64_t fragments_by_brush[4]; /* fragments shaded by solid, linear, radial
                                     (sweep and two-point conical included)
                                     and image (blur composite) brushes */
  double plan_ms;         /* device planning after the geometry: sweep buffers,
                             row tables, pass bins, sweep and tile orders */
  uint64_t host_syncs;    /* host waits on the device inside the render */
  /* skity_cuda_render_streams: wall time of its host stages */
  double parse_ms;        /* streams parsed into the batch (passes, brushes, caps) */
  double upload_ms;       /* inputs copied to the device */
  double readback_ms;     /* pixels copied back to the host */
} skity_cuda_stats;

/* Launch shape of the compositor and the granularity of its pass bins; no
 * effect on the pixels.  The autotuner (skity_gb300/autotune.py) picks one
 * per workload by timing batch renders. */
typedef struct skity_cuda_raster_config {
  uint32_t struct_size;   /* sizeof(skity_cuda_raster_config) */
  uint32_t tile_width;    /* compositor row tile in pixels: 32..2048 (default 1024) */
  uint32_t ctas_per_sm;   /* persistent compositor CTAs per SM, 0: one warp per
                             tile, no work queue (default 6) */
  uint32_t band_rows;     /* rows per pass-bin band: 8, 16, 32 or 64 (default 16) */
  uint32_t sweep_warps;   /* warps (one pass each) per CTA of the register-resident
                             sweeps: 1, 2 or 4 (default 2). A struct_size that ends
                             before this field keeps the default. */
} skity_cuda_raster_config;

/* ---- context ------------------------------------------------------------ */
SKITY_CUDA_API int32_t skity_cuda_context_create(
    const skity_cuda_context_create_info* info, skity_cuda_context* out);
SKITY_CUDA_API void skity_cuda_context_destroy(skity_cuda_context ctx);
/* Configuration of the context's batches and canvases created from now on. */
SKITY_CUDA_API int32_t skity_cuda_context_set_config(skity_cuda_context ctx,
                                                     const skity_cuda_raster_config* cfg);
/* Stats of the context's last flush or batch render. */
SKITY_CUDA_API int32_t skity_cuda_context_get_stats(skity_cuda_context ctx,
                                                    skity_cuda_stats* out);

/* ---- canvas (Canvas::MakeSoftwareCanvas counterpart) --------------------
 * Creates a canvas over a caller-owned premultiplied RGBA8 bitmap.  Like
 * MakeSoftwareCanvas, a NULL bitmap or a zero width/height yields no canvas
 * (SKITY_CUDA_ERROR_INVALID_ARGUMENT).  The bitmap must outlive the canvas;
 * its pixels are read at the first draw after a flush and written at flush. */
SKITY_CUDA_API int32_t skity_cuda_canvas_create(skity_cuda_context ctx,
                                                uint32_t width, uint32_t height,
                                                void* pixels, size_t row_bytes,
                                                skity_cuda_canvas* out);
SKITY_CUDA_API void skity_cuda_canvas_destroy(skity_cuda_canvas canvas);
/* Canvas::Clear(Color4f): DrawColor(color, kSrc) over the whole canvas. */
SKITY_CUDA_API int32_t skity_cuda_canvas_clear(skity_cuda_canvas canvas,
                                               const float color[4]);
/* Canvas::DrawPath(path, paint).  Path and paint data are copied; callers may
 * reuse their buffers after the call. */
SKITY_CUDA_API int32_t skity_cuda_canvas_draw_path(skity_cuda_canvas canvas,
                                                   const skity_cuda_path* path,
                                                   const skity_cuda_paint* paint);
/* Canvas::Save / Restore / Translate / Scale / Rotate / Skew / Concat /
 * SetMatrix (include/skity/render/canvas.hpp:51-122; canvas.cc:70-123 ->
 * LayerState, canvas_state.cc:18-46): the canvas matrix times the call's
 * matrix (Matrix::operator*, matrix.cc:452-460), later draws recorded under
 * it.  Rotation is about (px, py), in degrees (Matrix::RotateDeg,
 * matrix.cc:28-53); Concat / SetMatrix take a row-major 3x3 as
 * Matrix::Set9 does (scale x, skew x, translate x, skew y, scale y,
 * translate y, perspective 0, 1, 2).  Paths and clip paths are mapped by
 * any affine matrix (fills and strokes, solid colours, path clips);
 * shaders and blurs (whose filtered bitmap is drawn as an image) are taken
 * under scale and translation, layers under a translation.  Draws past
 * those limits (and draws under perspective) return
 * SKITY_CUDA_ERROR_NOT_SUPPORTED and draw nothing. */
SKITY_CUDA_API int32_t skity_cuda_canvas_save(skity_cuda_canvas canvas);
SKITY_CUDA_API int32_t skity_cuda_canvas_restore(skity_cuda_canvas canvas);
SKITY_CUDA_API int32_t skity_cuda_canvas_translate(skity_cuda_canvas canvas, float dx, float dy);
SKITY_CUDA_API int32_t skity_cuda_canvas_scale(skity_cuda_canvas canvas, float sx, float sy);
SKITY_CUDA_API int32_t skity_cuda_canvas_rotate(skity_cuda_canvas canvas, float degrees, float px,
                                                float py);
SKITY_CUDA_API int32_t skity_cuda_canvas_skew(skity_cuda_canvas canvas, float sx, float sy);
SKITY_CUDA_API int32_t skity_cuda_canvas_concat(skity_cuda_canvas canvas, const float m[9]);
SKITY_CUDA_API int32_t skity_cuda_canvas_set_matrix(skity_cuda_canvas canvas, const float m[9]);
/* Canvas::Concat / SetMatrix of a full 4x4 Matrix, its 16 floats in
 * column-major order (the Matrix(16 floats) constructor; pictures' CONCAT44
 * and SET_M44 records, module/io/src/picture.cc:431-460,991-1011). */
SKITY_CUDA_API int32_t skity_cuda_canvas_concat44(skity_cuda_canvas canvas, const float m[16]);
SKITY_CUDA_API int32_t skity_cuda_canvas_set_matrix44(skity_cuda_canvas canvas, const float m[16]);
/* Canvas::GetTotalMatrix as Matrix::Get9 (matrix.cc:106-116) gives it. */
SKITY_CUDA_API int32_t skity_cuda_canvas_get_matrix(skity_cuda_canvas canvas, float m[9]);
/* Canvas::ClipRect(rect, ClipOp::kIntersect) (canvas.hpp; canvas.cc:130-135,
 * 463-476): the rect, mapped by the canvas matrix (Matrix::MapRect, matrix.cc:
 * 306-337), narrows the canvas's global clip bounds (kept and restored by
 * Save / Restore); later DrawPath calls rasterise only inside them, as
 * SWCanvas does for a scale/translate matrix (sw_canvas.cc:279-295).  Under
 * a rotation or skew the canvas also clips by the rect as a path (Path::
 * AddRect under that matrix, Canvas::OnClipRect, canvas.cc:144-150), as the
 * reference does.  Clear is not clipped (SWCanvas::OnDrawPaint rasterises
 * the whole canvas); kDifference is a path clip of the rect
 * (skity_cuda_canvas_clip_path). */
SKITY_CUDA_API int32_t skity_cuda_canvas_clip_rect(skity_cuda_canvas canvas, float left, float top,
                                                   float right, float bottom);
/* Canvas::DrawImageRect(image, src, dst, sampling, paint) (canvas.hpp:342;
 * SWCanvas::OnDrawImageRect, sw_canvas.cc:641-677): a fill of dst with the
 * image's src rectangle mapped onto it (decal tiling, the paint's alpha and
 * blend mode).  src / dst are (left, top, right, bottom); a NULL image or an
 * empty src or dst draws nothing; paint NULL: Paint(). */
SKITY_CUDA_API int32_t skity_cuda_canvas_draw_image_rect(skity_cuda_canvas canvas,
                                                         const skity_cuda_image* image,
                                                         const float src[4], const float dst[4],
                                                         uint32_t filter,
                                                         const skity_cuda_paint* paint);
/* Canvas::ClipPath(path, op) (canvas.hpp; SWCanvas::OnClipPath,
 * sw_canvas.cc:317-336), op 0 kDifference / 1 kIntersect: later draws (and
 * Clear) are clipped by the path's spans the way the software canvas clips
 * them, nested clips combined as it combines them; Save / Restore keep and
 * restore the clip.  A kIntersect clip also narrows the global clip bounds
 * by the path's mapped bounds.  The path is rasterised under the canvas
 * matrix of the call (any affine matrix; perspective returns
 * SKITY_CUDA_ERROR_NOT_SUPPORTED).  ClipRRect and ClipRect with kDifference
 * are path clips of the rounded rect's / rect's path.  A blurred draw under
 * a clip keeps its temp canvas unclipped and clips the filtered bitmap's
 * image draw, as the reference does. */
SKITY_CUDA_API int32_t skity_cuda_canvas_clip_path(skity_cuda_canvas canvas,
                                                   const skity_cuda_path* path, uint32_t op);
/* Canvas::SaveLayer(bounds, paint) (canvas.hpp; canvas.cc:255-276;
 * SWCanvas::OnSaveLayer / OnLayerRestore, sw_canvas.cc:441-484, 891-902):
 * a Save whose matching Restore draws the layer -- every draw made in
 * between, rendered into a transparent bitmap over the layer's device
 * bounds -- onto the canvas with the paint's alpha and blend mode (paint
 * NULL: Paint()).  `bounds` is (left, top, right, bottom) in local
 * coordinates; empty bounds, or bounds outside the global clip bounds, save
 * no layer (a Save with an empty clip, as the reference does).  One level of
 * layers: a SaveLayer inside a layer, a layer paint with a mask or colour
 * filter, a blurred draw or a path clip inside a layer, and a flush while a
 * layer is open return SKITY_CUDA_ERROR_NOT_SUPPORTED. */
SKITY_CUDA_API int32_t skity_cuda_canvas_save_layer(skity_cuda_canvas canvas, const float bounds[4],
                                                    const skity_cuda_paint* paint);
/* Canvas::Flush: renders the recorded draws on the GPU and writes the
 * bitmap's pixels. */
SKITY_CUDA_API int32_t skity_cuda_canvas_flush(skity_cuda_canvas canvas);

/* ---- batched form -----------------------------------------------------------
 * Many canvases rendered in one pipeline.  Each canvas is a scene stream
 * (the flat draw-stream layout written by skity_gb300/scene.py: header,
 * verb/point/weight offsets, verbs, points, weights, 80-byte paint records,
 * 48-byte gradient records, stop colours and offsets).
 *
 * skity_cuda_render_streams: host streams in, host pixels out (each
 * out_pixels[i] receives width*height*4 bytes).  The whole call -- upload,
 * render, readback -- is timed in the stats. */
SKITY_CUDA_API int32_t skity_cuda_render_streams(skity_cuda_context ctx,
                                                 uint32_t count,
                                                 const uint8_t* const* streams,
                                                 const size_t* stream_bytes,
                                                 uint8_t* const* out_pixels);

/* Device-resident batches: the streams are parsed and uploaded once
 * (skity_cuda_batch_create); each skity_cuda_batch_render re-renders every
 * canvas from its clear colour with inputs already in device memory;
 * skity_cuda_batch_read copies canvas i's pixels to host memory.  The first
 * render plans the batch (geometry sizes, sweep buffers, row tables, pass
 * bins) and records its launches as a CUDA graph; later renders replay that
 * graph with one launch. */
SKITY_CUDA_API int32_t skity_cuda_batch_create(skity_cuda_context ctx, uint32_t count,
                                               const uint8_t* const* streams,
                                               const size_t* stream_bytes,
                                               skity_cuda_batch* out);
SKITY_CUDA_API int32_t skity_cuda_batch_render(skity_cuda_batch batch);
/* The plain per-draw form of the same render: every DrawPath of every
 * canvas rasterised and blended on its own, in order (geometry, sweep and
 * composite launches per draw, queued with no host round trip), as the
 * software canvas draws (SWCanvas::OnDrawPath, src/render/sw/
 * sw_canvas.cc:357-411).  Same pixels as skity_cuda_batch_render; it is the
 * baseline that batching is measured against.  Batches with blur mask
 * filters or path clips: SKITY_CUDA_ERROR_NOT_SUPPORTED. */
SKITY_CUDA_API int32_t skity_cuda_batch_render_per_draw(skity_cuda_batch batch);
SKITY_CUDA_API int32_t skity_cuda_batch_read(skity_cuda_batch batch, uint32_t index,
                                             uint8_t* out_pixels);
SKITY_CUDA_API void skity_cuda_batch_destroy(skity_cuda_batch batch);
/* Reconfigures a batch; its next render plans again (new replay graph). */
SKITY_CUDA_API int32_t skity_cuda_batch_set_config(skity_cuda_batch batch,
                                                   const skity_cuda_raster_config* cfg);
SKITY_CUDA_API int32_t skity_cuda_batch_get_config(skity_cuda_batch batch,
                                                   skity_cuda_raster_config* out);

/* ---- serving ------------------------------------------------------------
 * No single reference call: a request loop that renders canvases as they
 * arrive.  Each request is one canvas given as a scene stream (the layout of
 * skity_cuda_render_streams); it is copied at submit.  Requests are admitted
 * in arrival order against a device-memory budget (an estimate of each
 * request's footprint: canvas, span rows, geometry scratch) and rendered in
 * batches by `workers` worker threads, each with its own stream, so batches
 * overlap on the device: whatever is queued when a worker frees up goes into
 * its next batch (up to max_batch requests).  A request whose footprint alone
 * exceeds the budget is refused at submit (SKITY_CUDA_ERROR_OUT_OF_DEVICE_MEMORY).
 * A request's pixels do not depend on the batch it lands in. */
typedef struct skity_cuda_server_s* skity_cuda_server;

typedef struct skity_cuda_server_create_info {
  uint32_t struct_size;   /* sizeof(skity_cuda_server_create_info) */
  int32_t device;         /* CUDA device ordinal */
  uint64_t memory_budget; /* admission budget in bytes; 0 = 40 GiB */
  uint32_t workers;       /* concurrent batches; 0 = 2 */
  uint32_t max_batch;     /* requests per batch; 0 = 64 */
} skity_cuda_server_create_info;

typedef struct skity_cuda_request_info {
  double queue_ms;        /* submit -> its batch started */
  double latency_ms;      /* submit -> pixels ready */
  uint32_t batch_size;    /* requests in its batch */
  uint32_t width, height;
} skity_cuda_request_info;

SKITY_CUDA_API int32_t skity_cuda_server_create(const skity_cuda_server_create_info* info,
                                                skity_cuda_server* out);
/* Queues one request; *ticket names it in skity_cuda_server_wait. */
SKITY_CUDA_API int32_t skity_cuda_server_submit(skity_cuda_server server, const uint8_t* stream,
                                                size_t stream_bytes, uint64_t* ticket);
/* Waits up to timeout_ms for a request: SKITY_CUDA_NOT_READY if it is not
 * done yet (0 polls); otherwise its result code, with width*height*4 bytes of
 * premultiplied RGBA8 written to out_pixels on success.  A finished request's
 * ticket is released by this call. */
SKITY_CUDA_API int32_t skity_cuda_server_wait(skity_cuda_server server, uint64_t ticket,
                                              uint32_t timeout_ms, uint8_t* out_pixels,
                                              skity_cuda_request_info* info);
/* Cancels queued requests, waits for the batches in flight, frees the server. */
SKITY_CUDA_API void skity_cuda_server_destroy(skity_cuda_server server);

/* ---- drawing without allocation --------------------------------------------
 * No counterpart in the reference: its software canvas allocates as it draws.
 *
 * skity_cuda_draw_path_static draws ONE path with a solid-colour paint
 * (Canvas::DrawPath semantics: fill, stroke, stroke-and-fill or
 * stroke-then-fill; any BlendMode kClear..kLuminosity; no shader, no mask
 * filter) onto a premultiplied RGBA8 canvas that already lives in device
 * memory (`device_pixels`, `row_bytes` apart, a multiple of 4).  It allocates
 * nothing: no device memory (no cudaMalloc / cudaFree), no host heap.  Every
 * intermediate buffer comes from one fixed static device array of
 * SKITY_CUDA_STATIC_SCRATCH_BYTES per device, so it suits callers that must
 * not allocate while drawing -- a render loop held to a fixed footprint, or a
 * host that cannot afford the device-wide synchronisation that freeing
 * device memory implies.
 *
 * Limits: inputs whose path copy, geometry, sweep memory, row tables and
 * spans together need more than the static scratch are rejected with
 * SKITY_CUDA_ERROR_SCRATCH_LIMIT before the canvas is touched.  Both passes
 * of a stroke-and-fill or stroke-then-fill paint are sized and swept before
 * either is blended, so a draw is applied whole or not at all; a device
 * self-check failure (SKITY_CUDA_ERROR_DEVICE) likewise leaves the canvas
 * as it was.  A blend mode past kLuminosity is an invalid argument.
 *
 * The scratch is one per device, not one per call: calls that overlap on the
 * same device race on it, so callers on several host threads must serialise
 * them.  The call runs on `stream` (NULL: the default stream), waits on it
 * between its stages and returns once the draw is complete.  The first call on a device does a one-time
 * set-up (it looks up the scratch's device address with that device
 * current); make that first call -- an empty path is enough -- before any
 * stream capture begins. */
#define SKITY_CUDA_STATIC_SCRATCH_BYTES (16u << 20)
SKITY_CUDA_API int32_t skity_cuda_draw_path_static(int32_t device, uint8_t* device_pixels,
                                                   uint32_t width, uint32_t height,
                                                   size_t row_bytes,
                                                   const skity_cuda_path* path,
                                                   const skity_cuda_paint* paint,
                                                   void* stream);

/* ---- PictureRecorder / DisplayList -------------------------------------------
 * The reference's recorder (include/skity/recorder/picture_recorder.hpp,
 * display_list.hpp; C API module/capi/include/skity_c/skity_recorder.h):
 * skity_cuda_recorder_begin returns a canvas (of the recording's size) whose
 * calls -- clear, draw_path, draw_image_rect, save, restore, save_layer,
 * translate, clip_rect, clip_path -- are recorded instead of drawn, with
 * their paths, paints, shaders and images copied; flush on it does nothing.
 * skity_cuda_recorder_finish hands the recorded ops to a display list and
 * leaves the recorder empty (destroy it with skity_cuda_canvas_destroy).
 * skity_cuda_display_list_draw replays the ops, in order, through a canvas's
 * own calls (DisplayList::Draw, src/recorder/display_list.cc:330-343): the
 * canvas's current matrix and clips apply, and the first failing call's
 * code is returned after every op has been replayed.
 * skity_cuda_display_list_to_stream writes the display list as a scene
 * stream, the input of skity_cuda_render_streams, skity_cuda_batch_create
 * and skity_cuda_server_submit (out NULL: *size receives the byte count). */
typedef struct skity_cuda_display_list_s* skity_cuda_display_list;

SKITY_CUDA_API int32_t skity_cuda_recorder_begin(uint32_t width, uint32_t height,
                                                 skity_cuda_canvas* out);
SKITY_CUDA_API int32_t skity_cuda_recorder_finish(skity_cuda_canvas recorder,
                                                  skity_cuda_display_list* out);
SKITY_CUDA_API void skity_cuda_display_list_destroy(skity_cuda_display_list list);
SKITY_CUDA_API uint32_t skity_cuda_display_list_op_count(skity_cuda_display_list list);
SKITY_CUDA_API int32_t skity_cuda_display_list_draw(skity_cuda_display_list list,
                                                    skity_cuda_canvas canvas);
SKITY_CUDA_API int32_t skity_cuda_display_list_to_stream(skity_cuda_display_list list, uint8_t* out,
                                                         size_t* size);

/* Library version string. */
SKITY_CUDA_API const char* skity_cuda_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SKITY_CUDA_H */
