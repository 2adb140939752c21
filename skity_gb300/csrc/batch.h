// Host-side batch building for the raster pipeline (no CUDA runtime calls,
// so the CPU execution of the pipeline in tests uses it too).
//
// A batch is a set of canvases, each with its draws in order.  Every
// DrawPath becomes one or two rasterisation passes (fill / stroke, in
// Paint::Style order, src/render/paint_order.hpp:12-31).  A draw with a
// kNormal blur mask filter becomes a temp canvas holding the draw
// (SWCanvas::HandleFilter, src/render/sw/sw_canvas.cc:797-826) plus an image
// pass on the main canvas that samples the blurred temp
// (ImageFilterBase::BlurBitmapToCanvas, src/effect/image_filter.cc:184-194).
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/skity_cuda.h"
#include "kernels.cuh"
#include "stroke.cuh"
#include "sweep.cuh"

namespace skc {

// ---------------------------------------------------------------------------
// scene stream records (layout of skity_gb300/scene.py)
// ---------------------------------------------------------------------------
struct PaintRec {
  uint32_t style, cap, join, blend, fill_type;
  int32_t gradient;
  uint32_t blur_style;
  float blur_radius;
  float fill_color[4];
  float stroke_color[4];
  float stroke_width, miter;
  float translate[2];  // canvas translation of the draw (CTM = Translate(tx, ty))
};
static_assert(sizeof(PaintRec) == 80, "paint layout");
struct GradRec {
  uint32_t type, tile_mode, stop_count, stop_start, has_offsets, reserved;
  float p0[2], p1[2], radius[2];
};
static_assert(sizeof(GradRec) == 48, "gradient layout");
// A paint's colour filter (include/skity/effect/color_filter.hpp): type 0
// none, else 1 + ColorFilterType (1 blend, 2 matrix, 3 linear->sRGB gamma,
// 4 sRGB->linear gamma, 5 compose).
struct ColorFilterRec {
  uint32_t type, mode, color, pad;  // blend: BlendMode and ARGB colour
  float matrix[20];                 // matrix: row-major 4 x 5
};
static_assert(sizeof(ColorFilterRec) == 96, "colour filter layout");

// An image of the stream (header flag 8): size, AlphaType (2 premultiplied,
// 3 unpremultiplied) and the byte offset of its RGBA8 rows in the pixel blob.
struct ImageRec {
  uint32_t width, height, alpha_type, pad;
  uint64_t offset;
};
static_assert(sizeof(ImageRec) == 24, "image layout");
// A draw's image shader: Shader::MakeShader(image, sampling, tile_x, tile_y,
// local) (image 1-based, 0: none; filter 0 nearest, 1 linear, 2 cubic; local
// in MapPoint form, scale and translate only); rect = 1: the draw is
// DrawImageRect(image, src, dst), its path the dst rectangle.
struct ImageShaderRec {
  uint32_t image, filter, tile_x, tile_y;
  float local[6];
  uint32_t rect, pad;
  float src[4], dst[4];
};
static_assert(sizeof(ImageShaderRec) == 80, "image shader layout");

// Canvas::SaveLayer(bounds, paint) ... Restore around draws [start,
// restore) (restore kLayerOpen: not restored), with the canvas translation
// and global clip bounds in effect before the SaveLayer and the layer
// paint's alpha (Paint::GetAlphaF) and blend mode.  Layers do not nest.
struct LayerRec {
  float bounds[4], translate[2], clip[4];
  uint32_t start, restore;
  float alpha;
  uint32_t blend, pad[2];
};
static_assert(sizeof(LayerRec) == 64, "layer layout");
constexpr uint32_t kLayerOpen = 0xFFFFFFFFu;

struct StreamView {
  uint32_t width, height, has_clear;
  float clear[4];
  uint32_t nd, nv, np, nw, ng, ns;
  const uint32_t *vo, *po, *wo;
  const uint8_t* verbs;
  const float *pts, *wts;
  const PaintRec* paints;
  const GradRec* grads;
  const float *stop_colors, *stop_offsets;
  const float* clips;  // per draw device-space clip bounds (l, t, r, b), or null: none
  const ColorFilterRec* filters;  // per draw colour filter, or null: none
  // path clips (Canvas::ClipPath states) when the stream has them
  uint32_t n_clip_states;
  const struct ClipStateRec* clip_states;
  const uint8_t* clip_verbs;
  const float *clip_pts, *clip_wts;
  const uint32_t* draw_clip_state;  // per draw, 1-based (0: none)
  // images and per-draw image shaders when the stream has them
  uint32_t n_images;
  const ImageRec* images;
  const uint8_t* image_pixels;
  uint64_t image_bytes;
  const ImageShaderRec* image_shaders;
  // layers when the stream has them
  uint32_t n_layers;
  const LayerRec* layers;
  // per-draw canvas matrices (sx, kx, tx, ky, sy, ty) when the stream has
  // them (the paints' translations are then zero), else null
  const float* matrices;
  // per-clip-state canvas matrices of the ClipPath calls when the stream has
  // them (the states' translations are then zero), else null
  const float* clip_matrices;
};

// A ClipPath call of the stream: its parent state (1-based, 0: none), the
// op, the path's fill type and counts, the canvas translation and the global
// clip bounds at the call.
struct ClipStateRec {
  uint32_t parent, op, fill_type, nv, np, nw;
  float translate[2], bounds[4];
};
static_assert(sizeof(ClipStateRec) == 48, "clip state layout");

// A draw the device code can take: the verb sequence of a skity::Path
// (first verb kMove, a kMove after every kClose -- Path::LineTo/QuadTo/...
// inject one, path.cc:1327-1339), point and weight counts that match the
// verbs, finite coordinates inside the range the reference's 16.16 fixed
// point represents (|v| <= 16384 leaves room for stroke and blur margins),
// and sane paint parameters.
constexpr float kMaxCoord = 16384.f;
inline bool ValidPath(const uint8_t* verbs, uint32_t nv, const float* pts, uint32_t np,
                      const float* w, uint32_t nw) {
  uint64_t need_p = 0, need_w = 0;
  bool need_move = true;
  for (uint32_t i = 0; i < nv; ++i) {
    uint8_t v = verbs[i];
    if (v > kClose) return false;
    if (v != kMove && v != kClose && need_move) return false;
    if (v == kClose && need_move && i == 0) return false;
    switch (v) {
      case kMove: need_p += 1; need_move = false; break;
      case kLine: need_p += 1; break;
      case kQuad: need_p += 2; break;
      case kConic: need_p += 2; need_w += 1; break;
      case kCubic: need_p += 3; break;
      case kClose: need_move = true; break;
    }
  }
  if (need_p != np || need_w != nw) return false;
  for (uint64_t i = 0; i < 2ull * np; ++i) {
    float c = pts[i];
    if (!(c >= -kMaxCoord && c <= kMaxCoord)) return false;
  }
  for (uint32_t i = 0; i < nw; ++i) {
    if (std::isnan(w[i])) return false;
  }
  return true;
}
inline bool ValidPaint(uint32_t style, uint32_t cap, uint32_t join, float stroke_width, float miter,
                       float blur_radius) {
  if (style > 3 || cap > 2 || join > 2) return false;
  if (!(stroke_width >= 0.f && stroke_width <= 4096.f)) return false;
  if (!std::isfinite(miter)) return false;
  if (!(blur_radius <= 1024.f) || std::isnan(blur_radius)) return false;
  return true;
}

// A canvas translation keeps the draw's points inside the coordinate range
// ValidPath allows.
inline bool ValidTranslate(const float t[2], const float* pts, uint32_t np) {
  if (!(std::fabs(t[0]) <= kMaxCoord && std::fabs(t[1]) <= kMaxCoord)) return false;
  if (t[0] == 0.f && t[1] == 0.f) return true;
  for (uint32_t i = 0; i < np; ++i) {
    if (!(std::fabs(pts[2 * i] + t[0]) <= kMaxCoord && std::fabs(pts[2 * i + 1] + t[1]) <= kMaxCoord))
      return false;
  }
  return true;
}

// A canvas matrix keeps the draw's points inside the coordinate range
// ValidPath allows (points mapped as RastePath maps them; curves stay in
// their control points' hull).
inline bool ValidMatrix(const float m[6], const float* pts, uint32_t np) {
  Xform xf;
  xf.tx = m[2];
  xf.ty = m[5];
  xf.sx = m[0];
  xf.kx = m[1];
  xf.ky = m[3];
  xf.sy = m[4];
  xf.lin = true;
  for (uint32_t i = 0; i < np; ++i) {
    const P q = xf.map(mkP(pts[2 * i], pts[2 * i + 1]));
    if (!(std::fabs(q.x) <= kMaxCoord && std::fabs(q.y) <= kMaxCoord)) return false;
  }
  return true;
}

// Clip bounds: finite floats (the empty rect (0, 0, 0, 0) included).
inline bool ValidClip(const float c[4]) {
  return std::isfinite(c[0]) && std::isfinite(c[1]) && std::isfinite(c[2]) && std::isfinite(c[3]);
}
// The global clip bounds of a canvas that no ClipRect narrowed
// (kMaxCullRect, include/skity/render/canvas.hpp:26).
inline bool IsNoClip(const float c[4]) {
  return c[0] == -1e9f && c[1] == -1e9f && c[2] == 1e9f && c[3] == 1e9f;
}

// A colour filter record: a known type, a blend mode up to kLuminosity, and
// matrix terms whose int16 form (term * 255) is defined.
inline bool ValidColorFilter(const ColorFilterRec& f) {
  if (f.type > 5 || f.mode > 28) return false;
  if (f.type == 2) {
    for (float v : f.matrix)
      if (!(std::fabs(v * 255) < 32767.f)) return false;
  }
  return true;
}

// SRGBGammaColorFilter's tables (color_filter.cc:121-166), from the sRGB
// transfer functions: entry i = floor(255 * f(i / 255)), with i / 255 and the
// product in float and f in double.
inline void SRGBTables(uint8_t out[512]) {
  for (int i = 0; i < 256; ++i) {
    const float x = i / 255.f;
    const double xd = x;
    const double enc = xd <= 0.0031308 ? 12.92 * xd : 1.055 * std::pow(xd, 1 / 2.4) - 0.055;
    const double dec = xd <= 0.04045 ? xd / 12.92 : std::pow((xd + 0.055) / 1.055, 2.4);
    out[i] = (uint8_t)std::floor((float)enc * 255.f);
    out[256 + i] = (uint8_t)std::floor((float)dec * 255.f);
  }
}

inline bool ParseStream(const uint8_t* buf, size_t len, StreamView* s) {
  if (!buf || len < 72 || std::memcmp(buf, "SKSC", 4) != 0) return false;
  uint32_t hdr[7];
  std::memcpy(hdr, buf + 4, sizeof hdr);
  if (hdr[0] != 1) return false;
  s->width = hdr[1];
  s->height = hdr[2];
  s->has_clear = hdr[3];
  // 1: per-draw clip bounds follow the stops; 2: then per-draw colour
  // filters; 4: then the path clips
  const uint32_t flags = hdr[4];
  if (flags & ~127u) return false;
  size_t o = 32;
  std::memcpy(s->clear, buf + o, 16);
  o += 16;
  uint32_t cnt[6];
  std::memcpy(cnt, buf + o, sizeof cnt);
  o += sizeof cnt;
  s->nd = cnt[0];
  s->nv = cnt[1];
  s->np = cnt[2];
  s->nw = cnt[3];
  s->ng = cnt[4];
  s->ns = cnt[5];
  auto at = [&](size_t bytes) -> const uint8_t* {
    const uint8_t* p = buf + o;
    o += bytes;
    return p;
  };
  s->vo = (const uint32_t*)at(4 * (size_t)(s->nd + 1));
  s->po = (const uint32_t*)at(4 * (size_t)(s->nd + 1));
  s->wo = (const uint32_t*)at(4 * (size_t)(s->nd + 1));
  s->verbs = at(s->nv);
  o += (4 - s->nv % 4) % 4;
  s->pts = (const float*)at(8 * (size_t)s->np);
  s->wts = (const float*)at(4 * (size_t)s->nw);
  s->paints = (const PaintRec*)at(sizeof(PaintRec) * s->nd);
  s->grads = (const GradRec*)at(sizeof(GradRec) * s->ng);
  s->stop_colors = (const float*)at(16 * (size_t)s->ns);
  s->stop_offsets = (const float*)at(4 * (size_t)s->ns);
  s->clips = (flags & 1) ? (const float*)at(16 * (size_t)s->nd) : nullptr;
  s->filters = (flags & 2) ? (const ColorFilterRec*)at(sizeof(ColorFilterRec) * s->nd) : nullptr;
  s->n_clip_states = 0;
  s->clip_states = nullptr;
  s->clip_verbs = nullptr;
  s->clip_pts = s->clip_wts = nullptr;
  s->draw_clip_state = nullptr;
  if (flags & 4) {
    if (o + 4 > len) return false;
    std::memcpy(&s->n_clip_states, buf + o, 4);
    o += 4;
    if (s->n_clip_states > (1u << 20)) return false;
    s->clip_states = (const ClipStateRec*)at(sizeof(ClipStateRec) * (size_t)s->n_clip_states);
    if (o > len) return false;
    uint64_t tv = 0, tp = 0, tw = 0;
    for (uint32_t i = 0; i < s->n_clip_states; ++i) {
      const ClipStateRec& c = s->clip_states[i];
      if (c.parent > i || c.op > 1 || c.fill_type > 1 || !ValidClip(c.bounds) ||
          !(std::fabs(c.translate[0]) <= kMaxCoord && std::fabs(c.translate[1]) <= kMaxCoord))
        return false;
      tv += c.nv;
      tp += c.np;
      tw += c.nw;
    }
    if (tv + tp + tw > len) return false;
    s->clip_verbs = at(tv);
    o += (4 - tv % 4) % 4;
    s->clip_pts = (const float*)at(8 * tp);
    s->clip_wts = (const float*)at(4 * tw);
    s->draw_clip_state = (const uint32_t*)at(4 * (size_t)s->nd);
    if (o > len) return false;
    const uint8_t* v = s->clip_verbs;
    const float* p = s->clip_pts;
    const float* w = s->clip_wts;
    for (uint32_t i = 0; i < s->n_clip_states; ++i) {
      const ClipStateRec& c = s->clip_states[i];
      if (!ValidPath(v, c.nv, p, c.np, w, c.nw)) return false;
      float t[2] = {c.translate[0], c.translate[1]};
      if (!ValidTranslate(t, p, c.np)) return false;
      v += c.nv;
      p += 2 * (size_t)c.np;
      w += c.nw;
    }
    for (uint32_t d = 0; d < s->nd; ++d)
      if (s->draw_clip_state[d] > s->n_clip_states) return false;
  }
  s->n_images = 0;
  s->images = nullptr;
  s->image_pixels = nullptr;
  s->image_bytes = 0;
  s->image_shaders = nullptr;
  if (flags & 8) {
    if (o + 4 > len) return false;
    std::memcpy(&s->n_images, buf + o, 4);
    o += 4;
    if (s->n_images > (1u << 20)) return false;
    s->images = (const ImageRec*)at(sizeof(ImageRec) * (size_t)s->n_images);
    if (o + 8 > len) return false;
    std::memcpy(&s->image_bytes, buf + o, 8);
    o += 8;
    if (s->image_bytes > len) return false;
    s->image_pixels = at(s->image_bytes);
    o += (4 - s->image_bytes % 4) % 4;
    s->image_shaders = (const ImageShaderRec*)at(sizeof(ImageShaderRec) * (size_t)s->nd);
    if (o > len) return false;
    for (uint32_t i = 0; i < s->n_images; ++i) {
      const ImageRec& r = s->images[i];
      if (r.width == 0 || r.height == 0 || r.width > 16384 || r.height > 16384 ||
          (r.alpha_type != 2 && r.alpha_type != 3) || r.offset % 4 != 0 ||
          r.offset + (uint64_t)r.width * r.height * 4 > s->image_bytes)
        return false;
    }
    for (uint32_t d = 0; d < s->nd; ++d) {
      const ImageShaderRec& r = s->image_shaders[d];
      if (r.image == 0) continue;
      // scale and translate local matrices only, invertible
      const float* m = r.local;
      if (r.image > s->n_images || r.filter > 2 || r.tile_x > 3 || r.tile_y > 3 || r.rect > 1 ||
          m[1] != 0.f || m[3] != 0.f || !(std::fabs(m[0]) >= 1e-30f) ||
          !(std::fabs(m[4]) >= 1e-30f) || !(std::fabs(m[0]) <= 1e30f) ||
          !(std::fabs(m[4]) <= 1e30f) || !(std::fabs(m[2]) <= 1e30f) ||
          !(std::fabs(m[5]) <= 1e30f) || s->paints[d].gradient >= 0)
        return false;
    }
  }
  s->n_layers = 0;
  s->layers = nullptr;
  if (flags & 16) {
    if (o + 4 > len) return false;
    std::memcpy(&s->n_layers, buf + o, 4);
    o += 4;
    if (s->n_layers > (1u << 20)) return false;
    s->layers = (const LayerRec*)at(sizeof(LayerRec) * (size_t)s->n_layers);
    if (o > len) return false;
    for (uint32_t i = 0; i < s->n_layers; ++i) {
      const LayerRec& L = s->layers[i];
      const bool open = L.restore == kLayerOpen;
      // one level, in draw order, each restored before the next starts
      if (L.start > s->nd || (!open && (L.restore < L.start || L.restore > s->nd))) return false;
      if (i + 1 < s->n_layers && (open || s->layers[i + 1].start < L.restore)) return false;
      if (!ValidClip(L.bounds) || !ValidClip(L.clip) || L.blend > 28 ||
          !(L.alpha >= 0.f && L.alpha <= 1.f) || !(std::fabs(L.translate[0]) <= kMaxCoord) ||
          !(std::fabs(L.translate[1]) <= kMaxCoord))
        return false;
    }
  }
  s->matrices = nullptr;
  if (flags & 32) {
    s->matrices = (const float*)at(24 * (size_t)s->nd);
    if (o > len) return false;
    for (uint32_t d = 0; d < s->nd; ++d)
      for (int k = 0; k < 6; ++k)
        if (!std::isfinite(s->matrices[6 * (size_t)d + k])) return false;
  }
  s->clip_matrices = nullptr;
  if (flags & 64) {
    if (!(flags & 4)) return false;  // matrices of clip states the stream does not have
    s->clip_matrices = (const float*)at(24 * (size_t)s->n_clip_states);
    if (o > len) return false;
    const float* p = s->clip_pts;
    for (uint32_t i = 0; i < s->n_clip_states; ++i) {
      const ClipStateRec& c = s->clip_states[i];
      const float* m = s->clip_matrices + 6 * (size_t)i;
      for (int k = 0; k < 6; ++k)
        if (!std::isfinite(m[k])) return false;
      if (c.translate[0] != 0.f || c.translate[1] != 0.f || !ValidMatrix(m, p, c.np)) return false;
      p += 2 * (size_t)c.np;
    }
  }
  if (o > len) return false;
  if (s->width == 0 || s->height == 0 || s->width > 65535 || s->height > 65535) return false;
  for (uint32_t d = 0; d < s->nd; ++d) {
    if (s->vo[d] > s->vo[d + 1] || s->vo[d + 1] > s->nv) return false;
    if (s->po[d] > s->po[d + 1] || s->po[d + 1] > s->np) return false;
    if (s->wo[d] > s->wo[d + 1] || s->wo[d + 1] > s->nw) return false;
    if (s->paints[d].gradient >= (int32_t)s->ng) return false;
    const PaintRec& pr = s->paints[d];
    if (!ValidPaint(pr.style, pr.cap, pr.join, pr.stroke_width, pr.miter, pr.blur_radius))
      return false;
    if (!ValidTranslate(pr.translate, s->pts + 2 * (size_t)s->po[d], s->po[d + 1] - s->po[d]))
      return false;
    if (s->matrices) {
      if (pr.translate[0] != 0.f || pr.translate[1] != 0.f) return false;
      if (!ValidMatrix(s->matrices + 6 * (size_t)d, s->pts + 2 * (size_t)s->po[d],
                       s->po[d + 1] - s->po[d]))
        return false;
    }
    if (s->clips && !ValidClip(s->clips + 4 * (size_t)d)) return false;
    if (s->filters && !ValidColorFilter(s->filters[d])) return false;
    if (!ValidPath(s->verbs + s->vo[d], s->vo[d + 1] - s->vo[d], s->pts + 2 * (size_t)s->po[d],
                   s->po[d + 1] - s->po[d], s->wts + s->wo[d], s->wo[d + 1] - s->wo[d]))
      return false;
  }
  for (uint32_t g = 0; g < s->ng; ++g) {
    if ((uint64_t)s->grads[g].stop_start + s->grads[g].stop_count > s->ns) return false;
    if (s->grads[g].stop_count > 4096 || s->grads[g].tile_mode > 3) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// host-side brush setup (SWCanvas::GenerateBrush, sw_canvas.cc:727-795)
// ---------------------------------------------------------------------------
// PointsToUnit (sw_span_brush.cc:164-200) composed with device_to_local
inline Mat4 PointsToUnitMat(const GradRec& g) {
  if (g.type == 1) {
    float sx = g.p0[0], sy = g.p0[1];
    float ssx = g.p1[0] - sx, ssy = g.p1[1] - sy;
    float length = std::sqrt(ssx * ssx + ssy * ssy);
    float scale = length > 0 ? 1.0f / length : 0;
    float ux = ssx * scale, uy = ssy * scale;
    float sine = -uy, cosine = ux;
    Mat4 rot;
    rot.identity();
    rot.e[0][0] = cosine;
    rot.e[1][0] = -sine;
    rot.e[0][1] = sine;
    rot.e[1][1] = cosine;
    return MatMul(MatMul(rot, MatScale(scale, scale)), MatTranslate(-sx, -sy));
  }
  float radius = g.radius[0];
  float scale = radius > 0 ? 1.0f / radius : 0;
  return MatMul(MatScale(scale, scale), MatTranslate(-g.p0[0], -g.p0[1]));
}
// PointsToUnit(p0, p1) (sw_span_brush.cc:196-214): the line p0 -> p1 to
// the unit x axis.
inline Mat4 LineToUnit(float p0x, float p0y, float p1x, float p1y) {
  GradRec g;
  std::memset(&g, 0, sizeof g);
  g.type = 1;
  g.p0[0] = p0x;
  g.p0[1] = p0y;
  g.p1[0] = p1x;
  g.p1[1] = p1y;
  return PointsToUnitMat(g);
}
inline void MapPointForm(const Mat4& m, float out[6]) {  // MapPoint's six terms
  out[0] = m.e[0][0];
  out[1] = m.e[1][0];
  out[2] = m.e[3][0];
  out[3] = m.e[0][1];
  out[4] = m.e[1][1];
  out[5] = m.e[3][1];
}

// ConicalGradientColorBrush::OnPreBrush (sw_span_brush.cc:394-437) on the
// gradient's points (Points: z = 0, w = 1) and radii; vector lengths are
// glm lengths of the 4-component points.
inline ConicalParams ConicalSetup(const GradRec& g, const Mat4& device_to_local) {
  const float kNZ = 1.0f / (1 << 12);
  ConicalParams c;
  std::memset(&c, 0, sizeof c);
  MapPointForm(device_to_local, c.d2l);
  float c0[4] = {g.p0[0], g.p0[1], 0.f, 1.f}, c1[4] = {g.p1[0], g.p1[1], 0.f, 1.f};
  float r0 = g.radius[0], r1 = g.radius[1];
  auto len4 = [](const float a[4], const float b[4]) {
    const float d[4] = {a[0] - b[0], a[1] - b[1], a[2] - b[2], a[3] - b[3]};
    return std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3]);
  };
  const float delta_center = len4(c1, c0);
  const float delta_radius = std::fabs(r1 - r0);
  c.mode = 0;
  if (!(r0 < 0 || r1 < 0)) {
    const bool radial = delta_center < kNZ, strip = delta_radius < kNZ;
    if (radial) {
      c.mode = strip ? 2 : 1;
      if (!strip) {
        c.scale = (float)(1.0 / delta_radius);
        c.scale_sign = delta_radius < 0 ? -1.f : 1.f;
        c.bias = r0 / delta_radius;
      }
      c.c0x = c0[0];
      c.c0y = c0[1];
    } else if (strip) {
      c.mode = 3;
      MapPointForm(LineToUnit(c0[0], c0[1], c1[0], c1[1]), c.t);
      const float r = r0 / delta_center;
      c.r2 = r * r;
    } else {
      c.mode = 4;
      c.swap01 = r1 < kNZ ? 1u : 0u;
      if (c.swap01) {
        for (int i = 0; i < 4; ++i) std::swap(c0[i], c1[i]);
        std::swap(r0, r1);
      }
      const float f = r0 / (r0 - r1);
      float cf[4];
      for (int i = 0; i < 4; ++i) cf[i] = c0[i] * (1.f - f) + c1[i] * f;
      r1 = r1 / len4(c1, cf);
      c.f = f;
      c.r1 = r1;
      c.r1_square = r1 * r1;
      MapPointForm(LineToUnit(cf[0], cf[1], c1[0], c1[1]), c.t);
      if (r0 < 0 || r1 < 0) c.mode = 0;  // CalculateConical's check, on the final radii
    }
  }
  return c;
}

// Matrix::Invert of a scale-and-translate canvas matrix m = (sx, 0, tx, 0,
// sy, ty) (matrix.cc:134-142, 242-266): the identity for a matrix within
// FLT_EPSILON of it; else the reciprocal scales (an infinite one leaves the
// identity: Invert fails after Reset) and the translation times them.
inline Mat4 InvertScaleTranslate(const float m[6]) {
  Mat4 ctm = MatScale(m[0], m[4]);
  ctm.e[3][0] = m[2];
  ctm.e[3][1] = m[5];
  Mat4 inv;
  inv.identity();
  if (ctm.is_identity()) return inv;
  if (m[0] != 1.f || m[4] != 1.f) {
    const float ix = 1.f / m[0], iy = 1.f / m[4];
    if (ix == INFINITY || iy == INFINITY) return inv;
    inv.e[0][0] = ix;
    inv.e[1][1] = iy;
    inv.e[3][0] = -m[2] * ix;
    inv.e[3][1] = -m[5] * iy;
  } else {
    inv.e[3][0] = -m[2];
    inv.e[3][1] = -m[5];
  }
  return inv;
}
// The canvas matrix has a linear part (anything but a translation).
inline bool HasLinear(const float m[6]) {
  return !(m[0] == 1.f && m[1] == 0.f && m[3] == 0.f && m[4] == 1.f);
}
inline uint32_t SolidPM(const float c[4]) {
  return ColorToPMColor(Color4fToColor(c[0], c[1], c[2], c[3]));
}

struct HostBatch {
  std::vector<uint8_t> verbs;
  std::vector<P> pts;
  std::vector<float> weights;
  std::vector<DrawDesc> draws;
  std::vector<PassDesc> passes;
  std::vector<Brush> brushes;
  std::vector<ConicalParams> conicals;
  std::vector<int16_t> cf_matrices;  // colour-filter matrices, 20 terms each
  std::vector<ClipStateDesc> clip_states;  // path-clip states of all canvases, in call order
  std::vector<CanvasDesc> canvases;
  std::vector<float4> stop_colors;
  std::vector<float> stop_offsets;
  std::vector<uint32_t> main_canvases, temp_canvases;
  uint64_t pixel_bytes = 0;
  uint64_t draw_count = 0;
  uint32_t max_temp_w = 0, max_temp_h = 0;
  uint32_t max_temp_style = 0;  // largest BlurStyle of the temp canvases (1: kNormal only)

  // the images of the stream being added: their byte offsets in the pixel
  // buffer, and the uploads that put them there (offset, first byte, bytes)
  std::vector<uint64_t> image_off;
  struct ImageUpload {
    uint64_t off;
    std::vector<uint8_t> bytes;
  };
  std::vector<ImageUpload> image_uploads;

  uint64_t AllocPixels(uint64_t bytes) {
    uint64_t o = (pixel_bytes + 255) & ~uint64_t(255);
    pixel_bytes = o + bytes;
    return o;
  }
  uint32_t AddDraw(const uint8_t* v, uint32_t nv, const float* p, uint32_t np, const float* w,
                   uint32_t nw) {
    DrawDesc d;
    d.v0 = (uint32_t)verbs.size();
    d.nv = nv;
    d.p0 = (uint32_t)pts.size();
    d.np = np;
    d.w0 = (uint32_t)weights.size();
    d.nw = nw;
    verbs.insert(verbs.end(), v, v + nv);
    for (uint32_t i = 0; i < np; ++i) pts.push_back(mkP(p[2 * i], p[2 * i + 1]));
    weights.insert(weights.end(), w, w + nw);
    draws.push_back(d);
    return (uint32_t)draws.size() - 1;
  }
};

// Initial scratch capacities of a pass (counts that later overflow are
// retried with the exact sizes the geometry kernel reports).
inline void InitialCaps(const uint8_t* verbs, uint32_t nv, const float* pts, bool stroke,
                        int32_t cap[13]) {
  int64_t qv = 2, qp = 2;
  uint32_t pi = 0;
  P last = mkP(0, 0);
  for (uint32_t i = 0; i < nv; ++i) {
    switch (verbs[i]) {
      case kMove: qv += 1; qp += 1; last = mkP(pts[2 * pi], pts[2 * pi + 1]); pi += 1; break;
      case kLine: qv += 1; qp += 1; last = mkP(pts[2 * pi], pts[2 * pi + 1]); pi += 1; break;
      case kQuad: qv += 1; qp += 2; last = mkP(pts[2 * pi + 2], pts[2 * pi + 3]); pi += 2; break;
      case kConic: qv += 2; qp += 4; last = mkP(pts[2 * pi + 2], pts[2 * pi + 3]); pi += 2; break;
      case kCubic: {
        P c[4] = {last, mkP(pts[2 * pi], pts[2 * pi + 1]), mkP(pts[2 * pi + 2], pts[2 * pi + 3]),
                  mkP(pts[2 * pi + 4], pts[2 * pi + 5])};
        double n = CubicQuadCountD(c);
        int64_t k = (int64_t)n + 1;
        qv += k;
        qp += 2 * k;
        last = c[3];
        pi += 3;
      } break;
      case kClose: qv += 2; qp += 1; break;
      default: break;
    }
  }
  for (int k = 0; k < 13; ++k) cap[k] = 0;
  cap[0] = (int32_t)qv;
  cap[1] = (int32_t)qp;
  cap[2] = 0;
  if (stroke) {
    int64_t ov = 6 * qv + 16, op = 6 * qp + 16 * qv + 32, ow = 4 * qv + 8;
    cap[3] = (int32_t)ov;
    cap[4] = (int32_t)op;
    cap[5] = (int32_t)ow;
    cap[6] = (int32_t)ov;
    cap[7] = (int32_t)op;
    cap[8] = (int32_t)ow;
  }
}
// Bounds that follow exactly from earlier stages' sizes.
inline void DerivedCaps(int32_t cap[13], bool stroke) {
  if (stroke) {
    cap[9] = 2 * cap[3] + 2;
    cap[10] = 2 * cap[4] + cap[3] + 2;
    cap[11] = 0;
    cap[12] = cap[9] + cap[10] + 2;
  } else {
    cap[12] = cap[0] + cap[1] + 2;
  }
}

// The paint's colour filter on a brush (SWSpanBrush applies it to each
// covered colour before blending, sw_span_brush.cc:108-136).  Compose is
// the identity on this path (ComposeColorFilter::OnFilterColor,
// color_filter.cc:182-186).
inline void SetColorFilter(HostBatch& hb, const StreamView& s, uint32_t d, Brush* br) {
  br->cf_type = 0;
  if (!s.filters) return;
  const ColorFilterRec& f = s.filters[d];
  if (f.type == 1) {  // BlendColorFilter (color_filter.cc:109-111)
    br->cf_type = 1;
    br->cf_mode = f.mode;
    br->cf_pm = ColorToPMColor(f.color);
  } else if (f.type == 2) {  // MatrixColorFilter: int16 terms = row_major * 255 (truncated)
    br->cf_type = 2;
    br->cf_index = (uint32_t)hb.cf_matrices.size();
    for (int i = 0; i < 20; ++i) hb.cf_matrices.push_back((int16_t)(f.matrix[i] * 255));
  } else if (f.type == 3 || f.type == 4) {
    br->cf_type = f.type;
  }
}

// The draw has a colour filter that is not the identity (Compose is, here).
inline bool FiltersColor(const StreamView& s, uint32_t d) {
  return s.filters && s.filters[d].type != 0 && s.filters[d].type != 5;
}

// Appends the passes of one DrawPath (fill/stroke in paint order) to `out`.
// clip_shift: the draw's clip bounds moved by (dx, dy) -- a draw inside a
// layer, whose sub-canvas clips with the global clip bounds offset by the
// layer's origin (SWCanvas::GetScanClipBounds, sw_canvas.hpp:157-161).
// ctm: the canvas matrix (sx, kx, tx, ky, sy, ty); shaders are taken under
// scale and translation (NOT_SUPPORTED under rotation or skew).
inline int AddDrawPasses(HostBatch& hb, const StreamView& s, uint32_t d, uint32_t draw_index,
                         uint32_t canvas, const float ctm[6], std::vector<PassDesc>& out,
                         const float* clip_shift = nullptr, bool draw_clip = true) {
  const float tx = ctm[2], ty = ctm[5];
  const bool lin = HasLinear(ctm);
  const PaintRec& pr = s.paints[d];
  const uint8_t* verbs = s.verbs + s.vo[d];
  uint32_t nv = s.vo[d + 1] - s.vo[d];
  const float* pts = s.pts + 2 * (size_t)s.po[d];
  auto make_brush = [&](bool stroke) {
    Brush br;
    std::memset(&br, 0, sizeof br);
    br.blend = pr.blend;
    br.global_alpha = 255;
    const GradRec* g = pr.gradient >= 0 ? &s.grads[pr.gradient] : nullptr;
    // Shader::MakeLinear / MakeRadial return null for < 2 stops or a
    // negative radius (src/effect/shader.cc:21-45)
    if (g && (g->stop_count < 2 || (g->type == 2 && g->radius[0] < 0.f) || g->type < 1 ||
              g->type > 4)) {
      g = nullptr;
    }
    const ImageShaderRec* is =
        s.image_shaders && s.image_shaders[d].image ? &s.image_shaders[d] : nullptr;
    if (is) {
      // PixmapBrush (sw_canvas.cc:755-786, sw_span_brush.cc:555-579): unit
      // coordinates = Scale(1/w, 1/h) * inverse(local) * inverse(CTM)
      const ImageRec& im = s.images[is->image - 1];
      Mat4 inv;  // Matrix::InvertNonIdentity, scale-and-translate form (matrix.cc:242-268)
      inv.identity();
      const float lsx = is->local[0], lsy = is->local[4], ltx = is->local[2], lty = is->local[5];
      if (lsx != 1.f || lsy != 1.f) {
        const float ix = 1.f / lsx, iy = 1.f / lsy;
        inv.e[0][0] = ix;
        inv.e[1][1] = iy;
        inv.e[3][0] = -ltx * ix;
        inv.e[3][1] = -lty * iy;
      } else {
        inv.e[3][0] = -ltx;
        inv.e[3][1] = -lty;
      }
      Mat4 m = MatMul(MatMul(MatScale(1.f / (float)im.width, 1.f / (float)im.height), inv),
                      InvertScaleTranslate(ctm));
      br.kind = 6;
      br.m[0] = m.e[0][0];
      br.m[1] = m.e[1][0];
      br.m[2] = m.e[3][0];
      br.m[3] = m.e[0][1];
      br.m[4] = m.e[1][1];
      br.m[5] = m.e[3][1];
      br.img_w = im.width;
      br.img_h = im.height;
      br.img_off = hb.image_off[is->image - 1];
      br.tile = ImageMode(is->tile_x, is->tile_y, is->filter != 0, im.alpha_type == 3);
      // Paint::GetAlphaF (paint.cc:96-98) as SWSpanBrush's global alpha
      br.global_alpha = (uint8_t)(255 * (pr.style == 1 ? pr.stroke_color[3] : pr.fill_color[3]));
    } else if (g) {
      // brush kinds: 1 linear, 2 radial, 4 sweep, 5 conical (3 is the image brush)
      br.kind = g->type <= 2 ? g->type : g->type + 1;
      Mat4 dev_to_local = MatMul(MatTranslate(0, 0), InvertScaleTranslate(ctm));
      // PointsToUnit (sw_span_brush.cc:164-194): the sweep's is a translation
      // to its centre; the conical brush maps device_to_local and its own
      // transforms one after the other
      Mat4 m = g->type == 3   ? MatMul(MatTranslate(-g->p0[0], -g->p0[1]), dev_to_local)
               : g->type == 4 ? dev_to_local
                              : MatMul(PointsToUnitMat(*g), dev_to_local);
      if (g->type == 3) {
        br.bias = g->radius[0];
        br.scale = g->radius[1];
      }
      if (g->type == 4) {
        br.conical = (uint32_t)hb.conicals.size();
        hb.conicals.push_back(ConicalSetup(*g, dev_to_local));
      }
      br.m[0] = m.e[0][0];
      br.m[1] = m.e[1][0];
      br.m[2] = m.e[3][0];
      br.m[3] = m.e[0][1];
      br.m[4] = m.e[1][1];
      br.m[5] = m.e[3][1];
      br.tile = g->tile_mode;
      br.stop_count = g->stop_count;
      br.has_offsets = g->has_offsets;
      br.stop0 = (uint32_t)hb.stop_colors.size();
      for (uint32_t i = 0; i < g->stop_count; ++i) {
        const float* c = s.stop_colors + 4 * (size_t)(g->stop_start + i);
        hb.stop_colors.push_back(make_float4(c[0], c[1], c[2], c[3]));
        hb.stop_offsets.push_back(g->has_offsets ? s.stop_offsets[g->stop_start + i] : 0.f);
      }
      // EnsureColorOffsetsNonDescending (gradient_shader.cc:14-21)
      if (g->has_offsets) {
        for (uint32_t i = 0; i + 1 < g->stop_count; ++i) {
          float& a = hb.stop_offsets[br.stop0 + i];
          float& b = hb.stop_offsets[br.stop0 + i + 1];
          if (a > b) b = a;
        }
      }
    } else {
      br.kind = 0;
      br.solid = SolidPM(stroke ? pr.stroke_color : pr.fill_color);
    }
    SetColorFilter(hb, s, d, &br);
    hb.brushes.push_back(br);
    return (uint32_t)hb.brushes.size() - 1;
  };
  auto add = [&](bool stroke) {
    PassDesc pd;
    std::memset(&pd, 0, sizeof pd);
    pd.draw = draw_index;
    pd.canvas = canvas;
    // kPassSrcOver lets the sweep drop spans of zero coverage (a no-op under
    // src-over) -- unless a colour filter can turn transparent into a colour
    pd.flags = (stroke ? kPassStroke : 0) | ((!stroke && pr.fill_type == 1) ? kPassEvenOdd : 0) |
               ((pr.blend == 3 && !FiltersColor(s, d)) ? kPassSrcOver : 0);
    pd.cap_join = (pr.cap & 0xFF) | ((pr.join & 0xFF) << 8);
    pd.tx = tx;
    pd.ty = ty;
    if (lin) {
      pd.flags |= kPassMatrix;
      pd.lin[0] = ctm[0];
      pd.lin[1] = ctm[1];
      pd.lin[2] = ctm[3];
      pd.lin[3] = ctm[4];
    }
    if (draw_clip && s.clips && !IsNoClip(s.clips + 4 * (size_t)d)) {
      pd.clipped = 1;
      std::memcpy(pd.clip, s.clips + 4 * (size_t)d, sizeof pd.clip);
      if (clip_shift) {  // Rect::Offset
        pd.clip[0] = pd.clip[0] + clip_shift[0];
        pd.clip[1] = pd.clip[1] + clip_shift[1];
        pd.clip[2] = pd.clip[2] + clip_shift[0];
        pd.clip[3] = pd.clip[3] + clip_shift[1];
      }
    }
    pd.stroke_width = pr.stroke_width;
    pd.miter = pr.miter;
    pd.brush = make_brush(stroke);
    pd.ga = hb.brushes[pd.brush].global_alpha;
    InitialCaps(verbs, nv, pts, stroke, pd.cap);
    DerivedCaps(pd.cap, stroke);
    out.push_back(pd);
  };
  const bool shaded = (pr.gradient >= 0) || (s.image_shaders && s.image_shaders[d].image);
  if (shaded && (ctm[1] != 0.f || ctm[3] != 0.f)) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
  bool need_fill = pr.style != 1, need_stroke = pr.style != 0;
  if (pr.style == 3) {
    if (need_stroke) add(true);
    if (need_fill) add(false);
  } else {
    if (need_fill) add(false);
    if (need_stroke) add(true);
  }
  return SKITY_CUDA_SUCCESS;
}

// Layers (Canvas::SaveLayer, canvas.cc:255-276 -> SWCanvas::OnSaveLayer,
// sw_canvas.cc:441-484, on the canvas itself): the layer's bounds in local
// coordinates (log_bounds), the origin of its sub-canvas (rel_bounds'
// left/top) and its bitmap size.
struct LayerGeom {
  float log[4];
  float off[2];
  uint32_t w = 0, h = 0;
};
inline bool RectIntersect(float* a, const float* b) {  // Rect::Intersect (rect.cc:160-172)
  const float l = std::max(a[0], b[0]), r = std::min(a[2], b[2]);
  const float t = std::max(a[1], b[1]), bt = std::min(a[3], b[3]);
  if (!(l < r && t < bt)) return false;
  a[0] = l;
  a[1] = t;
  a[2] = r;
  a[3] = bt;
  return true;
}
// Matrix::MapRect of a translation (matrix.cc:306-337): corners x + tx, min/max.
inline void MapRectTranslate(const float* src, float tx, float ty, float* dst) {
  const float x0 = src[0] + tx, x1 = src[2] + tx, y0 = src[1] + ty, y1 = src[3] + ty;
  dst[0] = std::min(x0, x1);
  dst[2] = std::max(x0, x1);
  dst[1] = std::min(y0, y1);
  dst[3] = std::max(y0, y1);
}
inline LayerGeom LayerGeometry(const StreamView& s, const LayerRec& L) {
  LayerGeom g;
  const float tx = L.translate[0], ty = L.translate[1];
  // Canvas::SaveLayer narrows the global clip bounds by the mapped bounds
  // (CalculateGlobalClipBounds) before OnSaveLayer reads them
  float clip[4] = {L.clip[0], L.clip[1], L.clip[2], L.clip[3]};
  float mapped[4];
  MapRectTranslate(L.bounds, tx, ty, mapped);
  if (!RectIntersect(clip, mapped)) clip[0] = clip[1] = clip[2] = clip[3] = 0.f;
  // ComputeFastBounds of a fill paint without a mask filter: the bounds
  float layer[4] = {L.bounds[0] - 0.f, L.bounds[1] - 0.f, L.bounds[2] + 0.f, L.bounds[3] + 0.f};
  float device[4] = {0.f, 0.f, (float)s.width, (float)s.height};
  const float scan[4] = {clip[0] + -0.f, clip[1] + -0.f, clip[2] + -0.f, clip[3] + -0.f};
  if (!RectIntersect(device, scan)) device[0] = device[1] = device[2] = device[3] = 0.f;
  // device_to_local: the inverse translation (identity for none)
  const bool ident = tx == 0.f && ty == 0.f;
  float local_clip[4];
  MapRectTranslate(device, ident ? 0.f : -tx, ident ? 0.f : -ty, local_clip);
  if (!RectIntersect(layer, local_clip)) layer[0] = layer[1] = layer[2] = layer[3] = 0.f;
  float rel[4];
  MapRectTranslate(layer, tx, ty, rel);
  std::memcpy(g.log, layer, sizeof layer);
  g.off[0] = 0.f + rel[0];
  g.off[1] = 0.f + rel[1];
  g.w = (uint32_t)std::ceil(rel[2] - rel[0]);
  g.h = (uint32_t)std::ceil(rel[3] - rel[1]);
  return g;
}

// One canvas of a stream into the batch; returns false on invalid input.
inline int AddStreamCanvas(HostBatch& hb, const StreamView& s) {
  uint32_t cidx = (uint32_t)hb.canvases.size();
  CanvasDesc cd;
  std::memset(&cd, 0, sizeof cd);
  cd.w = s.width;
  cd.h = s.height;
  cd.px_off = hb.AllocPixels((uint64_t)s.width * s.height * 4);
  cd.has_clear = s.has_clear;
  cd.clear_pm = s.has_clear ? SolidPM(s.clear) : 0;
  hb.canvases.push_back(cd);
  hb.main_canvases.push_back(cidx);
  hb.image_off.assign(s.n_images, 0);
  for (uint32_t i = 0; i < s.n_images; ++i) {
    const ImageRec& r = s.images[i];
    const uint64_t bytes = (uint64_t)r.width * r.height * 4;
    hb.image_off[i] = hb.AllocPixels(bytes);
    hb.image_uploads.push_back({hb.image_off[i], std::vector<uint8_t>(s.image_pixels + r.offset,
                                                                     s.image_pixels + r.offset + bytes)});
  }
  std::vector<PassDesc> main_passes;
  std::vector<std::pair<uint32_t, std::vector<PassDesc>>> temps;
  // Path clips: one pass rasterising each ClipPath path (RastePath with the
  // canvas matrix and global clip bounds of the call, sw_canvas.cc:317-324),
  // its spans kept raw for the clip stages; states numbered across the
  // batch.
  const uint32_t state_base = (uint32_t)hb.clip_states.size();
  std::vector<uint32_t> clip_pass_pos;
  {
    const uint8_t* v = s.clip_verbs;
    const float* p = s.clip_pts;
    const float* w = s.clip_wts;
    for (uint32_t i = 0; i < s.n_clip_states; ++i) {
      const ClipStateRec& c = s.clip_states[i];
      const uint32_t draw = hb.AddDraw(v, c.nv, p, c.np, w, c.nw);
      PassDesc pd;
      std::memset(&pd, 0, sizeof pd);
      pd.draw = draw;
      pd.canvas = cidx;
      pd.flags = kPassClipPath | kPassRawSpans | (c.fill_type == 1 ? kPassEvenOdd : 0);
      pd.tx = c.translate[0];
      pd.ty = c.translate[1];
      if (s.clip_matrices) {
        const float* m = s.clip_matrices + 6 * (size_t)i;
        pd.tx = m[2];
        pd.ty = m[5];
        if (HasLinear(m)) {
          pd.flags |= kPassMatrix;
          pd.lin[0] = m[0];
          pd.lin[1] = m[1];
          pd.lin[2] = m[3];
          pd.lin[3] = m[4];
        }
      }
      if (!IsNoClip(c.bounds)) {
        pd.clipped = 1;
        std::memcpy(pd.clip, c.bounds, sizeof pd.clip);
      }
      pd.stroke_width = 1.f;
      pd.miter = 4.f;
      pd.ga = 255;
      InitialCaps(v, c.nv, p, false, pd.cap);
      DerivedCaps(pd.cap, false);
      clip_pass_pos.push_back((uint32_t)main_passes.size());
      main_passes.push_back(pd);
      ClipStateDesc st;
      std::memset(&st, 0, sizeof st);
      st.parent = c.parent ? state_base + c.parent : 0;
      st.op = c.op;
      hb.clip_states.push_back(st);
      v += c.nv;
      p += 2 * (size_t)c.np;
      w += c.nw;
    }
  }
  // Layers: each saved layer is a temp canvas (a zeroed bitmap over its
  // device bounds) holding the passes of its draws, and at its restore an
  // image pass draws it onto the canvas (SWCanvas::OnLayerRestore,
  // sw_canvas.cc:891-902).
  uint32_t li = 0;                 // next layer of the stream
  const LayerRec* layer = nullptr; // the open layer
  LayerGeom lg;
  uint32_t ltemp = 0;              // its temp canvas (0: none, the bitmap is empty)
  size_t ltemp_slot = 0;           // its entry in `temps`
  auto restore_layer = [&]() {
    if (ltemp) {
      // DrawImage(layer bitmap, log_bounds, &paint) with drawing_layer set:
      // a rect path with a decal / nearest pixmap brush whose unit
      // coordinates are Scale(1/w, 1/h) * inverse(local) * Scale(1/B.W,
      // 1/B.H) * Translate(-B.L, -B.T), local = Scale(1/w, 1/h) and B the
      // drawn rect's device bounds rounded out (OnDrawImageRect
      // sw_canvas.cc:659-662, GenerateBrush :772-784, SWRaster bounds_
      // sw_raster.cc:742-744)
      const LayerRec& L = *layer;
      const float tx = L.translate[0], ty = L.translate[1];
      const uint8_t rv[5] = {kMove, kLine, kLine, kLine, kClose};
      const float rp[8] = {lg.log[0], lg.log[1], lg.log[2], lg.log[1],
                           lg.log[2], lg.log[3], lg.log[0], lg.log[3]};
      float bl = 0, bt = 0, br = 0, bb = 0;
      for (int i = 0; i < 4; ++i) {
        // CopyWithMatrix(Translate(tx, ty)): (1*x + 0*y) + (0*0 + tx*1)
        const float x = (1.f * rp[2 * i] + 0.f * rp[2 * i + 1]) + (0.f * 0.f + tx * 1.f);
        const float y = (0.f * rp[2 * i] + 1.f * rp[2 * i + 1]) + (0.f * 0.f + ty * 1.f);
        if (i == 0) {
          bl = br = x;
          bt = bb = y;
        }
        bl = std::min(bl, x);
        br = std::max(br, x);
        bt = std::min(bt, y);
        bb = std::max(bb, y);
      }
      bl = std::floor(bl);
      bt = std::floor(bt);
      br = std::ceil(br);
      bb = std::ceil(bb);
      const float fw = (float)lg.w, fh = (float)lg.h;
      const Mat4 local = MatMul(MatScale(1.f / fw, 1.f / fh), MatTranslate(-0.f, -0.f));
      Mat4 inv;  // Matrix::Invert (matrix.cc:134-142, 242-266)
      inv.identity();
      if (!local.is_identity()) {
        const float sx = local.e[0][0], sy = local.e[1][1];
        if (sx != 1.f || sy != 1.f) {
          const float ix = 1.f / sx, iy = 1.f / sy;
          inv.e[0][0] = ix;
          inv.e[1][1] = iy;
          inv.e[3][0] = -local.e[3][0] * ix;
          inv.e[3][1] = -local.e[3][1] * iy;
        } else {
          inv.e[3][0] = -local.e[3][0];
          inv.e[3][1] = -local.e[3][1];
        }
      }
      const Mat4 m = MatMul(MatMul(MatMul(MatScale(1.f / fw, 1.f / fh), inv),
                                   MatScale(1.0f / (br - bl), 1.0f / (bb - bt))),
                            MatTranslate(-bl, -bt));
      const uint32_t rect = hb.AddDraw(rv, 5, rp, 4, nullptr, 0);
      Brush b;
      std::memset(&b, 0, sizeof b);
      b.kind = 3;
      b.blend = L.blend;
      b.global_alpha = (uint8_t)(255 * L.alpha);
      b.m[0] = m.e[0][0];
      b.m[1] = m.e[1][0];
      b.m[2] = m.e[3][0];
      b.m[3] = m.e[0][1];
      b.m[4] = m.e[1][1];
      b.m[5] = m.e[3][1];
      b.img_w = lg.w;
      b.img_h = lg.h;
      b.img_off = hb.canvases[ltemp].px_off;
      hb.brushes.push_back(b);
      PassDesc pd;
      std::memset(&pd, 0, sizeof pd);
      pd.draw = rect;
      pd.canvas = cidx;
      pd.flags = L.blend == 3 ? kPassSrcOver : 0;
      pd.brush = (uint32_t)hb.brushes.size() - 1;
      pd.ga = b.global_alpha;
      pd.tx = tx;
      pd.ty = ty;
      if (!IsNoClip(L.clip)) {  // the global clip bounds after the restore
        pd.clipped = 1;
        std::memcpy(pd.clip, L.clip, sizeof pd.clip);
      }
      pd.stroke_width = 1.f;
      pd.miter = 4.f;
      InitialCaps(rv, 5, rp, false, pd.cap);
      DerivedCaps(pd.cap, false);
      main_passes.push_back(pd);
    }
    layer = nullptr;
    ltemp = 0;
  };
  auto layer_events = [&](uint32_t d) -> int {
    if (layer && layer->restore == d) restore_layer();
    while (!layer && li < s.n_layers && s.layers[li].start == d) {
      layer = &s.layers[li++];
      lg = LayerGeometry(s, *layer);
      if (lg.w > 0 && lg.h > 0) {
        if (lg.w > 65535 || lg.h > 65535) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
        ltemp = (uint32_t)hb.canvases.size();
        CanvasDesc tc;
        std::memset(&tc, 0, sizeof tc);
        tc.w = lg.w;
        tc.h = lg.h;
        tc.px_off = hb.AllocPixels((uint64_t)lg.w * lg.h * 4);
        tc.blur_off = tc.out_off = tc.px_off;
        tc.has_clear = 1;  // a zeroed premultiplied bitmap (LayerState::Init)
        tc.clear_pm = 0;
        tc.blur_style = 0;  // a layer, not a blur: the blur stage passes it by
        hb.canvases.push_back(tc);
        hb.temp_canvases.push_back(ltemp);
        ltemp_slot = temps.size();
        temps.emplace_back(ltemp, std::vector<PassDesc>());
      }
      if (layer->restore == d) restore_layer();
    }
    return SKITY_CUDA_SUCCESS;
  };
  for (uint32_t d = 0; d < s.nd; ++d) {
    const PaintRec& pr = s.paints[d];
    const uint32_t path_clip = s.draw_clip_state ? s.draw_clip_state[d] : 0u;
    if (pr.blend > 28) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;  // past kLuminosity
    if (int rc = layer_events(d)) return rc;
    uint32_t draw = hb.AddDraw(s.verbs + s.vo[d], s.vo[d + 1] - s.vo[d], s.pts + 2 * (size_t)s.po[d],
                               s.po[d + 1] - s.po[d], s.wts + s.wo[d], s.wo[d + 1] - s.wo[d]);
    hb.draw_count++;
    bool blur = pr.blur_style != 0 && pr.blur_radius > 0;  // MakeBlur(r <= 0) is null
    // the draw's canvas matrix: the stream's, or the paint's translation
    float ctm[6] = {1.f, 0.f, pr.translate[0], 0.f, 1.f, pr.translate[1]};
    if (s.matrices) std::memcpy(ctm, s.matrices + 6 * (size_t)d, sizeof ctm);
    const bool lin = HasLinear(ctm);
    if (layer) {
      // a draw inside the layer: the sub-canvas's transform
      // Translate(-origin) * CTM (sw_canvas.hpp:179-182), its clip moved by
      // -origin; blurs, path clips and matrices past a translation inside
      // layers are not taken
      if (blur || path_clip || lin) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
      if (!ltemp) continue;  // an empty layer bitmap: nothing lands
      const float shift[2] = {-lg.off[0], -lg.off[1]};
      const float moved[6] = {1.f, 0.f, ctm[2] + shift[0], 0.f, 1.f, ctm[5] + shift[1]};
      if (int rc = AddDrawPasses(hb, s, d, draw, ltemp, moved, temps[ltemp_slot].second, shift))
        return rc;
      continue;
    }
    if (!blur) {
      // the canvas matrix goes where the reference's CopyWithMatrix and
      // device_to_local put it (sw_raster.cc:736-754, sw_canvas.cc:727-795)
      const size_t first_pass = main_passes.size();
      if (int rc = AddDrawPasses(hb, s, d, draw, cidx, ctm, main_passes)) return rc;
      if (path_clip) {  // DoBrush clips the raster's spans by the state (sw_canvas.cc:338-353)
        for (size_t q = first_pass; q < main_passes.size(); ++q) {
          main_passes[q].path_clip = state_base + path_clip;
          main_passes[q].flags |= kPassRawSpans;
        }
      }
      continue;
    }
    // the filtered bitmap's image draw inverts the canvas matrix: scale and
    // translate only (the short inverse, matrix.cc:242-268)
    if (ctm[1] != 0.f || ctm[3] != 0.f) return SKITY_CUDA_ERROR_NOT_SUPPORTED;
    if (pr.blur_style > 4) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;  // past BlurStyle::kInner
    // SWCanvas::HandleFilter: bounds of the source path (path.cc:1341-1360)
    const float* p = s.pts + 2 * (size_t)s.po[d];
    uint32_t np = s.po[d + 1] - s.po[d];
    uint32_t nv = s.vo[d + 1] - s.vo[d];
    if (nv > 1 && s.verbs[s.vo[d] + nv - 1] == kMove) np--;
    float l = 0, t = 0, r = 0, b = 0;
    if (np > 0) {
      l = r = p[0];
      t = b = p[1];
      for (uint32_t i = 1; i < np; ++i) {
        l = std::min(l, p[2 * i]);
        r = std::max(r, p[2 * i]);
        t = std::min(t, p[2 * i + 1]);
        b = std::max(b, p[2 * i + 1]);
      }
    }
    if (pr.style != 0) {  // ComputeBoundsIfStroke (sw_canvas.cc:135-144)
      float sw = pr.stroke_width;
      l = std::floor(l - sw);
      t = std::floor(t - sw);
      r = std::floor(r + sw);
      b = std::floor(b + sw);
    }
    float rad = pr.blur_radius;
    float fl = std::floor(l - rad), ft = std::floor(t - rad);  // image_filter.cc:33-41
    float fr = std::ceil(r + rad), fb = std::ceil(b + rad);
    uint32_t fw = (uint32_t)(fr - fl), fh = (uint32_t)(fb - ft);
    if (fw == 0 || fh == 0 || fw > 65535 || fh > 65535) continue;
    // temp canvas (zeroed premul bitmap), the draw translated by -(fl, ft)
    uint32_t tidx = (uint32_t)hb.canvases.size();
    CanvasDesc tc;
    std::memset(&tc, 0, sizeof tc);
    tc.w = fw;
    tc.h = fh;
    tc.px_off = hb.AllocPixels((uint64_t)fw * fh * 4);
    tc.blur_off = hb.AllocPixels((uint64_t)fw * fh * 4);
    tc.has_clear = 1;
    tc.clear_pm = 0;
    tc.blur_radius = (int32_t)std::round(std::max(rad, rad));
    tc.blur_style = pr.blur_style;
    // MaskFilterOnFilter (mask_filter.cc:51-103): kNormal draws the blurred
    // bitmap; the other styles combine it with the unblurred one, kept
    tc.out_off = pr.blur_style == 1 ? tc.px_off : hb.AllocPixels((uint64_t)fw * fh * 4);
    hb.canvases.push_back(tc);
    hb.temp_canvases.push_back(tidx);
    hb.max_temp_w = std::max(hb.max_temp_w, fw);
    hb.max_temp_h = std::max(hb.max_temp_h, fh);
    hb.max_temp_style = std::max<uint32_t>(hb.max_temp_style, pr.blur_style);
    std::vector<PassDesc> tp;
    // a fresh software canvas: no clip of the main canvas applies there
    const float to_temp[6] = {1.f, 0.f, -fl, 0.f, 1.f, -ft};
    if (int rc = AddDrawPasses(hb, s, d, draw, tidx, to_temp, tp, nullptr, false)) return rc;
    temps.emplace_back(tidx, std::move(tp));
    // DrawImage(blurred, filter_bounds, &paint) (sw_canvas.cc:641-677): a
    // rect path with a decal/nearest pixmap brush, alpha = paint alpha, drawn
    // under the canvas matrix, the global clip bounds and the path clip of
    // the draw (the temp canvas had none of them)
    const uint8_t rv[5] = {kMove, kLine, kLine, kLine, kClose};
    const float rp[8] = {fl, ft, fr, ft, fr, fb, fl, fb};
    uint32_t rect = hb.AddDraw(rv, 5, rp, 4, nullptr, 0);
    Brush br;
    std::memset(&br, 0, sizeof br);
    br.kind = 3;
    br.blend = pr.blend;
    br.global_alpha = (uint8_t)(255 * pr.fill_color[3]);
    Mat4 local = MatMul(MatMul(MatTranslate(fl, ft),
                               MatScale((fr - fl) / (float)fw, (fb - ft) / (float)fh)),
                        MatTranslate(-0.f, -0.f));
    Mat4 inv;
    inv.identity();
    if (!local.is_identity()) {
      inv.e[3][0] = -local.e[3][0];
      inv.e[3][1] = -local.e[3][1];
    }
    // GenerateBrush: Scale(1/w, 1/h) * inverse(local) * inverse(CTM)
    // (sw_canvas.cc:762-777)
    Mat4 m = MatMul(MatMul(MatScale(1.f / fw, 1.f / fh), inv), InvertScaleTranslate(ctm));
    br.m[0] = m.e[0][0];
    br.m[1] = m.e[1][0];
    br.m[2] = m.e[3][0];
    br.m[3] = m.e[0][1];
    br.m[4] = m.e[1][1];
    br.m[5] = m.e[3][1];
    br.img_w = fw;
    br.img_h = fh;
    br.img_off = tc.out_off;
    SetColorFilter(hb, s, d, &br);  // the image draw's paint keeps the filter
    hb.brushes.push_back(br);
    PassDesc pd;
    std::memset(&pd, 0, sizeof pd);
    pd.draw = rect;
    pd.canvas = cidx;
    pd.flags = (pr.blend == 3 && !FiltersColor(s, d)) ? kPassSrcOver : 0;
    pd.brush = (uint32_t)hb.brushes.size() - 1;
    pd.ga = br.global_alpha;
    pd.stroke_width = 1.f;
    pd.miter = 4.f;
    pd.tx = ctm[2];
    pd.ty = ctm[5];
    if (lin) {
      pd.flags |= kPassMatrix;
      pd.lin[0] = ctm[0];
      pd.lin[1] = ctm[1];
      pd.lin[2] = ctm[3];
      pd.lin[3] = ctm[4];
    }
    if (s.clips && !IsNoClip(s.clips + 4 * (size_t)d)) {
      pd.clipped = 1;
      std::memcpy(pd.clip, s.clips + 4 * (size_t)d, sizeof pd.clip);
    }
    if (path_clip) {  // DoBrush clips the rect's spans by the state (sw_canvas.cc:338-353)
      pd.path_clip = state_base + path_clip;
      pd.flags |= kPassRawSpans;
    }
    InitialCaps(rv, 5, rp, false, pd.cap);
    DerivedCaps(pd.cap, false);
    main_passes.push_back(pd);
  }
  if (int rc = layer_events(s.nd)) return rc;
  // canvases with passes the compositor's common form does not take
  auto general = [&](const std::vector<PassDesc>& ps) {
    for (const PassDesc& pd : ps) {
      if (pd.flags & kPassClipPath) continue;
      const Brush& br = hb.brushes[pd.brush];
      if (br.kind >= 4 || br.cf_type != 0 || br.blend > 3) return 1u;
    }
    return 0u;
  };
  hb.canvases[cidx].general = general(main_passes);
  for (auto& tpp : temps) hb.canvases[tpp.first].general = general(tpp.second);
  hb.canvases[cidx].pass0 = (uint32_t)hb.passes.size();
  for (uint32_t i = 0; i < (uint32_t)clip_pass_pos.size(); ++i)
    hb.clip_states[state_base + i].pass = hb.canvases[cidx].pass0 + clip_pass_pos[i];
  hb.passes.insert(hb.passes.end(), main_passes.begin(), main_passes.end());
  hb.canvases[cidx].pass1 = (uint32_t)hb.passes.size();
  for (auto& tpp : temps) {
    hb.canvases[tpp.first].pass0 = (uint32_t)hb.passes.size();
    hb.passes.insert(hb.passes.end(), tpp.second.begin(), tpp.second.end());
    hb.canvases[tpp.first].pass1 = (uint32_t)hb.passes.size();
  }
  return SKITY_CUDA_SUCCESS;
}

// Where a batch of canvases (built into an empty HostBatch) lands in a
// larger one: the sizes of the larger batch's arrays before it, and its
// first pixel byte.
struct BatchBase {
  size_t verbs = 0, pts = 0, weights = 0, draws = 0, passes = 0, brushes = 0, conicals = 0,
         cf = 0, clip_states = 0, canvases = 0, stops = 0, temps = 0, mains = 0;
  uint64_t px = 0;
  // the base of the batch after `l`
  BatchBase after(const HostBatch& l) const {
    BatchBase n;
    n.verbs = verbs + l.verbs.size();
    n.pts = pts + l.pts.size();
    n.weights = weights + l.weights.size();
    n.draws = draws + l.draws.size();
    n.passes = passes + l.passes.size();
    n.brushes = brushes + l.brushes.size();
    n.conicals = conicals + l.conicals.size();
    n.cf = cf + l.cf_matrices.size();
    n.clip_states = clip_states + l.clip_states.size();
    n.canvases = canvases + l.canvases.size();
    n.stops = stops + l.stop_colors.size();
    n.temps = temps + l.temp_canvases.size();
    n.mains = mains + l.main_canvases.size();
    n.px = px + l.pixel_bytes;
    return n;
  }
};

// Copies batch `l` into `g` (arrays already sized for it) at base `b`,
// moving every index and byte offset of `l` by the base: the result is the
// batch AddStreamCanvas builds by adding l's canvases to g one after the
// other.  b.px is 256-byte aligned, as AllocPixels places a canvas.
inline void PlaceBatch(HostBatch& g, const HostBatch& l, const BatchBase& b) {
  std::copy(l.verbs.begin(), l.verbs.end(), g.verbs.begin() + b.verbs);
  std::copy(l.pts.begin(), l.pts.end(), g.pts.begin() + b.pts);
  std::copy(l.weights.begin(), l.weights.end(), g.weights.begin() + b.weights);
  std::copy(l.conicals.begin(), l.conicals.end(), g.conicals.begin() + b.conicals);
  std::copy(l.cf_matrices.begin(), l.cf_matrices.end(), g.cf_matrices.begin() + b.cf);
  std::copy(l.stop_colors.begin(), l.stop_colors.end(), g.stop_colors.begin() + b.stops);
  std::copy(l.stop_offsets.begin(), l.stop_offsets.end(), g.stop_offsets.begin() + b.stops);
  for (size_t i = 0; i < l.draws.size(); ++i) {
    DrawDesc d = l.draws[i];
    d.v0 += (uint32_t)b.verbs;
    d.p0 += (uint32_t)b.pts;
    d.w0 += (uint32_t)b.weights;
    g.draws[b.draws + i] = d;
  }
  for (size_t i = 0; i < l.passes.size(); ++i) {
    PassDesc p = l.passes[i];
    p.draw += (uint32_t)b.draws;
    p.canvas += (uint32_t)b.canvases;
    if (!(p.flags & kPassClipPath)) p.brush += (uint32_t)b.brushes;  // a clip path's pass has none
    if (p.path_clip) p.path_clip += (uint32_t)b.clip_states;
    g.passes[b.passes + i] = p;
  }
  for (size_t i = 0; i < l.brushes.size(); ++i) {
    Brush r = l.brushes[i];
    if (r.kind == 1 || r.kind == 2 || r.kind == 4 || r.kind == 5) r.stop0 += (uint32_t)b.stops;
    if (r.kind == 5) r.conical += (uint32_t)b.conicals;
    if (r.kind == 3 || r.kind == 6) r.img_off += b.px;
    if (r.cf_type == 2) r.cf_index += (uint32_t)b.cf;
    g.brushes[b.brushes + i] = r;
  }
  for (size_t i = 0; i < l.clip_states.size(); ++i) {
    ClipStateDesc c = l.clip_states[i];
    if (c.parent) c.parent += (uint32_t)b.clip_states;
    c.pass += (uint32_t)b.passes;
    g.clip_states[b.clip_states + i] = c;
  }
  for (size_t i = 0; i < l.canvases.size(); ++i) {
    CanvasDesc c = l.canvases[i];
    c.px_off += b.px;
    c.pass0 += (uint32_t)b.passes;
    c.pass1 += (uint32_t)b.passes;
    g.canvases[b.canvases + i] = c;
  }
  for (size_t i = 0; i < l.temp_canvases.size(); ++i) {  // temp canvases own all three buffers
    const uint32_t t = l.temp_canvases[i];
    CanvasDesc& c = g.canvases[b.canvases + t];
    c.blur_off += b.px;
    c.out_off += b.px;
    g.temp_canvases[b.temps + i] = t + (uint32_t)b.canvases;
  }
  for (size_t i = 0; i < l.main_canvases.size(); ++i)
    g.main_canvases[b.mains + i] = l.main_canvases[i] + (uint32_t)b.canvases;
}

// Parses `count` scene streams into `hb` (empty on entry), the canvases in
// stream order.  The streams are cut into runs of consecutive canvases of
// about equal bytes; host threads (up to `threads`) build the runs into
// batches of their own, then copy them into `hb` at the places a one-thread
// loop over AddStreamCanvas gives them, so `hb` is the batch that loop
// builds.  Returns the first failing stream's status (in stream order), or
// success.
inline int32_t BuildStreams(HostBatch& hb, uint32_t count, const uint8_t* const* streams,
                            const size_t* bytes, unsigned threads) {
  auto add_range = [&](HostBatch& b, uint32_t i0, uint32_t i1) -> int32_t {
    for (uint32_t i = i0; i < i1; ++i) {
      StreamView sv;
      if (!ParseStream(streams[i], bytes[i], &sv)) return SKITY_CUDA_ERROR_INVALID_ARGUMENT;
      const int32_t rc = AddStreamCanvas(b, sv);
      if (rc != SKITY_CUDA_SUCCESS) return rc;
    }
    return SKITY_CUDA_SUCCESS;
  };
  if (threads > count / 4) threads = count / 4;
  if (threads < 2) return add_range(hb, 0, count);
  uint64_t total = 0;
  for (uint32_t i = 0; i < count; ++i) total += bytes[i] + 64;
  // runs of about total / (4 * threads) bytes: the threads take them in
  // order from a counter, so a heavy run does not hold the others up
  const uint64_t target = total / (4 * (uint64_t)threads) + 1;
  std::vector<uint32_t> cut{0};
  uint64_t acc = 0;
  for (uint32_t i = 0; i < count; ++i) {
    acc += bytes[i] + 64;
    if (acc >= target && i + 1 < count) {
      cut.push_back(i + 1);
      acc = 0;
    }
  }
  cut.push_back(count);
  const uint32_t runs = (uint32_t)cut.size() - 1;
  std::vector<HostBatch> part(runs);
  std::vector<int32_t> rc(runs, SKITY_CUDA_SUCCESS);
  std::vector<BatchBase> base(runs);
  auto parallel = [&](auto&& body) {
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
      for (uint32_t r; (r = next.fetch_add(1)) < runs;) body(r);
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
  };
  parallel([&](uint32_t r) { rc[r] = add_range(part[r], cut[r], cut[r + 1]); });
  for (uint32_t r = 0; r < runs; ++r)
    if (rc[r] != SKITY_CUDA_SUCCESS) return rc[r];
  BatchBase end;
  for (uint32_t r = 0; r < runs; ++r) {
    end.px = (end.px + 255) & ~uint64_t(255);  // every run starts with a canvas
    base[r] = end;
    end = end.after(part[r]);
  }
  hb.verbs.resize(end.verbs);
  hb.pts.resize(end.pts);
  hb.weights.resize(end.weights);
  hb.draws.resize(end.draws);
  hb.passes.resize(end.passes);
  hb.brushes.resize(end.brushes);
  hb.conicals.resize(end.conicals);
  hb.cf_matrices.resize(end.cf);
  hb.clip_states.resize(end.clip_states);
  hb.canvases.resize(end.canvases);
  hb.stop_colors.resize(end.stops);
  hb.stop_offsets.resize(end.stops);
  hb.temp_canvases.resize(end.temps);
  hb.main_canvases.resize(end.mains);
  parallel([&](uint32_t r) { PlaceBatch(hb, part[r], base[r]); });
  for (uint32_t r = 0; r < runs; ++r) {
    for (auto& u : part[r].image_uploads)
      hb.image_uploads.push_back({u.off + base[r].px, std::move(u.bytes)});
    hb.draw_count += part[r].draw_count;
    hb.max_temp_w = std::max(hb.max_temp_w, part[r].max_temp_w);
    hb.max_temp_h = std::max(hb.max_temp_h, part[r].max_temp_h);
    hb.max_temp_style = std::max(hb.max_temp_style, part[r].max_temp_style);
  }
  hb.pixel_bytes = end.px;
  return SKITY_CUDA_SUCCESS;
}

// Gives every canvas its range of row bands (1 << shift rows each);
// returns the number of bands.
inline uint32_t AssignBands(HostBatch& hb, int shift) {
  uint32_t n = 0;
  for (CanvasDesc& cd : hb.canvases) {
    cd.band0 = n;
    n += (cd.h + (1u << shift) - 1) >> shift;
  }
  return n;
}
// The compositor's pass bins: for every row band, the passes (in pass
// order, which is draw order within a canvas) that have rows in it.
inline void BuildBins(const HostBatch& hb, const std::vector<PassComp>& comp, uint32_t n_bands,
                      int shift, std::vector<uint32_t>& band_off, std::vector<uint32_t>& bins) {
  band_off.assign((size_t)n_bands + 1, 0);
  for (size_t p = 0; p < comp.size(); ++p) {
    const PassComp& c = comp[p];
    if (c.row1 <= c.row0) continue;
    const uint32_t b0 = hb.canvases[hb.passes[p].canvas].band0;
    for (int32_t k = c.row0 >> shift; k <= (c.row1 - 1) >> shift; ++k)
      band_off[b0 + (uint32_t)k + 1]++;
  }
  for (uint32_t i = 0; i < n_bands; ++i) band_off[i + 1] += band_off[i];
  bins.assign(std::max<size_t>(band_off[n_bands], 1), 0);
  std::vector<uint32_t> fill(band_off.begin(), band_off.end() - 1);
  for (size_t p = 0; p < comp.size(); ++p) {
    const PassComp& c = comp[p];
    if (c.row1 <= c.row0) continue;
    const uint32_t b0 = hb.canvases[hb.passes[p].canvas].band0;
    for (int32_t k = c.row0 >> shift; k <= (c.row1 - 1) >> shift; ++k)
      bins[fill[b0 + (uint32_t)k]++] = (uint32_t)p;
  }
}

// Row tiles in the order the compositor should take them: most work first
// (passes in the tile's band times its width), so that the heavy tiles do
// not form the tail of the launch.
inline void OrderRowTasks(const HostBatch& hb, const std::vector<uint32_t>& band_off, int shift,
                          std::vector<RowTask>& tasks) {
  std::vector<uint64_t> cost(tasks.size());
  for (size_t i = 0; i < tasks.size(); ++i) {
    const RowTask& t = tasks[i];
    const uint32_t band = hb.canvases[t.canvas].band0 + (t.y >> shift);
    cost[i] = (uint64_t)(band_off[band + 1] - band_off[band] + 1) * (t.x1 - t.x0);
  }
  std::vector<uint32_t> idx(tasks.size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = (uint32_t)i;
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
  std::vector<RowTask> out(tasks.size());
  for (size_t i = 0; i < idx.size(); ++i) out[i] = tasks[idx[i]];
  tasks.swap(out);
}

// Pass-bin segments of the device planner: for every band of every canvas,
// in band order, runs of at most kSegPasses of the canvas's passes (a band
// of a canvas without passes gets one empty segment, so every band has one).
constexpr uint32_t kSegPasses = 1024;
inline void BuildBandSegs(const HostBatch& hb, int shift, std::vector<BandSeg>& segs) {
  segs.clear();
  for (const CanvasDesc& cd : hb.canvases) {
    const uint32_t nb = (cd.h + (1u << shift) - 1) >> shift;
    for (uint32_t k = 0; k < nb; ++k) {
      uint32_t p0 = cd.pass0;
      bool first = true;
      do {
        const uint32_t p1 = std::min<uint32_t>(cd.pass1, p0 + kSegPasses);
        segs.push_back(BandSeg{cd.band0 + k, p0, p1, first ? 1u : 0u});
        first = false;
        p0 = p1;
      } while (p0 < cd.pass1);
    }
  }
}

inline void BuildRowTasks(const HostBatch& hb, const std::vector<uint32_t>& canv, uint32_t chunk,
                          std::vector<RowTask>& out) {
  out.clear();
  for (uint32_t c : canv) {
    const CanvasDesc& cd = hb.canvases[c];
    for (uint32_t y = 0; y < cd.h; ++y)
      for (uint32_t x0 = 0; x0 < cd.w; x0 += chunk)
        out.push_back(RowTask{c, y, x0, std::min(cd.w, x0 + chunk)});
  }
}


// Per-pass sweep buffers and row-span tables from the geometry results.
struct SweepPlan {
  uint64_t sweep_bytes = 0, rows = 0, edges = 0;
  uint64_t span_estimate = 0;  // first guess of the span pool size
  int32_t max_acc = 0;  // largest accumulator (acc_width + 1) of a swept pass
};
// Accumulator entries each register-sweep warp keeps in shared memory.
inline int32_t RegDiffCap(const SweepPlan& pl) {
  int32_t c = (pl.max_acc + 3) & ~3;
  return std::max<int32_t>(4, std::min<int32_t>(c, kRegDiffMax));
}
inline SweepPlan PlanSweep(const HostBatch& hb, const std::vector<PassGeom>& geom,
                           std::vector<PassSweep>& sw) {
  SweepPlan pl;
  sw.assign(geom.size(), PassSweep{});
  for (size_t p = 0; p < geom.size(); ++p) {
    const PassGeom& g = geom[p];
    const CanvasDesc& cd = hb.canvases[hb.passes[p].canvas];
    sw[p].work_off = pl.sweep_bytes;
    sw[p].rbase = (uint32_t)pl.rows;
    sw[p].chunk = SpanChunk(cd.w, g.n_edges);
    const int nr = g.row1 - g.row0;
    if (g.n_edges > 0 && nr > 0) {
      uint64_t b = SweepMemBytes(g.n_edges, std::max(g.acc_width, 0));
      b = (b + 255) & ~uint64_t(255);
      sw[p].bytes = b;
      pl.sweep_bytes += b;
      pl.max_acc = std::max(pl.max_acc, std::max(g.acc_width, 0) + 1);
      pl.span_estimate += (uint64_t)nr * 32 + sw[p].chunk;
    }
    if (g.n_edges > 0) pl.edges += (uint64_t)g.n_edges;
    if (nr > 0) pl.rows += (uint64_t)nr;
  }
  return pl;
}
// Compositor inputs per pass.
inline void PlanComp(const HostBatch& hb, const std::vector<PassGeom>& geom,
                     const std::vector<PassSweep>& sw, std::vector<PassComp>& comp) {
  comp.assign(geom.size(), PassComp{});
  for (size_t p = 0; p < geom.size(); ++p) {
    const PassGeom& g = geom[p];
    const bool has = g.n_edges > 0 && g.row1 > g.row0 && !(hb.passes[p].flags & kPassClipPath);
    comp[p].row0 = has ? g.row0 : 0;
    comp[p].row1 = has ? g.row1 : 0;
    comp[p].rbase = sw[p].rbase;
    comp[p].brush = hb.passes[p].brush;
  }
}
// Rows of the clip states (their clip path's rows and their parent's) and
// the (pass, row) items of the draws under a path clip; returns the number
// of state rows.
inline uint64_t PlanPathClips(HostBatch& hb, const std::vector<PassGeom>& geom,
                              std::vector<uint2>& items) {
  uint64_t rbase = 0;
  for (ClipStateDesc& st : hb.clip_states) {
    const PassGeom& g = geom[st.pass];
    int32_t y0 = 0, y1 = 0;
    if (g.n_edges > 0 && g.row1 > g.row0) {
      y0 = g.row0;
      y1 = g.row1;
    }
    if (st.parent) {
      const ClipStateDesc& ps = hb.clip_states[st.parent - 1];
      if (ps.y1 > ps.y0) {
        if (y1 > y0) {
          y0 = std::min(y0, ps.y0);
          y1 = std::max(y1, ps.y1);
        } else {
          y0 = ps.y0;
          y1 = ps.y1;
        }
      }
    }
    st.y0 = y0;
    st.y1 = y1;
    st.rbase = (uint32_t)rbase;
    rbase += (uint64_t)(y1 - y0);
  }
  items.clear();
  for (uint32_t p = 0; p < (uint32_t)hb.passes.size(); ++p) {
    if (!hb.passes[p].path_clip) continue;
    const PassGeom& g = geom[p];
    if (g.n_edges <= 0) continue;
    for (int32_t y = g.row0; y < g.row1; ++y) items.push_back(make_uint2(p, (uint32_t)y));
  }
  return rbase;
}

// The order in which the sweeps take the passes: longest expected sweep
// first (rows times the bound of the active list), so that the long sweeps
// start early instead of forming the tail of the launch.
inline void SweepOrder(const std::vector<PassGeom>& geom, std::vector<uint32_t>& order) {
  order.resize(geom.size());
  std::vector<uint64_t> cost(geom.size());
  for (size_t p = 0; p < geom.size(); ++p) {
    order[p] = (uint32_t)p;
    const PassGeom& g = geom[p];
    const int64_t rows = g.n_edges > 0 ? std::max<int64_t>(g.row1 - g.row0, 0) : 0;
    cost[p] = (uint64_t)rows * (uint64_t)(1 + std::max(g.max_active, 0));
  }
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t a, uint32_t b) { return cost[a] > cost[b]; });
}
// Grow the capacities of a pass whose geometry overflowed.
inline void GrowCaps(PassDesc& pd, const PassGeom& g) {
  bool stroke = (pd.flags & kPassStroke) != 0;
  for (int k = 0; k < 13; ++k) pd.cap[k] = std::max(pd.cap[k], g.need[k] + 2);
  DerivedCaps(pd.cap, stroke);
  for (int k = 9; k < 13; ++k) pd.cap[k] = std::max(pd.cap[k], g.need[k] + 2);
}

}  // namespace skc
