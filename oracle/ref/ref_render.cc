// Reference renderer: replays a scene stream (skity_gb300/scene.py layout)
// through the UNMODIFIED reference software backend -- Canvas::
// MakeSoftwareCanvas(Bitmap*) (src/render/sw/sw_canvas.cc:146-156), Clear,
// one DrawPath per draw, Flush -- and writes the premultiplied RGBA8 pixels.
//
// Built only from the reference sources by oracle/ref/Makefile into
// oracle/_ref/ref_render. Test infrastructure: golden vectors and the oracle
// pin come from here.
//
// usage: ref_render <scene.bin> <out.rgba> [first count] [--time]
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <skity/effect/color_filter.hpp>
#include <skity/effect/mask_filter.hpp>
#include <skity/effect/shader.hpp>
#include <skity/graphic/bitmap.hpp>
#include <skity/graphic/paint.hpp>
#include <skity/graphic/path.hpp>
#include <skity/render/canvas.hpp>
#include <string>
#include <vector>

#include "src/effect/gradient_shader.hpp"  // the sweep / conical shader classes

namespace {

struct PaintRec {
  uint32_t style, cap, join, blend, fill_type;
  int32_t gradient;
  uint32_t blur_style;
  float blur_radius;
  float fill_color[4];
  float stroke_color[4];
  float stroke_width, miter;
  float translate[2];  // Canvas::Translate in effect for the draw
};
static_assert(sizeof(PaintRec) == 80, "paint record layout");

struct GradRec {
  uint32_t type, tile_mode, stop_count, stop_start, has_offsets, reserved;
  float p0[2], p1[2], radius[2];
};
static_assert(sizeof(GradRec) == 48, "gradient record layout");

struct Scene {
  uint32_t width = 0, height = 0, has_clear = 0;
  float clear[4] = {0, 0, 0, 0};
  std::vector<uint32_t> vo, po, wo;
  std::vector<uint8_t> verbs;
  std::vector<float> pts, wts;
  std::vector<PaintRec> paints;
  std::vector<GradRec> grads;
  std::vector<float> stop_colors, stop_offsets;
  std::vector<float> clips;  // per draw device-space (l, t, r, b), when present
  struct Filter {
    uint32_t type, mode, color, pad;
    float matrix[20];
  };
  std::vector<Filter> filters;  // per draw colour filter, when present
  struct ClipState {
    uint32_t parent, op, fill_type, nv, np, nw;
    float translate[2], bounds[4];
  };
  std::vector<ClipState> clip_states;  // path clips, when present
  std::vector<uint8_t> clip_verbs;
  std::vector<float> clip_pts, clip_wts;
  std::vector<uint32_t> draw_clip_state;  // per draw, 1-based (0: none)
  struct Layer {  // Canvas::SaveLayer ... Restore around draws [start, restore)
    float bounds[4], translate[2], clip[4];
    uint32_t start, restore;
    float alpha;
    uint32_t blend, pad[2];
  };
  std::vector<Layer> layers;
  std::vector<float> matrices;  // per draw (sx, kx, tx, ky, sy, ty), or empty
  std::vector<float> clip_matrices;  // per clip state, or empty: their translations
};

template <typename T>
void Take(const std::vector<char>& buf, size_t& o, std::vector<T>& dst,
          size_t n) {
  dst.resize(n);
  if (n) std::memcpy(dst.data(), buf.data() + o, n * sizeof(T));
  o += n * sizeof(T);
}

bool Load(const char* path, Scene* s) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::vector<char> buf((std::istreambuf_iterator<char>(f)),
                        std::istreambuf_iterator<char>());
  if (buf.size() < 80 || std::memcmp(buf.data(), "SKSC", 4) != 0) return false;
  uint32_t hdr[7];
  std::memcpy(hdr, buf.data() + 4, sizeof(hdr));
  if (hdr[0] != 1) return false;
  s->width = hdr[1];
  s->height = hdr[2];
  s->has_clear = hdr[3];
  const uint32_t flags = hdr[4];  // 1: per-draw clip bounds follow the stops
  size_t o = 32;
  std::memcpy(s->clear, buf.data() + o, 16);
  o += 16;
  uint32_t cnt[6];
  std::memcpy(cnt, buf.data() + o, sizeof(cnt));
  o += sizeof(cnt);
  uint32_t nd = cnt[0];
  Take(buf, o, s->vo, nd + 1);
  Take(buf, o, s->po, nd + 1);
  Take(buf, o, s->wo, nd + 1);
  Take(buf, o, s->verbs, cnt[1]);
  o += (4 - cnt[1] % 4) % 4;
  Take(buf, o, s->pts, 2 * size_t(cnt[2]));
  Take(buf, o, s->wts, cnt[3]);
  Take(buf, o, s->paints, nd);
  Take(buf, o, s->grads, cnt[4]);
  Take(buf, o, s->stop_colors, 4 * size_t(cnt[5]));
  Take(buf, o, s->stop_offsets, cnt[5]);
  if (flags & 1) Take(buf, o, s->clips, 4 * size_t(nd));
  if (flags & 2) Take(buf, o, s->filters, nd);
  if (flags & 4) {
    uint32_t n_states = 0;
    if (o + 4 > buf.size()) return false;
    std::memcpy(&n_states, buf.data() + o, 4);
    o += 4;
    Take(buf, o, s->clip_states, n_states);
    size_t tv = 0, tp = 0, tw = 0;
    for (const auto& c : s->clip_states) {
      tv += c.nv;
      tp += c.np;
      tw += c.nw;
    }
    Take(buf, o, s->clip_verbs, tv);
    o += (4 - tv % 4) % 4;
    Take(buf, o, s->clip_pts, 2 * tp);
    Take(buf, o, s->clip_wts, tw);
    Take(buf, o, s->draw_clip_state, nd);
  }
  if (flags & 8) {  // images: not replayed here, skipped
    uint32_t n_images = 0;
    if (o + 4 > buf.size()) return false;
    std::memcpy(&n_images, buf.data() + o, 4);
    o += 4 + 24 * size_t(n_images);
    uint64_t nb = 0;
    if (o + 8 > buf.size()) return false;
    std::memcpy(&nb, buf.data() + o, 8);
    o += 8 + nb + (4 - nb % 4) % 4 + 80 * size_t(nd);
  }
  if (flags & 16) {
    uint32_t n_layers = 0;
    if (o + 4 > buf.size()) return false;
    std::memcpy(&n_layers, buf.data() + o, 4);
    o += 4;
    Take(buf, o, s->layers, n_layers);
  }
  if (flags & 32) Take(buf, o, s->matrices, 6 * size_t(nd));
  if (flags & 64) Take(buf, o, s->clip_matrices, 6 * s->clip_states.size());
  return o <= buf.size();
}

skity::Path BuildPathFrom(const uint8_t* verbs, uint32_t nv, const float* p,
                          const float* w) {
  skity::Path path;
  for (uint32_t v = 0; v < nv; ++v) {
    switch (verbs[v]) {
      case 0: path.MoveTo(p[0], p[1]); p += 2; break;
      case 1: path.LineTo(p[0], p[1]); p += 2; break;
      case 2: path.QuadTo(p[0], p[1], p[2], p[3]); p += 4; break;
      case 3: path.ConicTo(p[0], p[1], p[2], p[3], *w++); p += 4; break;
      case 4: path.CubicTo(p[0], p[1], p[2], p[3], p[4], p[5]); p += 6; break;
      case 5: path.Close(); break;
      default: break;
    }
  }
  return path;
}

// Replays the ClipPath calls of clip state k (1-based) and its ancestors,
// each with the global clip bounds and translation it was made under.
void ReplayClipState(const Scene& s, skity::Canvas* canvas, uint32_t k) {
  if (k == 0 || k > s.clip_states.size()) return;
  const Scene::ClipState& c = s.clip_states[k - 1];
  ReplayClipState(s, canvas, c.parent);
  size_t v0 = 0, p0 = 0, w0 = 0;
  for (uint32_t i = 0; i + 1 < k; ++i) {
    v0 += s.clip_states[i].nv;
    p0 += s.clip_states[i].np;
    w0 += s.clip_states[i].nw;
  }
  skity::Path path = BuildPathFrom(s.clip_verbs.data() + v0, c.nv, s.clip_pts.data() + 2 * p0,
                                   s.clip_wts.data() + w0);
  if (c.fill_type == 1) path.SetFillType(skity::Path::PathFillType::kEvenOdd);
  canvas->ClipRect(skity::Rect::MakeLTRB(c.bounds[0], c.bounds[1], c.bounds[2], c.bounds[3]));
  if (!s.clip_matrices.empty()) {
    // the canvas matrix of the call, then back to the identity the draw's
    // replay starts from (a Restore would drop the clip as well)
    const float* mx = s.clip_matrices.data() + 6 * (k - 1);
    const float nine[9] = {mx[0], mx[1], mx[2], mx[3], mx[4], mx[5], 0.f, 0.f, 1.f};
    skity::Matrix m;
    m.Set9(nine);
    canvas->SetMatrix(m);
    canvas->ClipPath(path, static_cast<skity::Canvas::ClipOp>(c.op));
    canvas->ResetMatrix();
    return;
  }
  canvas->Translate(c.translate[0], c.translate[1]);
  canvas->ClipPath(path, static_cast<skity::Canvas::ClipOp>(c.op));
  canvas->Translate(-c.translate[0], -c.translate[1]);
}

skity::Path BuildPath(const Scene& s, uint32_t d) {
  skity::Path path;
  const float* p = s.pts.data() + 2 * size_t(s.po[d]);
  const float* w = s.wts.data() + s.wo[d];
  for (uint32_t v = s.vo[d]; v < s.vo[d + 1]; ++v) {
    switch (s.verbs[v]) {
      case 0: path.MoveTo(p[0], p[1]); p += 2; break;
      case 1: path.LineTo(p[0], p[1]); p += 2; break;
      case 2: path.QuadTo(p[0], p[1], p[2], p[3]); p += 4; break;
      case 3: path.ConicTo(p[0], p[1], p[2], p[3], *w++); p += 4; break;
      case 4: path.CubicTo(p[0], p[1], p[2], p[3], p[4], p[5]); p += 6; break;
      case 5: path.Close(); break;
      default: break;
    }
  }
  path.SetFillType(s.paints[d].fill_type == 1
                       ? skity::Path::PathFillType::kEvenOdd
                       : skity::Path::PathFillType::kWinding);
  return path;
}

skity::Paint BuildPaint(const Scene& s, uint32_t d) {
  const PaintRec& r = s.paints[d];
  skity::Paint paint;
  paint.SetStyle(static_cast<skity::Paint::Style>(r.style));
  paint.SetStrokeCap(static_cast<skity::Paint::Cap>(r.cap));
  paint.SetStrokeJoin(static_cast<skity::Paint::Join>(r.join));
  paint.SetBlendMode(static_cast<skity::BlendMode>(r.blend));
  paint.SetFillColor(r.fill_color[0], r.fill_color[1], r.fill_color[2],
                     r.fill_color[3]);
  paint.SetStrokeColor(r.stroke_color[0], r.stroke_color[1], r.stroke_color[2],
                       r.stroke_color[3]);
  paint.SetStrokeWidth(r.stroke_width);
  paint.SetStrokeMiter(r.miter);
  if (r.gradient >= 0) {
    const GradRec& g = s.grads[r.gradient];
    std::vector<skity::Vec4> colors(g.stop_count);
    for (uint32_t i = 0; i < g.stop_count; ++i) {
      const float* c = s.stop_colors.data() + 4 * size_t(g.stop_start + i);
      colors[i] = skity::Vec4{c[0], c[1], c[2], c[3]};
    }
    const float* pos =
        g.has_offsets ? s.stop_offsets.data() + g.stop_start : nullptr;
    auto tile = static_cast<skity::TileMode>(g.tile_mode);
    if (g.type == 1) {
      skity::Point pts[2] = {skity::Point{g.p0[0], g.p0[1], 0, 1},
                             skity::Point{g.p1[0], g.p1[1], 0, 1}};
      paint.SetShader(skity::Shader::MakeLinear(pts, colors.data(), pos,
                                                int(g.stop_count), tile));
    } else if (g.type == 2) {
      paint.SetShader(skity::Shader::MakeRadial(
          skity::Point{g.p0[0], g.p0[1], 0, 1}, g.radius[0], colors.data(),
          pos, int(g.stop_count), tile));
    } else if (g.type == 3 && g.stop_count >= 2) {
      // the record holds the shader's GradientInfo (bias, scale), which is
      // what Shader::MakeSweep builds from its angles (shader.cc:88-104)
      paint.SetShader(std::make_shared<skity::SweepGradientShader>(
          g.p0[0], g.p0[1], g.radius[0], g.radius[1], colors.data(), pos,
          int(g.stop_count), tile, 0));
    } else if (g.type == 4 && g.stop_count >= 2) {
      // the two-point conical shader itself (MakeTwoPointConical's
      // concentric special cases are radial records)
      paint.SetShader(std::make_shared<skity::TwoPointConicalGradientShader>(
          skity::Point{g.p0[0], g.p0[1], 0, 1}, g.radius[0],
          skity::Point{g.p1[0], g.p1[1], 0, 1}, g.radius[1], colors.data(), pos,
          int(g.stop_count), tile, 0));
    }
  }
  if (!s.filters.empty() && s.filters[d].type != 0) {
    const Scene::Filter& f = s.filters[d];
    using skity::ColorFilters;
    switch (f.type) {
      case 1:
        paint.SetColorFilter(ColorFilters::Blend(f.color, static_cast<skity::BlendMode>(f.mode)));
        break;
      case 2:
        paint.SetColorFilter(ColorFilters::Matrix(f.matrix));
        break;
      case 3:
        paint.SetColorFilter(ColorFilters::LinearToSRGBGamma());
        break;
      case 4:
        paint.SetColorFilter(ColorFilters::SRGBToLinearGamma());
        break;
      default:  // a composition (of two gamma filters)
        paint.SetColorFilter(ColorFilters::Compose(ColorFilters::LinearToSRGBGamma(),
                                                   ColorFilters::SRGBToLinearGamma()));
        break;
    }
  }
  if (r.blur_style != 0) {
    paint.SetMaskFilter(skity::MaskFilter::MakeBlur(
        static_cast<skity::BlurStyle>(r.blur_style), r.blur_radius));
  }
  return paint;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s scene.bin out.rgba [first count] [--time]\n",
                 argv[0]);
    return 2;
  }
  Scene s;
  if (!Load(argv[1], &s)) {
    std::fprintf(stderr, "cannot read scene %s\n", argv[1]);
    return 2;
  }
  uint32_t first = 0, count = uint32_t(s.paints.size());
  bool timed = false;
  int pos = 3;
  if (argc >= 5 && argv[3][0] != '-') {
    first = uint32_t(std::strtoul(argv[3], nullptr, 10));
    count = uint32_t(std::strtoul(argv[4], nullptr, 10));
    pos = 5;
  }
  for (; pos < argc; ++pos) timed |= std::strcmp(argv[pos], "--time") == 0;
  uint32_t last = std::min<uint32_t>(first + count, uint32_t(s.paints.size()));

  // Inputs are built before the timed region (scene load is not timed).
  std::vector<skity::Path> paths;
  std::vector<skity::Paint> paints;
  for (uint32_t d = first; d < last; ++d) {
    paths.push_back(BuildPath(s, d));
    paints.push_back(BuildPaint(s, d));
  }
  skity::Bitmap bitmap(s.width, s.height, skity::AlphaType::kPremul_AlphaType);
  auto t0 = std::chrono::steady_clock::now();
  auto canvas = skity::Canvas::MakeSoftwareCanvas(&bitmap);
  if (!canvas) return 3;
  if (s.has_clear) {
    canvas->Clear(skity::Color4f{s.clear[0], s.clear[1], s.clear[2], s.clear[3]});
  }
  // Layers: SaveLayer under the translation and clip bounds recorded for
  // it, the translation then undone, so the draws inside replay as outside;
  // Restore composites the layer.
  size_t li = 0;
  while (li < s.layers.size() && s.layers[li].start < first) ++li;
  const Scene::Layer* open_layer = nullptr;
  auto layer_events = [&](uint32_t d) {
    if (open_layer && open_layer->restore == d) {
      canvas->Restore();  // the layer
      canvas->Restore();  // the Save around it
      open_layer = nullptr;
    }
    while (!open_layer && li < s.layers.size() && s.layers[li].start == d) {
      const Scene::Layer& L = s.layers[li++];
      canvas->Save();
      const bool lclipped = !(L.clip[0] == -1e9f && L.clip[1] == -1e9f && L.clip[2] == 1e9f &&
                              L.clip[3] == 1e9f);
      if (lclipped) canvas->ClipRect(skity::Rect::MakeLTRB(L.clip[0], L.clip[1], L.clip[2], L.clip[3]));
      const bool lmoved = L.translate[0] != 0.f || L.translate[1] != 0.f;
      if (lmoved) canvas->Translate(L.translate[0], L.translate[1]);
      skity::Paint lp;
      lp.SetAlphaF(L.alpha);
      lp.SetBlendMode(static_cast<skity::BlendMode>(L.blend));
      canvas->SaveLayer(skity::Rect::MakeLTRB(L.bounds[0], L.bounds[1], L.bounds[2], L.bounds[3]),
                        lp);
      if (lmoved) canvas->Translate(-L.translate[0], -L.translate[1]);
      open_layer = &L;
      if (L.restore == d) {
        canvas->Restore();
        canvas->Restore();
        open_layer = nullptr;
      }
    }
  };
  for (size_t i = 0; i < paths.size(); ++i) {
    layer_events(first + uint32_t(i));
    const PaintRec& pr = s.paints[first + i];
    const float* mx = s.matrices.empty() ? nullptr : s.matrices.data() + 6 * (first + i);
    const bool concat = mx && !(mx[0] == 1.f && mx[1] == 0.f && mx[2] == 0.f && mx[3] == 0.f &&
                                mx[4] == 1.f && mx[5] == 0.f);
    const bool moved = concat || pr.translate[0] != 0.f || pr.translate[1] != 0.f;
    const float* c = s.clips.empty() ? nullptr : s.clips.data() + 4 * (first + i);
    const bool clipped =
        c && !(c[0] == -1e9f && c[1] == -1e9f && c[2] == 1e9f && c[3] == 1e9f);
    const uint32_t cstate = s.draw_clip_state.empty() ? 0 : s.draw_clip_state[first + i];
    if (moved || clipped || cstate) canvas->Save();
    ReplayClipState(s, canvas.get(), cstate);
    // the stored clip is already in device space: ClipRect before the
    // translation leaves exactly these global clip bounds
    if (clipped) canvas->ClipRect(skity::Rect::MakeLTRB(c[0], c[1], c[2], c[3]));
    if (concat) {
      // Canvas::Concat onto the identity: the CTM becomes the matrix itself
      const float nine[9] = {mx[0], mx[1], mx[2], mx[3], mx[4], mx[5], 0.f, 0.f, 1.f};
      skity::Matrix m;
      m.Set9(nine);
      canvas->Concat(m);
    } else if (moved) {
      canvas->Translate(pr.translate[0], pr.translate[1]);
    }
    canvas->DrawPath(paths[i], paints[i]);
    if (moved || clipped || cstate) canvas->Restore();
  }
  layer_events(last);
  canvas->Flush();
  auto t1 = std::chrono::steady_clock::now();
  if (timed) {
    std::printf("{\"seconds\": %.6f, \"draws\": %zu}\n",
                std::chrono::duration<double>(t1 - t0).count(), paths.size());
  }
  std::ofstream out(argv[2], std::ios::binary);
  for (uint32_t y = 0; y < s.height; ++y) {
    out.write(reinterpret_cast<const char*>(bitmap.GetPixelAddr() +
                                            size_t(y) * bitmap.RowBytes()),
              std::streamsize(size_t(s.width) * 4));
  }
  return 0;
}
