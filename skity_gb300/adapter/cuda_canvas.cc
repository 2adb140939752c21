// skity::Canvas over the GB300 raster backend's C ABI; see cuda_canvas.hpp.
#include "cuda_canvas.hpp"

#include <cstring>
#include <skity/effect/color_filter.hpp>
#include <skity/effect/mask_filter.hpp>
#include <skity/effect/shader.hpp>
#include <skity/graphic/paint.hpp>
#include <skity/graphic/path.hpp>
#include <vector>

#include "src/effect/color_filter_base.hpp"  // the filter kinds and their parameters

namespace skity {
namespace cuda {

CUDACanvas::CUDACanvas(skity_cuda_canvas canvas, Bitmap* bitmap)
    : Canvas(), canvas_(canvas), bitmap_(bitmap) {}

CUDACanvas::~CUDACanvas() { skity_cuda_canvas_destroy(canvas_); }

// The canvas matrix as a translation, or false when it is anything else.
static bool TranslationOf(const Matrix& m, float* tx, float* ty) {
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r)
      if (!(c == 3 && r < 2) && m.Get(r, c) != (r == c ? 1.f : 0.f)) return false;
  *tx = m.GetTranslateX();
  *ty = m.GetTranslateY();
  return true;
}

static void PathStorage(const Path& path, std::vector<uint8_t>* verbs, std::vector<float>* pts,
                        std::vector<float>* weights, skity_cuda_path* p);

// The canvas matrix as Matrix::Get9 gives it, or false under perspective
// (the C ABI canvas maps paths by affine matrices; the z terms meet z = 0).
static bool AffineOf(const Matrix& m, float nine[9]) {
  if (m.Get(3, 0) != 0.f || m.Get(3, 1) != 0.f || m.Get(3, 3) != 1.f) return false;
  m.Get9(nine);
  return true;
}
static bool IsIdentity9(const float n[9]) {
  return n[0] == 1.f && n[1] == 0.f && n[2] == 0.f && n[3] == 0.f && n[4] == 1.f && n[5] == 0.f;
}

// Canvas::ClipRect has already narrowed the global clip bounds
// (canvas.cc:130-135,463-476); for kIntersect under scale and translation that is
// all SWCanvas does too (sw_canvas.cc:279-295).  kDifference goes on as a
// path clip of the rect (Canvas::OnClipRect, canvas.cc:144-150).
void CUDACanvas::OnClipRect(Rect const& rect, ClipOp op) {
  if (!GetTotalMatrix().OnlyScaleAndTranslate()) {
    // SWCanvas::OnClipRect clips by the rect as a path under any other
    // matrix (sw_canvas.cc:305-309): OnClipPath takes it (or refuses it)
    Canvas::OnClipRect(rect, op);
    return;
  }
  if (op != ClipOp::kIntersect) {
    Canvas::OnClipRect(rect, op);
    return;
  }
  status_ = SKITY_CUDA_SUCCESS;
}

// SWCanvas::OnClipPath (sw_canvas.cc:317-336): the C ABI canvas records the
// clip on its state for this save level, with the canvas matrix and the
// global clip bounds in effect (the base class has already narrowed them).
void CUDACanvas::OnClipPath(Path const& path, ClipOp op) {
  float nine[9];
  if (!AffineOf(GetTotalMatrix(), nine)) {
    bad_clip_.back() = true;
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    return;
  }
  std::vector<uint8_t> verbs;
  std::vector<float> pts, weights;
  skity_cuda_path p{};
  PathStorage(path, &verbs, &pts, &weights, &p);
  const Rect& g = GetGlobalClipBounds();
  if (!(g.Left() == -1e9f && g.Top() == -1e9f && g.Right() == 1e9f && g.Bottom() == 1e9f))
    skity_cuda_canvas_clip_rect(canvas_, g.Left(), g.Top(), g.Right(), g.Bottom());
  // the matrix for this call only (a Restore would drop the clip too)
  const bool moved = !IsIdentity9(nine);
  if (moved) skity_cuda_canvas_set_matrix(canvas_, nine);
  status_ = skity_cuda_canvas_clip_path(canvas_, &p, op == ClipOp::kIntersect ? 1u : 0u);
  if (moved) {
    static const float kIdentity[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
    skity_cuda_canvas_set_matrix(canvas_, kIdentity);
  }
}

void CUDACanvas::OnDrawPath(Path const& path, Paint const& paint) {
  float nine[9];
  if (bad_clip_.back() || !AffineOf(GetTotalMatrix(), nine)) {
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    return;
  }
  std::vector<uint8_t> verbs;
  std::vector<float> pts;
  std::vector<float> weights;
  skity_cuda_path p{};
  PathStorage(path, &verbs, &pts, &weights, &p);

  skity_cuda_paint q{};
  q.style = static_cast<uint32_t>(paint.GetStyle());
  q.cap = static_cast<uint32_t>(paint.GetStrokeCap());
  q.join = static_cast<uint32_t>(paint.GetStrokeJoin());
  q.blend_mode = static_cast<uint32_t>(paint.GetBlendMode());
  const Vector fc = paint.GetFillColor(), sc = paint.GetStrokeColor();
  const float fill[4] = {fc.x, fc.y, fc.z, fc.w}, stroke[4] = {sc.x, sc.y, sc.z, sc.w};
  std::memcpy(q.fill_color, fill, sizeof fill);
  std::memcpy(q.stroke_color, stroke, sizeof stroke);
  q.stroke_width = paint.GetStrokeWidth();
  q.miter_limit = paint.GetStrokeMiter();

  skity_cuda_gradient g{};
  std::vector<float> colors;
  std::vector<float> offsets;
  if (const Shader* s = paint.GetShader().get()) {
    Shader::GradientInfo info;
    const Shader::GradientType t = s->AsGradient(&info);
    if ((t != Shader::kLinear && t != Shader::kRadial && t != Shader::kSweep &&
         t != Shader::kConical) ||
        !info.local_matrix.IsIdentity()) {
      status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
      return;
    }
    g.type = t == Shader::kLinear ? 1u : t == Shader::kRadial ? 2u : t == Shader::kSweep ? 3u : 4u;
    g.tile_mode = static_cast<uint32_t>(info.tile_mode);
    g.stop_count = static_cast<uint32_t>(info.colors.size());
    g.has_offsets = info.color_offsets.empty() ? 0u : 1u;
    g.p0[0] = info.point[0].x;
    g.p0[1] = info.point[0].y;
    g.p1[0] = info.point[1].x;
    g.p1[1] = info.point[1].y;
    g.radius[0] = info.radius[0];
    g.radius[1] = info.radius[1];
    for (const Vec4& c : info.colors) colors.insert(colors.end(), {c.x, c.y, c.z, c.w});
    offsets = info.color_offsets;
    g.colors = colors.data();
    g.offsets = offsets.empty() ? nullptr : offsets.data();
    q.shader = &g;
  }
  skity_cuda_color_filter cf{};
  if (const ColorFilter* f = paint.GetColorFilter().get()) {
    const ColorFilterBase* base = As_CFB(f);
    switch (base->GetType()) {
      case ColorFilterType::kBlend: {
        const auto* b = static_cast<const BlendColorFilter*>(base);
        cf.type = 1;
        cf.blend_mode = static_cast<uint32_t>(b->GetBlendMode());
        cf.color = b->GetColor();
        break;
      }
      case ColorFilterType::kMatrix: {
        // GetMatrix: columns of the 4 x 4 part, then the bias column
        auto mm = const_cast<MatrixColorFilter*>(static_cast<const MatrixColorFilter*>(base))
                      ->GetMatrix();
        const Matrix& mul = std::get<0>(mm);
        const Vec4& add = std::get<1>(mm);
        cf.type = 2;
        for (int r = 0; r < 4; ++r) {
          for (int c = 0; c < 4; ++c) cf.matrix[5 * r + c] = mul.Get(r, c);
        }
        cf.matrix[4] = add.x;
        cf.matrix[9] = add.y;
        cf.matrix[14] = add.z;
        cf.matrix[19] = add.w;
        break;
      }
      case ColorFilterType::kLinearToSRGBGamma:
        cf.type = 3;
        break;
      case ColorFilterType::kSRGBToLinearGamma:
        cf.type = 4;
        break;
      default:
        cf.type = 5;  // compose: the identity on the software path
        break;
    }
    q.color_filter = &cf;
  }
  if (const MaskFilter* mf = paint.GetMaskFilter().get()) {
    q.blur_style = static_cast<uint32_t>(mf->GetBlurStyle());
    q.blur_radius = mf->GetBlurRadius();
  }
  // the C-ABI canvas holds no state between draws: each draw carries its
  // device-space clip bounds (set before the matrix, so they stay as they
  // are) and the canvas matrix this canvas computed
  const Rect& clip = GetGlobalClipBounds();
  const bool clipped = !(clip.Left() == -1e9f && clip.Top() == -1e9f && clip.Right() == 1e9f &&
                         clip.Bottom() == 1e9f);
  const bool moved = !IsIdentity9(nine);
  if (moved || clipped) skity_cuda_canvas_save(canvas_);
  if (clipped)
    skity_cuda_canvas_clip_rect(canvas_, clip.Left(), clip.Top(), clip.Right(), clip.Bottom());
  if (moved) skity_cuda_canvas_set_matrix(canvas_, nine);
  if ((q.shader || q.image_shader || q.blur_style) && !GetTotalMatrix().OnlyScaleAndTranslate()) {
    // a shader's (or a blur's image draw's) inverse past scale and translation
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    if (moved || clipped) skity_cuda_canvas_restore(canvas_);
    return;
  }
  status_ = skity_cuda_canvas_draw_path(canvas_, &p, &q);
  if (moved || clipped) skity_cuda_canvas_restore(canvas_);
}

// Path storage as the reference keeps it (path.hpp:590-596), in the C ABI's
// path record (pointing into the vectors).
static void PathStorage(const Path& path, std::vector<uint8_t>* verbs, std::vector<float>* pts,
                        std::vector<float>* weights, skity_cuda_path* p) {
  verbs->reserve(path.CountVerbs());
  uint32_t conics = 0;
  for (const Path::Verb* v = path.VerbsBegin(); v != path.VerbsEnd(); ++v) {
    verbs->push_back(static_cast<uint8_t>(*v));
    if (*v == Path::Verb::kConic) conics++;
  }
  pts->reserve(2 * path.CountPoints());
  for (size_t i = 0; i < path.CountPoints(); ++i) {
    pts->push_back(path.Points()[i].x);
    pts->push_back(path.Points()[i].y);
  }
  weights->assign(path.ConicWeights(), path.ConicWeights() + conics);
  p->verbs = verbs->data();
  p->verb_count = static_cast<uint32_t>(verbs->size());
  p->points = pts->data();
  p->point_count = static_cast<uint32_t>(path.CountPoints());
  p->conic_weights = weights->data();
  p->conic_weight_count = conics;
  p->fill_type = path.GetFillType() == Path::PathFillType::kEvenOdd ? 1u : 0u;
}

// Canvas::SaveLayer has saved the level and narrowed the global clip bounds
// by the bounds (canvas.cc:255-276); the C-ABI canvas gets a level with
// those clip bounds and the translation, then the layer, then the
// translation undone (draws carry their own).  Restore pops both levels:
// the inner one composites the layer.
void CUDACanvas::OnSaveLayer(const Rect& bounds, const Paint& paint) {
  float tx = 0.f, ty = 0.f;
  bad_clip_.push_back(bad_clip_.back());
  if (!TranslationOf(GetTotalMatrix(), &tx, &ty)) {
    saves_.push_back(1);
    skity_cuda_canvas_save(canvas_);
    bad_clip_.back() = true;
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    return;
  }
  skity_cuda_canvas_save(canvas_);
  const Rect& g = GetGlobalClipBounds();
  if (!(g.Left() == -1e9f && g.Top() == -1e9f && g.Right() == 1e9f && g.Bottom() == 1e9f))
    skity_cuda_canvas_clip_rect(canvas_, g.Left(), g.Top(), g.Right(), g.Bottom());
  const bool moved = tx != 0.f || ty != 0.f;
  if (moved) skity_cuda_canvas_translate(canvas_, tx, ty);
  skity_cuda_paint q{};
  q.style = static_cast<uint32_t>(paint.GetStyle());
  q.blend_mode = static_cast<uint32_t>(paint.GetBlendMode());
  const Vector fc = paint.GetFillColor(), sc = paint.GetStrokeColor();
  const float fill[4] = {fc.x, fc.y, fc.z, fc.w}, stroke[4] = {sc.x, sc.y, sc.z, sc.w};
  std::memcpy(q.fill_color, fill, sizeof fill);
  std::memcpy(q.stroke_color, stroke, sizeof stroke);
  q.stroke_width = 1.f;
  q.miter_limit = 4.f;
  if (paint.GetMaskFilter() || paint.GetColorFilter()) {
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    bad_clip_.back() = true;
  } else {
    const float b[4] = {bounds.Left(), bounds.Top(), bounds.Right(), bounds.Bottom()};
    status_ = skity_cuda_canvas_save_layer(canvas_, b, &q);
  }
  if (status_ != SKITY_CUDA_SUCCESS) {
    if (moved) skity_cuda_canvas_translate(canvas_, -tx, -ty);
    saves_.push_back(1);
    bad_clip_.back() = true;
    return;
  }
  if (moved) skity_cuda_canvas_translate(canvas_, -tx, -ty);
  saves_.push_back(2);
}

void CUDACanvas::OnDrawBlob(const TextBlob*, float, float, Paint const&) {
  status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
}

// Canvas::DrawImageRect / DrawImage of a pixmap image (SWCanvas::
// OnDrawImageRect, sw_canvas.cc:641-677) under the canvas matrix: the pixels,
// src / dst and the paint's alpha and blend mode go to the C-ABI canvas.
void CUDACanvas::OnDrawImageRect(std::shared_ptr<Image> image, const Rect& src, const Rect& dst,
                                 const SamplingOptions& sampling, Paint const* paint) {
  float nine[9];
  if (bad_clip_.back() || !AffineOf(GetTotalMatrix(), nine) || !image) {
    status_ = image ? SKITY_CUDA_ERROR_NOT_SUPPORTED : SKITY_CUDA_SUCCESS;
    return;
  }
  const std::shared_ptr<Pixmap>* pm = image->GetPixmap();
  if (!pm || !*pm || (paint && (paint->GetShader() || paint->GetMaskFilter() ||
                                paint->GetColorFilter()))) {
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    return;
  }
  const Pixmap& px = **pm;
  skity_cuda_image im{};
  im.width = static_cast<uint32_t>(px.Width());
  im.height = static_cast<uint32_t>(px.Height());
  im.alpha_type = static_cast<uint32_t>(px.GetAlphaType());
  im.pixels = px.Addr();
  skity_cuda_paint q{};
  q.blend_mode = 3;
  q.fill_color[3] = q.stroke_color[3] = 1.f;
  q.stroke_width = 1.f;
  q.miter_limit = 4.f;
  if (paint) {
    q.style = static_cast<uint32_t>(paint->GetStyle());
    q.blend_mode = static_cast<uint32_t>(paint->GetBlendMode());
    const Vector fc = paint->GetFillColor(), sc = paint->GetStrokeColor();
    const float fill[4] = {fc.x, fc.y, fc.z, fc.w}, stroke[4] = {sc.x, sc.y, sc.z, sc.w};
    std::memcpy(q.fill_color, fill, sizeof fill);
    std::memcpy(q.stroke_color, stroke, sizeof stroke);
  }
  const float s4[4] = {src.Left(), src.Top(), src.Right(), src.Bottom()};
  const float d4[4] = {dst.Left(), dst.Top(), dst.Right(), dst.Bottom()};
  const uint32_t filter = sampling.UseCubic() ? 2u : sampling.filter == FilterMode::kLinear ? 1u : 0u;
  const Rect& clip = GetGlobalClipBounds();
  const bool clipped = !(clip.Left() == -1e9f && clip.Top() == -1e9f && clip.Right() == 1e9f &&
                         clip.Bottom() == 1e9f);
  const bool moved = !IsIdentity9(nine);
  if (moved || clipped) skity_cuda_canvas_save(canvas_);
  if (clipped)
    skity_cuda_canvas_clip_rect(canvas_, clip.Left(), clip.Top(), clip.Right(), clip.Bottom());
  if (moved) skity_cuda_canvas_set_matrix(canvas_, nine);
  if (!GetTotalMatrix().OnlyScaleAndTranslate()) {
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;  // the pixmap brush's inverse past scale and translation
    if (moved || clipped) skity_cuda_canvas_restore(canvas_);
    return;
  }
  status_ = skity_cuda_canvas_draw_image_rect(canvas_, &im, s4, d4, filter, &q);
  if (moved || clipped) skity_cuda_canvas_restore(canvas_);
}

void CUDACanvas::OnDrawGlyphs(uint32_t, const GlyphID[], const float[], const float[],
                              const Font&, const Paint&) {
  status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
}

// Canvas::Clear(color) is DrawColor(color, kSrc) -> DrawPaint (canvas.cc:241-253):
// a kSrc fill of the whole canvas with no shader is the clear entry point.
void CUDACanvas::OnDrawPaint(Paint const& paint) {
  if (paint.GetBlendMode() != BlendMode::kSrc || paint.GetShader() || paint.GetMaskFilter()) {
    status_ = SKITY_CUDA_ERROR_NOT_SUPPORTED;
    return;
  }
  const Vector c = paint.GetFillColor();
  const float rgba[4] = {c.x, c.y, c.z, c.w};
  status_ = skity_cuda_canvas_clear(canvas_, rgba);
}

void CUDACanvas::OnFlush() { status_ = skity_cuda_canvas_flush(canvas_); }

uint32_t CUDACanvas::OnGetWidth() const { return bitmap_->Width(); }

uint32_t CUDACanvas::OnGetHeight() const { return bitmap_->Height(); }

std::unique_ptr<CUDACanvas> MakeCUDACanvas(Bitmap* bitmap) {
  static skity_cuda_context ctx = [] {
    skity_cuda_context c = nullptr;
    return skity_cuda_context_create(nullptr, &c) == SKITY_CUDA_SUCCESS ? c : nullptr;
  }();
  if (!ctx) return nullptr;
  return MakeCUDACanvas(ctx, bitmap);
}

std::unique_ptr<CUDACanvas> MakeCUDACanvas(skity_cuda_context ctx, Bitmap* bitmap) {
  if (!bitmap || bitmap->Width() == 0 || bitmap->Height() == 0) return nullptr;
  skity_cuda_canvas c = nullptr;
  if (skity_cuda_canvas_create(ctx, bitmap->Width(), bitmap->Height(), bitmap->GetPixelAddr(),
                               bitmap->RowBytes(), &c) != SKITY_CUDA_SUCCESS)
    return nullptr;
  return std::make_unique<CUDACanvas>(c, bitmap);
}

}  // namespace cuda
}  // namespace skity
