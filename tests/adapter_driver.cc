// Drives skity::cuda::CUDACanvas (skity_gb300/adapter) through Skity's own
// Canvas / Path / Paint / Shader / MaskFilter API, with the C ABI replaced
// by a recorder, and prints what reached the C ABI.  Built and run by
// tests/test_adapter.py against the reference's headers and the reference
// software library built by oracle/ref (CPU only).
#include <cstdio>
#include <skity/effect/color_filter.hpp>
#include <skity/effect/mask_filter.hpp>
#include <skity/effect/shader.hpp>
#include <skity/graphic/bitmap.hpp>
#include <skity/graphic/color.hpp>
#include <skity/graphic/paint.hpp>
#include <skity/graphic/image.hpp>
#include <skity/graphic/path.hpp>
#include <skity/io/pixmap.hpp>

#include "../skity_gb300/adapter/cuda_canvas.hpp"

extern "C" {
int32_t skity_cuda_canvas_create(skity_cuda_context ctx, uint32_t w, uint32_t h, void* pixels,
                                 size_t row_bytes, skity_cuda_canvas* out) {
  std::printf("create ctx=%p w=%u h=%u pixels=%d row_bytes=%zu\n", (void*)ctx, w, h,
              pixels != nullptr, row_bytes);
  *out = reinterpret_cast<skity_cuda_canvas>(0x10);
  return SKITY_CUDA_SUCCESS;
}
void skity_cuda_canvas_destroy(skity_cuda_canvas c) { std::printf("destroy %p\n", (void*)c); }
int32_t skity_cuda_canvas_clear(skity_cuda_canvas, const float c[4]) {
  std::printf("clear %g %g %g %g\n", c[0], c[1], c[2], c[3]);
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_draw_path(skity_cuda_canvas, const skity_cuda_path* p,
                                    const skity_cuda_paint* q) {
  std::printf("draw verbs=");
  for (uint32_t i = 0; i < p->verb_count; ++i) std::printf("%u,", p->verbs[i]);
  std::printf(" points=");
  for (uint32_t i = 0; i < 2 * p->point_count; ++i) std::printf("%g,", p->points[i]);
  std::printf(" weights=");
  for (uint32_t i = 0; i < p->conic_weight_count; ++i) std::printf("%g,", p->conic_weights[i]);
  std::printf(" fill_type=%u style=%u cap=%u join=%u blend=%u width=%g miter=%g", p->fill_type,
              q->style, q->cap, q->join, q->blend_mode, q->stroke_width, q->miter_limit);
  std::printf(" fill=%g,%g,%g,%g stroke=%g,%g,%g,%g", q->fill_color[0], q->fill_color[1],
              q->fill_color[2], q->fill_color[3], q->stroke_color[0], q->stroke_color[1],
              q->stroke_color[2], q->stroke_color[3]);
  if (q->shader) {
    const skity_cuda_gradient* g = q->shader;
    std::printf(" shader=%u tile=%u stops=%u offsets=%u p0=%g,%g p1=%g,%g r=%g colors=", g->type,
                g->tile_mode, g->stop_count, g->has_offsets, g->p0[0], g->p0[1], g->p1[0],
                g->p1[1], g->radius[0]);
    for (uint32_t i = 0; i < 4 * g->stop_count; ++i) std::printf("%g,", g->colors[i]);
    if (g->has_offsets) {
      std::printf(" pos=");
      for (uint32_t i = 0; i < g->stop_count; ++i) std::printf("%g,", g->offsets[i]);
    }
  }
  if (q->color_filter) {
    const skity_cuda_color_filter* f = q->color_filter;
    std::printf(" filter=%u mode=%u color=%08x m=", f->type, f->blend_mode, f->color);
    for (float v : f->matrix) std::printf("%g,", v);
  }
  std::printf(" blur=%u,%g\n", q->blur_style, q->blur_radius);
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_save(skity_cuda_canvas) {
  std::printf("save\n");
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_restore(skity_cuda_canvas) {
  std::printf("restore\n");
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_translate(skity_cuda_canvas, float dx, float dy) {
  std::printf("translate %g %g\n", dx, dy);
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_set_matrix(skity_cuda_canvas, const float m[9]) {
  std::printf("set_matrix");
  for (int i = 0; i < 9; ++i) std::printf(" %a", m[i]);
  std::printf("\n");
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_clip_path(skity_cuda_canvas, const skity_cuda_path* p, uint32_t op) {
  std::printf("clip_path op=%u fill=%u verbs=", op, p->fill_type);
  for (uint32_t i = 0; i < p->verb_count; ++i) std::printf("%u,", p->verbs[i]);
  std::printf(" points=");
  for (uint32_t i = 0; i < 2 * p->point_count; ++i) std::printf("%g,", p->points[i]);
  std::printf("\n");
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_clip_rect(skity_cuda_canvas, float l, float t, float r, float b) {
  std::printf("clip %g %g %g %g\n", l, t, r, b);
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_flush(skity_cuda_canvas) {
  std::printf("flush\n");
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_save_layer(skity_cuda_canvas, const float b[4],
                                     const skity_cuda_paint* q) {
  std::printf("save_layer %g %g %g %g alpha=%g blend=%u\n", b[0], b[1], b[2], b[3],
              q ? q->fill_color[3] : 1.f, q ? q->blend_mode : 3u);
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_canvas_draw_image_rect(skity_cuda_canvas, const skity_cuda_image* im,
                                          const float s[4], const float d[4], uint32_t filter,
                                          const skity_cuda_paint* q) {
  std::printf("image %ux%u alpha_type=%u src=%g,%g,%g,%g dst=%g,%g,%g,%g filter=%u alpha=%g "
              "blend=%u\n",
              im->width, im->height, im->alpha_type, s[0], s[1], s[2], s[3], d[0], d[1], d[2],
              d[3], filter, q ? q->fill_color[3] : 1.f, q ? q->blend_mode : 3u);
  return SKITY_CUDA_SUCCESS;
}
int32_t skity_cuda_context_create(const skity_cuda_context_create_info*, skity_cuda_context* out) {
  *out = reinterpret_cast<skity_cuda_context>(0x30);
  return SKITY_CUDA_SUCCESS;
}
}

int main() {
  using namespace skity;
  auto ctx = reinterpret_cast<skity_cuda_context>(0x20);
  std::printf("null=%d\n", cuda::MakeCUDACanvas(ctx, nullptr) == nullptr);
  Bitmap empty;
  std::printf("empty=%d\n", cuda::MakeCUDACanvas(ctx, &empty) == nullptr);
  Bitmap bm(40, 30, AlphaType::kPremul_AlphaType);
  auto canvas = cuda::MakeCUDACanvas(ctx, &bm);
  canvas->Clear(Color4fFromColor(ColorSetARGB(255, 255, 128, 0)));
  Path path;
  path.MoveTo(1, 2);
  path.LineTo(3, 4);
  path.QuadTo(5, 6, 7, 8);
  path.ConicTo(9, 10, 11, 12, 0.5f);
  path.CubicTo(13, 14, 15, 16, 17, 18);
  path.Close();
  path.SetFillType(Path::PathFillType::kEvenOdd);
  Paint paint;
  paint.SetStyle(Paint::kStrokeAndFill_Style);
  paint.SetStrokeWidth(3.f);
  paint.SetStrokeCap(Paint::kRound_Cap);
  paint.SetStrokeJoin(Paint::kBevel_Join);
  paint.SetStrokeMiter(5.f);
  paint.SetColor(ColorSetARGB(255, 0, 255, 0));
  paint.SetAlphaF(0.5f);
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  Vec4 colors[3] = {{1, 0, 0, 1}, {0, 1, 0, 0.5f}, {0, 0, 1, 1}};
  float pos[3] = {0.f, 0.25f, 1.f};
  Point pts[2] = {{0, 0, 0, 1}, {40, 30, 0, 1}};
  paint.SetShader(Shader::MakeLinear(pts, colors, pos, 3, TileMode::kMirror));
  paint.SetMaskFilter(MaskFilter::MakeBlur(BlurStyle::kNormal, 4.5f));
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  paint.SetShader(Shader::MakeRadial(Point{20, 15, 0, 1}, 12.f, colors, nullptr, 3, TileMode::kClamp));
  paint.SetMaskFilter(nullptr);
  canvas->DrawPath(path, paint);
  canvas->Save();
  canvas->Translate(5, 0);
  canvas->Translate(0.5f, -2);
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  // a perspective matrix is outside the GPU path
  Matrix persp;
  const float p9[9] = {1, 0, 0, 0, 1, 0, 0.001f, 0, 1};
  persp.Set9(p9);
  canvas->Concat(persp);
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->Restore();
  // ClipRect(kIntersect) under a translation: device-space bounds per draw
  canvas->Save();
  canvas->Translate(2, 1);
  canvas->ClipRect(Rect::MakeLTRB(1.5f, 0, 30, 20));
  canvas->ClipRect(Rect::MakeLTRB(-5, 2, 25, 40));
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->Save();
  canvas->ClipRect(Rect::MakeLTRB(0, 0, 10, 10), Canvas::ClipOp::kDifference);
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->Restore();
  canvas->Restore();
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  // sweep and two-point conical shaders reach the C ABI as GradientInfo
  paint.SetShader(Shader::MakeSweep(20, 15, 90, 270, colors, pos, 3, TileMode::kRepeat));
  canvas->DrawPath(path, paint);
  paint.SetShader(Shader::MakeTwoPointConical(Point{5, 6, 0, 1}, 2.f, Point{30, 20, 0, 1}, 12.f,
                                              colors, nullptr, 3, TileMode::kClamp));
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  // colour filters reach the C ABI with their parameters
  paint.SetShader(nullptr);
  paint.SetColorFilter(ColorFilters::Blend(0x80102030u, BlendMode::kScreen));
  canvas->DrawPath(path, paint);
  const float rm[20] = {0, 1, 0, 0, 0.25f, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0.5f, 0};
  paint.SetColorFilter(ColorFilters::Matrix(rm));
  canvas->DrawPath(path, paint);
  paint.SetColorFilter(ColorFilters::SRGBToLinearGamma());
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->Flush();
  std::printf("status=%d\n", canvas->LastStatus());
  // SaveLayer under a translation and a clip: the C-ABI canvas gets a level
  // with the narrowed clip bounds and the translation, the layer, then the
  // translation undone; Restore pops both levels
  paint.SetColorFilter(nullptr);
  canvas->Save();
  canvas->Translate(3, 2);
  Paint lp;
  lp.SetAlphaF(0.25f);
  lp.SetBlendMode(BlendMode::kMultiply);
  canvas->SaveLayer(Rect::MakeLTRB(1, 1, 21, 11), lp);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->DrawPath(path, paint);
  canvas->Restore();
  canvas->Restore();
  // DrawImageRect / DrawImage of a pixmap image reach the C ABI
  auto pixmap = std::make_shared<Pixmap>(4, 3, AlphaType::kPremul_AlphaType);
  auto image = Image::MakeImage(pixmap);
  Paint ip;
  ip.SetAlphaF(0.5f);
  canvas->DrawImageRect(image, Rect::MakeLTRB(0, 0, 4, 3), Rect::MakeLTRB(5, 6, 13, 12),
                        SamplingOptions{FilterMode::kLinear, MipmapMode::kNone}, &ip);
  std::printf("status=%d\n", canvas->LastStatus());
  std::printf("default_ctx=%d\n", cuda::MakeCUDACanvas(&bm) != nullptr);
  // Scale / Rotate / Skew: the canvas matrix this canvas computed reaches
  // the C ABI as Get9 gives it (printed beside it by the reference's
  // GetTotalMatrix); a gradient under a rotation is refused, and a ClipRect
  // under a rotation becomes a path clip of the rect under that matrix
  Paint solid;
  solid.SetColor(ColorSetARGB(255, 10, 20, 30));
  paint.SetShader(Shader::MakeRadial(Point{20, 15, 0, 1}, 12.f, colors, nullptr, 3, TileMode::kClamp));
  canvas->Save();
  canvas->Translate(3, 2);
  canvas->Scale(2, 0.5f);
  canvas->DrawPath(path, paint);  // the radial shader under scale and translation
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->Rotate(30, 4, 5);
  canvas->Skew(0.25f, 0);
  float m9[9];
  canvas->GetTotalMatrix().Get9(m9);
  std::printf("total");
  for (float v : m9) std::printf(" %a", v);
  std::printf("\n");
  canvas->DrawPath(path, solid);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->DrawPath(path, paint);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->ClipRect(Rect::MakeLTRB(0, 0, 10, 10));
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->DrawPath(path, solid);
  std::printf("status=%d\n", canvas->LastStatus());
  canvas->Restore();
  canvas.reset();
  return 0;
}
