// skity::Canvas over the GB300 raster backend's C ABI (include/skity_cuda.h).
//
// The drop-in for Canvas::MakeSoftwareCanvas(Bitmap*)
// (include/skity/render/canvas.hpp:359, src/render/sw/sw_canvas.cc:146-156):
// MakeCUDACanvas(ctx, bitmap) returns a Canvas whose DrawPath / Clear /
// DrawPaint(kSrc) / Flush run on the GPU.  It compiles inside a Skity tree
// (it needs Skity's public headers) and links against libskity_cuda.so.
//
// What differs from the software canvas: pixels are written to the bitmap at
// Flush(), not during each draw.  ClipRect(kIntersect) under a translation is
// taken (the global clip bounds the base class keeps bound each draw's scan,
// as SWCanvas::OnClipRect relies on, sw_canvas.cc:279-295), and so are
// ClipPath, ClipRRect and ClipRect(kDifference) under a translation (path
// clips the C ABI canvas keeps per save level, as SWCanvas does), SaveLayer
// (one level, a layer paint's alpha and blend mode) and DrawImageRect /
// DrawImage under a translation.  Operations outside the GPU raster path --
// clips under other matrices, nested layers, text, canvas matrices other
// than translations, shader local matrices --
// draw nothing and leave
// SKITY_CUDA_ERROR_NOT_SUPPORTED in LastStatus(); draws under a clip this
// canvas did not take draw nothing either, until the Restore that drops it.
#ifndef SKITY_GB300_ADAPTER_CUDA_CANVAS_HPP
#define SKITY_GB300_ADAPTER_CUDA_CANVAS_HPP

#include <memory>
#include <skity/graphic/bitmap.hpp>
#include <vector>
#include <skity/render/canvas.hpp>

#include "../../include/skity_cuda.h"

namespace skity {
namespace cuda {

class CUDACanvas : public Canvas {
 public:
  CUDACanvas(skity_cuda_canvas canvas, Bitmap* bitmap);
  ~CUDACanvas() override;

  // Result of the last operation (SKITY_CUDA_SUCCESS or an error code).
  int32_t LastStatus() const { return status_; }

 protected:
  void OnClipRect(Rect const& rect, ClipOp op) override;
  void OnClipPath(Path const& path, ClipOp op) override;
  void OnDrawPath(Path const& path, Paint const& paint) override;
  void OnSaveLayer(const Rect& bounds, const Paint& paint) override;
  void OnDrawBlob(const TextBlob* blob, float x, float y, Paint const& paint) override;
  void OnDrawImageRect(std::shared_ptr<Image> image, const Rect& src, const Rect& dst,
                       const SamplingOptions& sampling, Paint const* paint) override;
  void OnDrawGlyphs(uint32_t count, const GlyphID glyphs[], const float position_x[],
                    const float position_y[], const Font& font, const Paint& paint) override;
  void OnDrawPaint(Paint const& paint) override;
  void OnSave() override {
    bad_clip_.push_back(bad_clip_.back());
    saves_.push_back(1);
    skity_cuda_canvas_save(canvas_);
  }
  void OnRestore() override {
    if (bad_clip_.size() > 1) bad_clip_.pop_back();
    // a SaveLayer level holds two C-ABI levels (the clip and the layer)
    int n = 1;
    if (!saves_.empty()) {
      n = saves_.back();
      saves_.pop_back();
    }
    for (int i = 0; i < n; ++i) skity_cuda_canvas_restore(canvas_);
  }
  void OnRestoreToCount(int) override {}
  void OnFlush() override;
  uint32_t OnGetWidth() const override;
  uint32_t OnGetHeight() const override;

 private:
  skity_cuda_canvas canvas_;
  Bitmap* bitmap_;
  int32_t status_ = SKITY_CUDA_SUCCESS;
  // per save level: a clip this canvas does not take is in effect
  std::vector<bool> bad_clip_{false};
  // per save level: the C-ABI canvas levels it pushed (1, or 2 for a SaveLayer)
  std::vector<int> saves_;
};

// Same null / empty semantics as MakeSoftwareCanvas: nullptr for a null
// bitmap or a zero width or height.  The bitmap must be kPremul_AlphaType,
// kRGBA, and outlive the canvas.
std::unique_ptr<CUDACanvas> MakeCUDACanvas(skity_cuda_context ctx, Bitmap* bitmap);
// The same over a process-wide context on CUDA device 0, created at the
// first call: the drop-in for Canvas::MakeSoftwareCanvas(Bitmap*).
std::unique_ptr<CUDACanvas> MakeCUDACanvas(Bitmap* bitmap);

}  // namespace cuda
}  // namespace skity

#endif  // SKITY_GB300_ADAPTER_CUDA_CANVAS_HPP
