// Test-only: the module/capi binding INTEGRATION.md shows, compiled against
// the reference's C API headers and wrapper structs (module/capi/src/
// handle.hpp): a skity_canvas handle over the CUDA canvas adapter, made the
// way skity_surface_lock_canvas wraps a surface's canvas
// (module/capi/src/surface_c.cpp:81-95).
#include <skity/graphic/bitmap.hpp>
#include <skity_c/skity_bitmap.h>
#include <skity_c/skity_canvas.h>

#include "handle.hpp"
#include "skity_gb300/adapter/cuda_canvas.hpp"

namespace {
skity::Bitmap* bitmap_of(skity_bitmap handle) {
  auto* w = skity::capi::resolve<skity_bitmap_s>(handle, SKITY_OBJECT_TYPE_BITMAP);
  return w ? static_cast<skity::Bitmap*>(w->impl.get()) : nullptr;
}
}  // namespace

skity_canvas skity_canvas_make_cuda(skity_bitmap bitmap) {
  skity::Bitmap* bm = bitmap_of(bitmap);
  std::unique_ptr<skity::Canvas> c = skity::cuda::MakeCUDACanvas(bm);  // null: no canvas
  if (!c) return nullptr;
  std::shared_ptr<void> impl(c.release(), [](void* p) { delete static_cast<skity::Canvas*>(p); });
  return skity::capi::alloc_handle<skity_canvas_s>(SKITY_OBJECT_TYPE_CANVAS, 0, std::move(impl));
}
