// Test infrastructure: plays an SKP file back through the reference's own IO
// module (module/io: Picture::MakeFromStream, Picture::PlayBack) onto the
// reference's software canvas and writes the premultiplied RGBA8 pixels.
//   ref_skp in.skp out.rgba  ->  prints "w h" of the canvas (the cull rect
//   rounded out), cleared to opaque white before the playback.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <skity/graphic/bitmap.hpp>
#include "src/io/memory_writer.hpp"  // complete type of Picture's writer member
#include <skity/io/picture.hpp>
#include <skity/io/stream.hpp>
#include <skity/render/canvas.hpp>
#include <vector>

namespace {
// A ReadStream over a byte vector.
class BytesStream : public skity::ReadStream {
 public:
  explicit BytesStream(std::vector<uint8_t> b) : b_(std::move(b)) {}
  size_t Read(void* buffer, size_t size) override {
    const size_t n = std::min(size, b_.size() - at_);
    if (buffer) std::memcpy(buffer, b_.data() + at_, n);
    at_ += n;
    return n;
  }
  size_t Peek(void* buffer, size_t size) override {
    const size_t n = std::min(size, b_.size() - at_);
    std::memcpy(buffer, b_.data() + at_, n);
    return n;
  }
  bool IsAtEnd() const override { return at_ >= b_.size(); }

 private:
  std::vector<uint8_t> b_;
  size_t at_ = 0;
};
}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  std::ifstream f(argv[1], std::ios::binary);
  std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  BytesStream s(std::move(bytes));
  auto pic = skity::Picture::MakeFromStream(s);
  if (!pic) {
    std::fprintf(stderr, "not a picture\n");
    return 3;
  }
  const skity::Rect cull = pic->GetCullRect();
  const int w = (int)std::ceil(cull.Right()), h = (int)std::ceil(cull.Bottom());
  if (w <= 0 || h <= 0) return 4;
  skity::Bitmap bitmap(w, h, skity::AlphaType::kPremul_AlphaType);
  auto canvas = skity::Canvas::MakeSoftwareCanvas(&bitmap);
  canvas->Clear(skity::Color4f{1.f, 1.f, 1.f, 1.f});
  pic->PlayBack(canvas.get());
  canvas->Flush();
  std::ofstream out(argv[2], std::ios::binary);
  for (int y = 0; y < h; ++y)
    out.write(reinterpret_cast<const char*>(bitmap.GetPixelAddr() + size_t(y) * bitmap.RowBytes()),
              std::streamsize(size_t(w) * 4));
  std::printf("%d %d\n", w, h);
  return 0;
}
