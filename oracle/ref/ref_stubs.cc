// Link stubs for the reference-software-backend oracle build (oracle/_ref).
//
// The reference's canvas and image translation units reference font and text
// symbols that the software raster path never calls for path
// draws. Those live in translation units that need freetype and other absent
// dependencies, so they are replaced here by stubs that abort if reached.
// Image::MakeImage is the one symbol the path really uses (the blur mask
// filter draws its blurred temp bitmap back through DrawImage); it is
// re-implemented as a plain pixmap-backed image (own code, written against
// the public interface in include/skity/graphic/image.hpp).
//
// Test infrastructure only: nothing here is part of the shipped library.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <skity/graphic/image.hpp>
#include <skity/text/font.hpp>
#include <skity/text/font_style.hpp>
#include <skity/text/text_blob.hpp>
#include <skity/text/text_run.hpp>
#include <skity/text/typeface.hpp>
#include <skity/text/utf.hpp>


namespace {
[[noreturn]] void Unreachable(const char* what) {
  std::fprintf(stderr, "oracle: unsupported reference symbol reached: %s\n",
               what);
  std::abort();
}

class OraclePixmapImage final : public skity::Image {
 public:
  explicit OraclePixmapImage(std::shared_ptr<skity::Pixmap> pixmap)
      : pixmap_(std::move(pixmap)) {}
  bool IsTextureBackend() const override { return false; }
  const std::shared_ptr<skity::Texture>* GetTexture() const override {
    return nullptr;
  }
  const std::shared_ptr<skity::Pixmap>* GetPixmap() const override {
    return &pixmap_;
  }
  size_t Width() const override { return pixmap_ ? pixmap_->Width() : 0; }
  size_t Height() const override { return pixmap_ ? pixmap_->Height() : 0; }
  skity::AlphaType GetAlphaType() const override {
    return pixmap_ ? pixmap_->GetAlphaType() : skity::kUnknown_AlphaType;
  }
  skity::ImageType GetImageType() const override {
    return skity::ImageType::kPixmap;
  }

 private:
  std::shared_ptr<skity::Pixmap> pixmap_;
};
}  // namespace

namespace skity {

std::shared_ptr<Image> Image::MakeImage(std::shared_ptr<Pixmap> pixmap,
                                        GPUContext*) {
  if (!pixmap) return nullptr;
  return std::make_shared<OraclePixmapImage>(std::move(pixmap));
}

bool Typeface::ContainsColorTable() const { Unreachable("Typeface"); }
std::shared_ptr<Typeface> Typeface::GetDefaultTypeface(FontStyle) {
  Unreachable("Typeface::GetDefaultTypeface");
}
void Typeface::UnicharsToGlyphs(const uint32_t*, int, GlyphID*) const {
  Unreachable("Typeface::UnicharsToGlyphs");
}
FontStyle::FontStyle() { Unreachable("FontStyle"); }
std::vector<GlyphID> const& TextRun::GetGlyphInfo() const {
  Unreachable("TextRun");
}
std::vector<float> const& TextRun::GetPosX() const { Unreachable("TextRun"); }
Font::Font(std::shared_ptr<Typeface>, float) { Unreachable("Font"); }
void Font::LoadGlyphMetrics(const GlyphID*, uint32_t, const GlyphData**,
                            const Paint&) const {
  Unreachable("Font::LoadGlyphMetrics");
}
void Font::LoadGlyphPath(const GlyphID*, uint32_t, const GlyphData**) const {
  Unreachable("Font::LoadGlyphPath");
}
void Font::LoadGlyphBitmap(const GlyphID*, uint32_t, const GlyphData**,
                           const Paint&, float, const Matrix&) const {
  Unreachable("Font::LoadGlyphBitmap");
}
Rect TextBlob::ComputeBounds(uint32_t, const GlyphID*, const float*,
                             const float*, const Font&, const Paint&) {
  Unreachable("TextBlob::ComputeBounds");
}
std::shared_ptr<TextBlob> TextBlobBuilder::BuildTextBlob(const char*,
                                                         Paint const&,
                                                         TypefaceDelegate*) {
  Unreachable("TextBlobBuilder::BuildTextBlob");
}
bool UTF::UTF8ToCodePoint(const char*, size_t, std::vector<Unichar>&) {
  Unreachable("UTF::UTF8ToCodePoint");
}

}  // namespace skity
