// Link stubs for ref_skp (the reference IO module's SKP playback, oracle/_ref):
// the text, font, image-codec and display-list symbols the module's readers
// reference but a picture of path draws never reaches.  Each aborts if
// reached.  Test infrastructure only.
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <skity/codec/codec.hpp>
#include <skity/recorder/display_list.hpp>
#include <skity/text/font.hpp>
#include <skity/text/font_manager.hpp>
#include <skity/text/font_style.hpp>
#include <skity/text/text_blob.hpp>
#include <skity/text/text_run.hpp>
#include <skity/text/typeface.hpp>

namespace {
[[noreturn]] void Unreachable(const char* what) {
  std::fprintf(stderr, "ref_skp: unsupported reference symbol reached: %s\n", what);
  std::abort();
}
}  // namespace

namespace skity {

std::shared_ptr<Codec> Codec::MakeFromData(const std::shared_ptr<Data>&) {
  Unreachable("Codec::MakeFromData");
}
std::shared_ptr<Codec> Codec::MakePngCodec() { Unreachable("Codec::MakePngCodec"); }
void DisplayList::Draw(Canvas*) const { Unreachable("DisplayList::Draw"); }
Font::Font() { Unreachable("Font"); }
void Font::SetSize(float) { Unreachable("Font::SetSize"); }
std::shared_ptr<Typeface> FontManager::GetDefaultTypeface(FontStyle) const {
  Unreachable("FontManager::GetDefaultTypeface");
}
std::shared_ptr<Typeface> FontManager::MakeFromData(const std::shared_ptr<Data>&, int) {
  Unreachable("FontManager::MakeFromData");
}
std::shared_ptr<FontManager> FontManager::RefDefault() { Unreachable("FontManager::RefDefault"); }
FontStyle::FontStyle(int, int, FontStyle::Slant) { Unreachable("FontStyle"); }
FontStyle::Width FontStyle::WidthFromAxisWidth(float) { Unreachable("FontStyle::WidthFromAxisWidth"); }
Rect TextBlob::GetBoundsRect() const { Unreachable("TextBlob::GetBoundsRect"); }
std::vector<float> const& TextRun::GetPosY() const { Unreachable("TextRun::GetPosY"); }
TextRun::TextRun(const Font&, std::vector<GlyphID>, std::vector<float>, std::vector<float>) {
  Unreachable("TextRun");
}
TextRun::~TextRun() {}
FontDescriptor Typeface::GetFontDescriptor() const { Unreachable("Typeface::GetFontDescriptor"); }

}  // namespace skity
