// Test infrastructure: the path the reference's Canvas::DrawOval /
// DrawCircle hand to DrawPath (Canvas::OnDrawCircle -> OnDrawOval ->
// RRect::SetOval -> OnDrawRRect -> Path::AddRRect, canvas.cc:407-430),
// printed as verbs, then points (x y, %a), then conic weights (%a).
// Usage: ref_shapes o l t r b | ref_shapes c cx cy radius
#include <cstdio>
#include <cstdlib>
#include <skity/geometry/rrect.hpp>
#include <skity/graphic/path.hpp>

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  auto f = [&](int i) { return i < argc ? std::strtof(argv[i], nullptr) : 0.f; };
  skity::Rect r;
  if (argv[1][0] == 'o') {
    r = skity::Rect::MakeLTRB(f(2), f(3), f(4), f(5));
  } else {
    float cx = f(2), cy = f(3), radius = f(4);
    if (radius < 0) radius = 0;  // Canvas::OnDrawCircle
    r.SetLTRB(cx - radius, cy - radius, cx + radius, cy + radius);
  }
  skity::RRect rr;
  rr.SetOval(r);
  skity::Path path;
  path.AddRRect(rr);
  std::printf("verbs");
  for (const skity::Path::Verb* v = path.VerbsBegin(); v != path.VerbsEnd(); ++v)
    std::printf(" %d", static_cast<int>(*v));
  std::printf("\npoints");
  for (size_t i = 0; i < path.CountPoints(); ++i) {
    const skity::Point p = path.GetPoint(static_cast<int>(i));
    std::printf(" %a %a", p.x, p.y);
  }
  std::printf("\nweights");
  size_t conics = 0;
  for (const skity::Path::Verb* v = path.VerbsBegin(); v != path.VerbsEnd(); ++v)
    if (*v == skity::Path::Verb::kConic) conics++;
  for (size_t i = 0; i < conics; ++i) std::printf(" %a", path.ConicWeights()[i]);
  std::printf("\n");
  return 0;
}
