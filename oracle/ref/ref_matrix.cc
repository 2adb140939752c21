// Test infrastructure: the canvas matrix the reference's Canvas computes for
// a sequence of transform calls (Canvas::Translate / Scale / Rotate / Skew /
// Concat / SetMatrix on a software canvas), printed as Matrix::Get9 gives it
// (nine %a floats).  Usage: ref_matrix op args... ; ops:
//   t dx dy | s sx sy | r deg px py | k kx ky | c m0..m8 | m m0..m8 |
//   S (Save) | R (Restore) | L l t r b (SaveLayer with a default paint)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <skity/graphic/bitmap.hpp>
#include <skity/graphic/paint.hpp>
#include <skity/render/canvas.hpp>

int main(int argc, char** argv) {
  skity::Bitmap bitmap(4, 4, skity::AlphaType::kPremul_AlphaType);
  auto canvas = skity::Canvas::MakeSoftwareCanvas(&bitmap);
  int i = 1;
  auto f = [&]() { return i < argc ? std::strtof(argv[i++], nullptr) : 0.f; };
  while (i < argc) {
    const char op = argv[i++][0];
    if (op == 't') {
      const float x = f(), y = f();
      canvas->Translate(x, y);
    } else if (op == 's') {
      const float x = f(), y = f();
      canvas->Scale(x, y);
    } else if (op == 'r') {
      const float d = f(), px = f(), py = f();
      canvas->Rotate(d, px, py);
    } else if (op == 'k') {
      const float x = f(), y = f();
      canvas->Skew(x, y);
    } else if (op == 'c' || op == 'm') {
      float b[9];
      for (float& v : b) v = f();
      skity::Matrix m;
      m.Set9(b);
      if (op == 'c') canvas->Concat(m);
      else canvas->SetMatrix(m);
    } else if (op == 'S') {
      canvas->Save();
    } else if (op == 'R') {
      canvas->Restore();
    } else if (op == 'L') {
      const float l = f(), t = f(), r = f(), b = f();
      canvas->SaveLayer(skity::Rect::MakeLTRB(l, t, r, b), skity::Paint());
    } else {
      return 2;
    }
  }
  float out[9];
  canvas->GetTotalMatrix().Get9(out);
  for (float v : out) std::printf("%a\n", v);
  return 0;
}
