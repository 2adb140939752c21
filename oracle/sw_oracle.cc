// CPU restatement of the reference software raster path -- THE ORACLE.
//
// Test infrastructure only: tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline leg load it, as the checker and the timed CPU baseline. The
// shipped CUDA library never links or calls it.
//
// It restates, in scalar C++ written for this project, the path
//   Canvas::MakeSoftwareCanvas(Bitmap*) -> Clear -> DrawPath -> Flush
// of the reference software backend (src/render/sw/*, src/geometry/*,
// src/graphic/*, src/effect/*), one function per reference function, each
// citing the reference file:line it follows. Integer work (fixed-point edges,
// coverage, spans, blending) is bit-exact by construction; float work follows
// the reference's operation order and must be compiled with
// -ffp-contract=off (no FMA contraction) on every host.
//
// Pinning: tests/test_oracle_pin.py compares this oracle pixel-for-pixel with
// the reference's own sources compiled by oracle/ref/Makefile (oracle/_ref)
// on seeded scenes, and tests/test_oracle_golden.py against the committed
// golden fixtures generated from that build.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "sw_oracle.h"

namespace sko {

// ---------------------------------------------------------------------------
// Fixed point (src/render/sw/sw_subpixel.hpp:18-97)
// ---------------------------------------------------------------------------
typedef int32_t Fixed;
typedef int32_t FDot6;
constexpr Fixed kFixed1 = 1 << 16;
constexpr Fixed kFixedHalf = 1 << 15;
constexpr int32_t kMaxS32 = INT32_MAX;
constexpr int32_t kMinS32 = -INT32_MAX;
constexpr int32_t kNaN32 = INT32_MIN;
constexpr int kAccuracy = 2;  // SWEdge::kDefaultAccuracy (sw_edge.hpp:33)

static inline int32_t wrap_add(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a + (uint32_t)b);
}
static inline int32_t wrap_sub(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a - (uint32_t)b);
}
static inline int32_t wrap_mul(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a * (uint32_t)b);
}
static inline Fixed FixedMul(Fixed a, Fixed b) {  // sw_subpixel.hpp:40
  return (Fixed)(((int64_t)a * b) >> 16);
}
static inline Fixed FDot6ToFixed(FDot6 x) { return (Fixed)((uint32_t)x << 10); }
static inline int32_t LeftShift(int32_t v, int s) {
  return (int32_t)((uint32_t)v << s);
}
static inline Fixed FDot6ToFixedDiv2(FDot6 v) { return LeftShift(v, 16 - 6 - 1); }
static inline Fixed FixedDiv(int32_t numer, int32_t denom) {  // :67-70
  int64_t q = (int64_t)((uint64_t)(int64_t)numer << 16) / denom;
  if (q < kMinS32) q = kMinS32;
  if (q > kMaxS32) q = kMaxS32;
  return (Fixed)q;
}
static inline Fixed FDot6Div(FDot6 a, FDot6 b) { return FixedDiv(a, b); }
static inline int FDot6Round(FDot6 x) { return (x + 32) >> 6; }
// (SWFDot6)((x) * 64): C conversion truncates toward zero.
static inline FDot6 ScalarToFDot6(float x) { return (FDot6)(x * 64); }
static inline FDot6 FixedToFDot6(Fixed x) { return x >> 10; }
static inline Fixed FixedRoundToFixed(Fixed x) {
  return (Fixed)((uint32_t)(x + kFixedHalf) & 0xFFFF0000u);
}
static inline Fixed FixedCeilToFixed(Fixed x) {
  return (Fixed)((uint32_t)(x + kFixed1 - 1) & 0xFFFF0000u);
}
static inline Fixed FixedFloorToFixed(Fixed x) {
  return (Fixed)((uint32_t)x & 0xFFFF0000u);
}
static inline Fixed IntToFixed(int n) { return (Fixed)((uint32_t)n << 16); }
static inline int FixedRoundToInt(Fixed x) { return (x + kFixedHalf) >> 16; }
static inline int FixedCeilToInt(Fixed x) { return (x + kFixed1 - 1) >> 16; }
static inline int FixedFloorToInt(Fixed x) { return x >> 16; }
static inline int CLZ(uint32_t x) { return x ? __builtin_clz(x) : 32; }

struct P {
  float x, y;
};
static inline bool PEq(P a, P b) { return a.x == b.x && a.y == b.y; }

// ---------------------------------------------------------------------------
// Path storage and builders (src/graphic/path.cc:494-569,837-860,1327-1339)
// ---------------------------------------------------------------------------
enum Verb : uint8_t { kMove = 0, kLine, kQuad, kConic, kCubic, kClose };

struct Path {
  std::vector<uint8_t> verbs;
  std::vector<P> pts;
  std::vector<float> w;
  int32_t last_move = ~0;

  void MoveTo(P p) {
    if (!verbs.empty() && verbs.back() == kMove) {
      pts.back() = p;
    } else {
      last_move = (int32_t)pts.size();
      verbs.push_back(kMove);
      pts.push_back(p);
    }
  }
  void Inject() {  // InjectMoveToIfNeed (path.cc:1327-1339)
    if (last_move < 0) {
      P p = verbs.empty() ? P{0, 0} : pts[~last_move];
      MoveTo(p);
    }
  }
  void LineTo(P p) {
    Inject();
    verbs.push_back(kLine);
    pts.push_back(p);
  }
  void QuadTo(P a, P b) {
    Inject();
    verbs.push_back(kQuad);
    pts.push_back(a);
    pts.push_back(b);
  }
  void ConicTo(P a, P b, float weight) {  // path.cc:533-555
    if (!(weight > 0)) {
      LineTo(b);
    } else if (std::isinf(weight)) {
      LineTo(a);
      LineTo(b);
    } else if (weight == 1.0f) {
      QuadTo(a, b);
    } else {
      Inject();
      verbs.push_back(kConic);
      w.push_back(weight);
      pts.push_back(a);
      pts.push_back(b);
    }
  }
  void CubicTo(P a, P b, P c) {
    Inject();
    verbs.push_back(kCubic);
    pts.push_back(a);
    pts.push_back(b);
    pts.push_back(c);
  }
  void Close() {  // path.cc:837-860
    if (!verbs.empty()) {
      if (verbs.back() != kClose) verbs.push_back(kClose);
    }
    last_move ^= (~last_move >> 31);
  }
  bool GetLastPt(P* p) const {
    if (pts.empty()) return false;
    *p = pts.back();
    return true;
  }
  void Reset() {
    verbs.clear();
    pts.clear();
    w.clear();
    last_move = ~0;
  }
};

// Path::Iter with forceClose = false (path.cc:234-397)
struct PathIter {
  const Path* path;
  size_t v = 0, p = 0, wi = 0;
  P move_to{0, 0}, last_pt{0, 0};
  int seg_state = 0;  // 0 empty contour, 1 after move, 2 after primitive
  float weight = 0;
  explicit PathIter(const Path& src) : path(&src) {}

  P ConsMoveTo() {
    if (seg_state == 1) {
      seg_state = 2;
      return move_to;
    }
    return path->pts[p - 1];
  }
  // AutoClose (path.cc:372-388)
  uint8_t AutoClose(P* out) {
    if (!PEq(last_pt, move_to)) {
      if (std::isnan(last_pt.x) || std::isnan(last_pt.y) ||
          std::isnan(move_to.x) || std::isnan(move_to.y)) {
        return kClose;
      }
      out[0] = last_pt;
      out[1] = move_to;
      last_pt = move_to;
      return kLine;
    }
    out[0] = move_to;
    return kClose;
  }
  // returns verb, or 6 for kDone
  uint8_t Next(P out[4]) {
    const auto& verbs = path->verbs;
    if (v == verbs.size()) return 6;
    uint8_t verb = verbs[v++];
    switch (verb) {
      case kMove:
        if (v == verbs.size()) return 6;
        move_to = path->pts[p];
        out[0] = move_to;
        p += 1;
        seg_state = 1;
        last_pt = move_to;
        break;
      case kLine:
        out[0] = ConsMoveTo();
        out[1] = path->pts[p];
        last_pt = out[1];
        p += 1;
        break;
      case kConic:
        weight = path->w[wi++];
        [[fallthrough]];
      case kQuad:
        out[0] = ConsMoveTo();
        out[1] = path->pts[p];
        out[2] = path->pts[p + 1];
        last_pt = out[2];
        p += 2;
        break;
      case kCubic:
        out[0] = ConsMoveTo();
        out[1] = path->pts[p];
        out[2] = path->pts[p + 1];
        out[3] = path->pts[p + 2];
        last_pt = out[3];
        p += 3;
        break;
      case kClose:
        verb = AutoClose(out);
        if (verb == kLine) {
          v--;
        } else {
          seg_state = 0;
        }
        last_pt = move_to;
        break;
    }
    return verb;
  }
};

// ---------------------------------------------------------------------------
// Curve helpers (src/geometry/geometry.cc:39-190, cubic.cc:29-61)
// ---------------------------------------------------------------------------
struct QuadCoeff {  // geometry.cc:39-46, eval at :64
  P A, B, C;
  QuadCoeff(P p0, P p1, P p2) {
    C = p0;
    P d{p1.x - C.x, p1.y - C.y};
    B = P{d.x + d.x, d.y + d.y};
    P t2{p1.x + p1.x, p1.y + p1.y};
    A = P{(p2.x - t2.x) + C.x, (p2.y - t2.y) + C.y};
  }
  P eval(float t) const {
    return P{(A.x * t + B.x) * t + C.x, (A.y * t + B.y) * t + C.y};
  }
};

struct CubicCoeff {  // geometry.cc:126-137, eval at :160
  P A, B, C, D;
  CubicCoeff(P p0, P p1, P p2, P p3) {
    A = P{(p3.x + 3.f * (p1.x - p2.x)) - p0.x, (p3.y + 3.f * (p1.y - p2.y)) - p0.y};
    P t{p1.x + p1.x, p1.y + p1.y};
    B = P{3.f * ((p2.x - t.x) + p0.x), 3.f * ((p2.y - t.y) + p0.y)};
    C = P{3.f * (p1.x - p0.x), 3.f * (p1.y - p0.y)};
    D = p0;
  }
  P eval(float t) const {
    return P{((A.x * t + B.x) * t + C.x) * t + D.x,
             ((A.y * t + B.y) * t + C.y) * t + D.y};
  }
};

// Cubic::ToQuads count (cubic.cc:29-38): max(1, ceil(pow(err/432*0.01, 1/6)))
static int CubicQuadCount(const P c[4]) {
  float accuracy = 0.1f;
  double max_hypot2 = 432.0 * accuracy * accuracy;
  P p1x2{c[1].x * 3.f - c[0].x, c[1].y * 3.f - c[0].y};
  P p2x2{c[2].x * 3.f - c[3].x, c[2].y * 3.f - c[3].y};
  P d{p2x2.x - p1x2.x, p2x2.y - p1x2.y};
  float err = d.x * d.x + d.y * d.y;
  double n = std::max(1., std::ceil(std::pow(err / max_hypot2, 1. / 6.0)));
  return (int)n;
}

// Cubic::ToQuads (cubic.cc:29-61): each sub-cubic -> one quad
static void CubicToQuads(const P c[4], std::vector<P>* out /* 3 per quad */) {
  float accuracy = 0.1f;
  double max_hypot2 = 432.0 * accuracy * accuracy;
  P p1x2{c[1].x * 3.f - c[0].x, c[1].y * 3.f - c[0].y};
  P p2x2{c[2].x * 3.f - c[3].x, c[2].y * 3.f - c[3].y};
  P d{p2x2.x - p1x2.x, p2x2.y - p1x2.y};
  float err = d.x * d.x + d.y * d.y;
  double quad_count = std::max(1., std::ceil(std::pow(err / max_hypot2, 1. / 6.0)));
  CubicCoeff cc(c[0], c[1], c[2], c[3]);
  // cubic_tangent(p2, p1) = 3 * (p2 - p1) (cubic.cc:13-17)
  QuadCoeff qc(P{3.f * (c[1].x - c[0].x), 3.f * (c[1].y - c[0].y)},
               P{3.f * (c[2].x - c[1].x), 3.f * (c[2].y - c[1].y)},
               P{3.f * (c[3].x - c[2].x), 3.f * (c[3].y - c[2].y)});
  for (size_t i = 0; i < quad_count; i++) {
    double t0d = i / quad_count;
    double t1d = (i + 1) / quad_count;
    float t1 = (float)t0d, t2 = (float)t1d;
    // Subsegment (cubic.cc:54-61)
    P s0 = cc.eval(t1);
    P s3 = cc.eval(t2);
    float scale = (t2 - t1) * (1.f / 3.f);
    P q1 = qc.eval(t1), q2 = qc.eval(t2);
    P s1{s0.x + q1.x * scale, s0.y + q1.y * scale};
    P s2{s3.x - q2.x * scale, s3.y - q2.y * scale};
    P a{s1.x * 3.f - s0.x, s1.y * 3.f - s0.y};
    P b{s2.x * 3.f - s3.x, s2.y * 3.f - s3.y};
    out->push_back(s0);
    out->push_back(P{(a.x + b.x) / 4.f, (a.y + b.y) / 4.f});
    out->push_back(s3);
  }
}

// Conic::ChopIntoQuadsPOW2(pts, 1) (conic.cc:300-327, chop at :200-260)
static void ConicChopInto2Quads(P p0, P p1, P p2, float w, P out[5]);

// Stroke::QuadPath (stroke.cc:914-962)
static void QuadPath(const Path& src, Path* dst) {
  PathIter iter(src);
  P pts[4];
  std::vector<P> quads;
  for (;;) {
    uint8_t verb = iter.Next(pts);
    switch (verb) {
      case kMove: dst->MoveTo(pts[0]); break;
      case kLine: dst->LineTo(pts[1]); break;
      case kQuad: dst->QuadTo(pts[1], pts[2]); break;
      case kConic: {
        P q[5];
        ConicChopInto2Quads(pts[0], pts[1], pts[2], iter.weight, q);
        dst->QuadTo(q[1], q[2]);
        dst->QuadTo(q[3], q[4]);
      } break;
      case kCubic: {
        quads.clear();
        CubicToQuads(pts, &quads);
        for (size_t i = 0; i < quads.size(); i += 3) dst->QuadTo(quads[i + 1], quads[i + 2]);
      } break;
      case kClose: dst->Close(); break;
      default: return;
    }
  }
}

// ---------------------------------------------------------------------------
// Edges (src/render/sw/sw_edge.hpp:18-81, sw_edge.cc:18-336)
// ---------------------------------------------------------------------------
struct Edge {
  int32_t prev, next;
  Fixed x, y, dx, dy, upper_x, upper_y, lower_y;
  int8_t curve_count;
  uint8_t curve_shift;
  int8_t winding;
  bool is_quad;
  Fixed qx, qy, qdx, qdy, qddx, qddy, q_first_y, q_last_x, q_last_y;
  Fixed snapped_x, snapped_y;
};

static inline Fixed SnapY(Fixed y) {  // sw_edge.hpp:36-41
  return (Fixed)((((uint32_t)y + (uint32_t)(kFixed1 >> (kAccuracy + 1))) >>
                  (16 - kAccuracy))
                 << (16 - kAccuracy));
}
static inline void GoYShift(Edge* e, Fixed dst_y, int y_shift) {  // :55-58
  e->y = dst_y;
  e->x = wrap_add(e->x, e->dx >> y_shift);
}
static inline void GoY(Edge* e, Fixed dst_y) {  // :43-51
  if (dst_y == wrap_add(e->y, kFixed1)) {
    e->x = wrap_add(e->x, e->dx);
    e->y = dst_y;
  } else if (e->y != dst_y) {
    e->x = wrap_add(e->upper_x, FixedMul(e->dx, wrap_sub(e->y, e->upper_y)));
    e->y = dst_y;
  }
}

static bool UpdateLine(Edge* e, Fixed x0, Fixed y0, Fixed x1, Fixed y1,
                       Fixed slope) {  // sw_edge.cc:45-70
  if (y0 > y1) {
    std::swap(x0, x1);
    std::swap(y0, y1);
    e->winding = (int8_t)-e->winding;
  }
  FDot6 x0x1 = FixedToFDot6(wrap_sub(x1, x0));
  FDot6 y0y1 = FixedToFDot6(wrap_sub(y1, y0));
  if (y0y1 == 0) return false;
  e->x = x0;
  e->y = y0;
  e->dx = slope;
  e->dy = (x0x1 == 0 || slope == 0) ? kMaxS32 : std::abs(FDot6Div(y0y1, x0x1));
  e->upper_x = x0;
  e->upper_y = y0;
  e->lower_y = y1;
  return true;
}

static bool SetLine(Edge* e, P p0, P p1) {  // sw_edge.cc:18-43
  const int mul = 1 << kAccuracy;
  Fixed x0 = FDot6ToFixed(ScalarToFDot6(p0.x * mul)) >> kAccuracy;
  Fixed y0 = SnapY(FDot6ToFixed(ScalarToFDot6(p0.y * mul)) >> kAccuracy);
  Fixed x1 = FDot6ToFixed(ScalarToFDot6(p1.x * mul)) >> kAccuracy;
  Fixed y1 = SnapY(FDot6ToFixed(ScalarToFDot6(p1.y * mul)) >> kAccuracy);
  e->winding = 1;
  FDot6 y0y1 = FixedToFDot6(wrap_sub(y1, y0));
  if (y0y1 == 0) return false;
  FDot6 x0x1 = FixedToFDot6(wrap_sub(x1, x0));
  Fixed slope = FDot6Div(x0x1, y0y1);
  e->curve_count = 0;
  e->curve_shift = 0;
  e->is_quad = false;
  return UpdateLine(e, x0, y0, x1, y1, slope);
}

static bool CanBeIgnored(float top, float bottom, Fixed y0, Fixed y1) {  // :72-88
  const int mul = 1 << kAccuracy;
  Fixed start_y = SnapY(FDot6ToFixed(ScalarToFDot6(top * mul)) >> kAccuracy);
  Fixed stop_y = SnapY(FDot6ToFixed(ScalarToFDot6(bottom * mul)) >> kAccuracy);
  return y0 >= stop_y || y1 <= start_y;
}

static inline FDot6 cheap_distance(FDot6 dx, FDot6 dy) {  // :97-102
  dx = std::abs(dx);
  dy = std::abs(dy);
  return std::max(dx, dy) + (std::min(dx, dy) >> 1);
}
static inline int diff_to_shift(FDot6 dx, FDot6 dy, int shiftAA) {  // :104-119
  FDot6 dist = cheap_distance(dx, dy);
  dist = (dist + (1 << (2 + shiftAA))) >> (3 + shiftAA);
  return (32 - CLZ((uint32_t)dist)) >> 1;
}

static bool UpdateQuad(Edge* e) {  // sw_edge.cc:233-292
  int success = 0;
  int count = e->curve_count;
  Fixed oldx = e->qx, oldy = e->qy;
  Fixed dx = e->qdx, dy = e->qdy;
  Fixed newx = 0, newy = 0, nsx = 0, nsy = 0;
  int shift = e->curve_shift;
  do {
    Fixed slope;
    if (--count > 0) {
      newx = wrap_add(oldx, dx >> shift);
      newy = wrap_add(oldy, dy >> shift);
      if (std::abs(dy >> shift) >= kFixed1 * 2) {
        FDot6 diffY = FixedToFDot6(wrap_sub(newy, e->snapped_y));
        slope = diffY ? FDot6Div(FixedToFDot6(wrap_sub(newx, e->snapped_x)), diffY)
                      : kMaxS32;
        nsy = std::min<Fixed>(e->q_last_y, FixedRoundToFixed(newy));
        nsx = wrap_sub(newx, FixedMul(slope, wrap_sub(newy, nsy)));
      } else {
        nsy = std::min(e->q_last_y, SnapY(newy));
        nsx = newx;
        FDot6 diffY = FixedToFDot6(wrap_sub(nsy, e->snapped_y));
        slope = diffY ? FDot6Div(FixedToFDot6(wrap_sub(newx, e->snapped_x)), diffY)
                      : kMaxS32;
      }
      dx = wrap_add(dx, e->qddx);
      dy = wrap_add(dy, e->qddy);
    } else {
      newx = e->q_last_x;
      newy = e->q_last_y;
      nsy = newy;
      nsx = newx;
      FDot6 diffY = wrap_sub(newy, e->snapped_y) >> 10;
      slope = diffY ? FDot6Div(wrap_sub(newx, e->snapped_x) >> 10, diffY) : kMaxS32;
    }
    if (slope < kMaxS32) {
      success = UpdateLine(e, e->snapped_x, e->snapped_y, nsx, nsy, slope);
    }
    oldx = newx;
    oldy = newy;
  } while (count > 0 && !success);
  e->qx = newx;
  e->qy = newy;
  e->qdx = dx;
  e->qdy = dy;
  e->snapped_x = nsx;
  e->snapped_y = nsy;
  e->curve_count = (int8_t)count;
  return success;
}

static bool SetQuad(Edge* e, const P pts[3]) {  // sw_edge.cc:121-231
  float scale = (float)(1 << (kAccuracy + 6));
  FDot6 x0 = (int)(pts[0].x * scale), y0 = (int)(pts[0].y * scale);
  FDot6 x1 = (int)(pts[1].x * scale), y1 = (int)(pts[1].y * scale);
  FDot6 x2 = (int)(pts[2].x * scale), y2 = (int)(pts[2].y * scale);
  int w = 1;
  if (y0 > y2) {
    std::swap(x0, x2);
    std::swap(y0, y2);
    w = -1;
  }
  int top = FDot6Round(y0);
  int bottom = FDot6Round(y2);
  if (top == bottom) return false;
  FDot6 dx = (LeftShift(x1, 1) - x0 - x2) >> 2;
  FDot6 dy = (LeftShift(y1, 1) - y0 - y2) >> 2;
  int shift = diff_to_shift(dx, dy, kAccuracy);
  if (shift == 0) {
    shift = 1;
  } else if (shift > 6) {
    shift = 6;
  }
  e->winding = (int8_t)w;
  e->curve_count = (int8_t)(1 << shift);
  e->curve_shift = (uint8_t)(shift - 1);
  e->is_quad = true;
  Fixed A = FDot6ToFixedDiv2(x0 - x1 - x1 + x2);
  Fixed B = FDot6ToFixed(x1 - x0);
  e->qx = FDot6ToFixed(x0);
  e->qdx = B + (A >> shift);
  e->qddx = A >> (shift - 1);
  A = FDot6ToFixedDiv2(y0 - y1 - y1 + y2);
  B = FDot6ToFixed(y1 - y0);
  e->qy = FDot6ToFixed(y0);
  e->qdy = B + (A >> shift);
  e->qddy = A >> (shift - 1);
  e->q_last_x = FDot6ToFixed(x2);
  e->q_last_y = FDot6ToFixed(y2);
  e->qx >>= kAccuracy;
  e->qy >>= kAccuracy;
  e->qdx >>= kAccuracy;
  e->qdy >>= kAccuracy;
  e->qddx >>= kAccuracy;
  e->qddy >>= kAccuracy;
  e->q_last_x >>= kAccuracy;
  e->q_last_y >>= kAccuracy;
  e->qy = SnapY(e->qy);
  e->q_last_y = SnapY(e->q_last_y);
  e->q_first_y = e->qy;
  e->snapped_x = e->qx;
  e->snapped_y = e->qy;
  UpdateQuad(e);
  return true;
}

static inline void KeepContinuous(Edge* e) {  // sw_edge.cc:294-297
  e->snapped_x = e->x;
  e->snapped_y = e->y;
}

// valid_unit_divide (geometry.hpp:102-125)
static int valid_unit_divide(float number, float denom, float* ratio) {
  if (number < 0) {
    number = -number;
    denom = -denom;
  }
  if (denom == 0 || number == 0 || number >= denom) return 0;
  float r = number / denom;
  if (std::isnan(r)) return 0;
  if (r == 0) return 0;
  *ratio = r;
  return 1;
}

// ChopQuadAtYExtrema (geometry.cc:311-349), ChopQuadAt (:111-124)
static int is_not_monotonic(float a, float b, float c) {
  float ab = a - b;
  float bc = b - c;
  if (ab < 0) bc = -bc;
  return ab == 0 || bc < 0;
}
static void ChopQuadAt(const P src[3], P dst[5], float t) {
  auto interp = [](P a, P b, float tt) {
    return P{a.x + (b.x - a.x) * tt, a.y + (b.y - a.y) * tt};
  };
  P p01 = interp(src[0], src[1], t);
  P p12 = interp(src[1], src[2], t);
  dst[0] = src[0];
  dst[1] = p01;
  dst[2] = interp(p01, p12, t);
  dst[3] = p12;
  dst[4] = src[2];
}
static int ChopQuadAtYExtrema(const P src[3], P dst[5]) {
  float a = src[0].y, b = src[1].y, c = src[2].y;
  if (is_not_monotonic(a, b, c)) {
    float t;
    if (valid_unit_divide(a - b, a - b - b + c, &t)) {
      ChopQuadAt(src, dst, t);
      dst[1].y = dst[3].y = dst[2].y;
      return 1;
    }
    b = std::fabs(a - b) < std::fabs(b - c) ? a : c;
  }
  dst[0] = src[0];
  dst[1] = src[1];
  dst[2] = src[2];
  dst[1].y = b;
  return 0;
}

// SWEdgeBuilder::BuildEdges over PathEdgeIter (sw_edge.cc:299-336,
// src/graphic/path_priv.hpp:75-170)
static void BuildEdges(const Path& path, float top, float bottom,
                       std::vector<Edge>* edges) {
  const auto& verbs = path.verbs;
  size_t vi = 0, pi = 0;
  size_t move_to = 0;
  bool needs_close = false;
  auto add_line = [&](P a, P b) {
    Edge e{};
    if (SetLine(&e, a, b) && !CanBeIgnored(top, bottom, e.upper_y, e.lower_y)) {
      edges->push_back(e);
    }
  };
  auto add_quad = [&](const P* q) {
    Edge e{};
    if (SetQuad(&e, q) && !CanBeIgnored(top, bottom, e.q_first_y, e.q_last_y)) {
      edges->push_back(e);
    }
  };
  auto close_line = [&]() {
    add_line(path.pts[pi - 1], path.pts[move_to]);
    needs_close = false;
  };
  while (true) {
    if (vi == verbs.size()) {
      if (needs_close) close_line();
      return;
    }
    uint8_t v = verbs[vi++];
    switch (v) {
      case kMove:
        if (needs_close) close_line();
        move_to = pi++;
        break;
      case kClose:
        if (needs_close) close_line();
        break;
      default: {
        int n = (v + 2) / 2;
        needs_close = true;
        pi += n;
        const P* seg = &path.pts[pi - (n + 1)];
        if (v == kLine) {
          add_line(seg[0], seg[1]);
        } else if (v == kQuad) {
          P mono[5];
          int k = ChopQuadAtYExtrema(seg, mono);
          for (int i = 0; i <= k; i++) add_quad(&mono[i * 2]);
        }
      } break;
    }
  }
}

// ---------------------------------------------------------------------------
// Span builders (src/render/sw/sw_raster.cc:19-136)
// ---------------------------------------------------------------------------
struct Span {
  int32_t x, y, len, cover;
};

struct SpanBuilder {
  float scan_top;
  int left;
  std::vector<uint8_t> alphas;
  int curr_y = kNaN32;
  std::vector<Span>* out;
  int32_t touch_lo = INT32_MAX, touch_hi = -1;

  void Real(int x, int y, int len, uint8_t a) {  // RealSpanBuilder::BuildSpan
    if (y < scan_top) return;
    out->push_back(Span{x, y, len, a});
  }
  void RealSpans(int x, int y, const uint8_t* aa, int len) {
    if (y < scan_top) return;
    for (int i = 0; i < len; i++) Real(x + i, y, 1, aa[i]);
  }
  static inline uint8_t sat_add(uint8_t a, uint8_t d) {
    return (uint16_t)a + (uint16_t)d > 255 ? 255 : (uint8_t)(a + d);
  }
  // The reference indexes alphas_ without a bounds check; writes outside
  // the path's pixel bounds cannot happen for finite inputs and are dropped.
  void Acc(int x, int y, int width, uint8_t a) {
    if (y < scan_top) return;
    FlushYIfNeed(y);
    int off = x - left;
    for (int i = 0; i < width; i++) {
      if ((unsigned)(off + i) < alphas.size())
        alphas[off + i] = sat_add(alphas[off + i], a);
    }
  }
  void AccSpans(int x, int y, const uint8_t* aa, int len) {
    if (y < scan_top) return;
    FlushYIfNeed(y);
    int off = x - left;
    for (int i = 0; i < len; i++) {
      if ((unsigned)(off + i) < alphas.size())
        alphas[off + i] = sat_add(alphas[off + i], aa[i]);
    }
  }
  void FlushYIfNeed(int new_y) {
    if (curr_y == new_y) return;
    if (curr_y == kNaN32) {
      curr_y = new_y;
      return;
    }
    Flush();
    std::fill(alphas.begin(), alphas.end(), 0);
    curr_y = new_y;
  }
  void Flush() {  // SpanBuilder::Flush (sw_raster.cc:103-136)
    if (curr_y == kNaN32) return;
    size_t curr = 0, n = alphas.size();
    while (curr < n) {
      if (alphas[curr] > 0) {
        size_t start = curr, width = 1;
        uint8_t a = alphas[curr];
        do {
          curr++;
          if (curr >= n) break;
          if (alphas[curr] == a) {
            width++;
          } else {
            break;
          }
        } while (alphas[curr]);
        Real(left + (int)start, curr_y, (int)width, a);
      } else {
        curr++;
      }
    }
  }
};

// ---------------------------------------------------------------------------
// AAA coverage (src/render/sw/sw_raster.cc:138-544)
// ---------------------------------------------------------------------------
static inline uint8_t partial_alpha_h(uint8_t alpha, Fixed h) {  // :151-153
  return (uint8_t)FixedRoundToInt(wrap_mul(alpha, h));
}
static inline uint8_t partial_alpha_a(uint8_t alpha, uint8_t full) {  // :155-157
  return (uint8_t)((alpha * full) >> 8);
}
static inline uint8_t fixed_to_alpha(Fixed f) { return partial_alpha_h(0xFF, f); }
static Fixed approximate_intersection(Fixed l1, Fixed r1, Fixed l2, Fixed r2) {
  if (l1 > r1) std::swap(l1, r1);
  if (l2 > r2) std::swap(l2, r2);
  return wrap_add(std::max(l1, l2), std::min(r1, r2)) / 2;  // :253-262
}
static inline uint8_t trapezoid_to_alpha(Fixed l1, Fixed l2) {  // :264-269
  Fixed area = wrap_add(l1, l2) / 2;
  return (uint8_t)(area >> 8);
}
static inline uint8_t partial_triangle_to_alpha(Fixed a, Fixed b) {  // :271-278
  Fixed area = wrap_mul(wrap_mul(a >> 11, a >> 11), b >> 11);
  return (uint8_t)((area >> 8) & 0xFF);
}

static void blit_single_alpha(SpanBuilder* sb, int y, int x, uint8_t alpha,
                              uint8_t full, bool no_real) {  // :281-289
  if (full == 0xFF && !no_real) {
    sb->Real(x, y, 1, alpha);
  } else {
    sb->Acc(x, y, 1, partial_alpha_a(alpha, full));
  }
}
static void blit_two_alphas(SpanBuilder* sb, int y, int x, uint8_t a1,
                            uint8_t a2, uint8_t full, bool no_real) {  // :291-301
  if (full == 0xFF && !no_real) {
    sb->Real(x, y, 1, a1);
    sb->Real(x + 1, y, 1, a2);
  } else {
    sb->Acc(x, y, 1, a1);
    sb->Acc(x + 1, y, 1, a2);
  }
}
static void blit_full_alpha(SpanBuilder* sb, int y, int x, int len,
                            uint8_t full, bool no_real) {  // :303-310
  if (full == 0xFF && !no_real) {
    sb->Real(x, y, len, full);
  } else {
    sb->Acc(x, y, len, full);
  }
}

static void compute_alpha_above_line(uint8_t* alphas, Fixed l, Fixed r,
                                     Fixed dY, uint8_t full) {  // :314-340
  int R = FixedCeilToInt(r);
  if (R == 0) {
    return;
  } else if (R == 1) {
    alphas[0] = partial_alpha_a((uint8_t)((wrap_sub(wrap_sub(R << 17, l), r)) >> 9), full);
  } else {
    Fixed first = kFixed1 - l;
    Fixed last = r - ((R - 1) << 16);
    Fixed firstH = FixedMul(first, dY);
    alphas[0] = (uint8_t)(FixedMul(first, firstH) >> 9);
    Fixed alpha16 = wrap_add(firstH, dY >> 1);
    for (int i = 1; i < R - 1; ++i) {
      alphas[i] = (uint8_t)(alpha16 >> 8);
      alpha16 = wrap_add(alpha16, dY);
    }
    alphas[R - 1] = (uint8_t)(full - partial_triangle_to_alpha(last, dY));
  }
}

static void compute_alpha_below_line(uint8_t* alphas, Fixed l, Fixed r,
                                     Fixed dY, uint8_t full) {  // :344-370
  int R = FixedCeilToInt(r);
  if (R == 0) {
    return;
  } else if (R == 1) {
    alphas[0] = partial_alpha_a(trapezoid_to_alpha(l, r), full);
  } else {
    Fixed first = kFixed1 - l;
    Fixed last = r - ((R - 1) << 16);
    Fixed lastH = FixedMul(last, dY);
    alphas[R - 1] = (uint8_t)(FixedMul(last, lastH) >> 9);
    Fixed alpha16 = wrap_add(lastH, dY >> 1);
    for (int i = R - 2; i > 0; i--) {
      alphas[i] = (uint8_t)((alpha16 >> 8) & 0xFF);
      alpha16 = wrap_add(alpha16, dY);
    }
    alphas[0] = (uint8_t)(full - partial_triangle_to_alpha(first, dY));
  }
}

static void blit_aaa_trapezoid_row(SpanBuilder* sb, int y, Fixed ul, Fixed ur,
                                   Fixed ll, Fixed lr, Fixed lDY, Fixed rDY,
                                   uint8_t full, bool no_real) {  // :372-455
  int L = FixedFloorToInt(ul), R = FixedCeilToInt(lr);
  int len = R - L;
  if (len == 1) {
    uint8_t alpha = trapezoid_to_alpha(ur - ul, lr - ll);
    blit_single_alpha(sb, y, L, alpha, full, no_real);
    return;
  }
  static thread_local std::vector<uint8_t> buf;
  buf.assign((size_t)(len + 1) * 2, 0);
  uint8_t* alphas = buf.data();
  uint8_t* temp = alphas + len + 1;
  for (int i = 0; i < len; ++i) alphas[i] = full;

  int uL = FixedFloorToInt(ul);
  int lL = FixedCeilToInt(ll);
  if (uL + 2 == lL) {
    Fixed first = IntToFixed(uL) + kFixed1 - ul;
    Fixed second = ll - ul - first;
    uint8_t a1 = (uint8_t)(full - partial_triangle_to_alpha(first, lDY));
    uint8_t a2 = partial_triangle_to_alpha(second, lDY);
    alphas[0] = alphas[0] > a1 ? (uint8_t)(alphas[0] - a1) : 0;
    alphas[1] = alphas[1] > a2 ? (uint8_t)(alphas[1] - a2) : 0;
  } else {
    compute_alpha_below_line(temp + uL - L, ul - IntToFixed(uL), ll - IntToFixed(uL),
                             lDY, full);
    for (int i = uL; i < lL; ++i) {
      if (alphas[i - L] > temp[i - L]) {
        alphas[i - L] = (uint8_t)(alphas[i - L] - temp[i - L]);
      } else {
        alphas[i - L] = 0;
      }
    }
  }
  int uR = FixedFloorToInt(ur);
  int lR = FixedCeilToInt(lr);
  if (uR + 2 == lR) {
    Fixed first = IntToFixed(uR) + kFixed1 - ur;
    Fixed second = lr - ur - first;
    uint8_t a1 = partial_triangle_to_alpha(first, rDY);
    uint8_t a2 = (uint8_t)(full - partial_triangle_to_alpha(second, rDY));
    alphas[len - 2] = alphas[len - 2] > a1 ? (uint8_t)(alphas[len - 2] - a1) : 0;
    alphas[len - 1] = alphas[len - 1] > a2 ? (uint8_t)(alphas[len - 1] - a2) : 0;
  } else {
    compute_alpha_above_line(temp + uR - L, ur - IntToFixed(uR), lr - IntToFixed(uR),
                             rDY, full);
    for (int i = uR; i < lR; ++i) {
      if (alphas[i - L] > temp[i - L]) {
        alphas[i - L] = (uint8_t)(alphas[i - L] - temp[i - L]);
      } else {
        alphas[i - L] = 0;
      }
    }
  }
  if (full == 0xFF && !no_real) {
    sb->RealSpans(L, y, alphas, len);
  } else {
    sb->AccSpans(L, y, alphas, len);
  }
}

static void blit_trapezoid_row(SpanBuilder* sb, int y, Fixed ul, Fixed ur,
                               Fixed ll, Fixed lr, Fixed lDY, Fixed rDY,
                               uint8_t full, bool no_real) {  // :457-544
  if (ul > ur) return;
  if (ll > lr) ll = lr = approximate_intersection(ul, ll, ur, lr);
  if (ul == ur && ll == lr) return;
  if (ul > ll) std::swap(ul, ll);
  if (ur > lr) std::swap(ur, lr);
  Fixed joinLeft = FixedCeilToFixed(ll);
  Fixed joinRite = FixedFloorToFixed(ur);
  if (joinLeft <= joinRite) {
    if (ul < joinLeft) {
      int len = FixedCeilToInt(joinLeft - ul);
      if (len == 1) {
        uint8_t alpha = trapezoid_to_alpha(joinLeft - ul, joinLeft - ll);
        blit_single_alpha(sb, y, ul >> 16, alpha, full, no_real);
      } else if (len == 2) {
        Fixed first = joinLeft - kFixed1 - ul;
        Fixed second = ll - ul - first;
        uint8_t a1 = partial_triangle_to_alpha(first, lDY);
        uint8_t a2 = (uint8_t)(full - partial_triangle_to_alpha(second, lDY));
        blit_two_alphas(sb, y, ul >> 16, a1, a2, full, no_real);
      } else {
        blit_aaa_trapezoid_row(sb, y, ul, joinLeft, ll, joinLeft, lDY, kMaxS32, full,
                               no_real);
      }
    }
    if (joinLeft < joinRite) {
      blit_full_alpha(sb, y, FixedFloorToInt(joinLeft),
                      FixedFloorToInt(joinRite - joinLeft), full, no_real);
    }
    if (lr > joinRite) {
      int len = FixedCeilToInt(lr - joinRite);
      if (len == 1) {
        uint8_t alpha = trapezoid_to_alpha(ur - joinRite, lr - joinRite);
        blit_single_alpha(sb, y, joinRite >> 16, alpha, full, no_real);
      } else if (len == 2) {
        Fixed first = joinRite + kFixed1 - ur;
        Fixed second = lr - ur - first;
        uint8_t a1 = (uint8_t)(full - partial_triangle_to_alpha(first, rDY));
        uint8_t a2 = partial_triangle_to_alpha(second, rDY);
        blit_two_alphas(sb, y, joinRite >> 16, a1, a2, full, no_real);
      } else {
        blit_aaa_trapezoid_row(sb, y, joinRite, ur, joinRite, lr, kMaxS32, rDY, full,
                               no_real);
      }
    }
  } else {
    blit_aaa_trapezoid_row(sb, y, ul, ur, ll, lr, lDY, rDY, full, no_real);
  }
}

// ---------------------------------------------------------------------------
// Scanline sweep (src/render/sw/sw_raster.cc:138-247, 546-677)
// ---------------------------------------------------------------------------
struct EdgeList {
  std::vector<Edge>& e;  // e[n] = head sentinel, e[n+1] = tail sentinel
  int32_t head, tail;
};

static inline bool edges_too_close_e(const std::vector<Edge>& E, int prev,
                                     int next, Fixed lowerY, int head_unused) {
  (void)head_unused;
  // :139-143 ("next && prev": sentinel pointers are never null here)
  if (next < 0 || prev < 0) return false;
  return E[next].upper_y < lowerY &&
         wrap_add(E[prev].x, kFixed1) >= wrap_sub(E[next].x, std::abs(E[next].dx));
}
static inline bool edges_too_close_r(int prevRite, Fixed ul, Fixed ll) {  // :147-149
  return prevRite > FixedFloorToInt(ul) || prevRite > FixedFloorToInt(ll);
}
static inline void update_next_next_y(Fixed y, Fixed next_y, Fixed* nny) {  // :159-163
  *nny = y > next_y && y < *nny ? y : *nny;
}
static inline void check_intersection(const std::vector<Edge>& E, int edge,
                                      Fixed next_y, Fixed* nny) {  // :164-169
  const Edge& e = E[edge];
  const Edge& p = E[e.prev];
  if (p.prev >= 0 && wrap_add(p.x, p.dx) > wrap_add(e.x, e.dx)) {
    *nny = next_y + (kFixed1 >> kAccuracy);
  }
}
static inline void remove_edge(std::vector<Edge>& E, int edge) {
  E[E[edge].prev].next = E[edge].next;
  E[E[edge].next].prev = E[edge].prev;
}
static inline void insert_edge_after(std::vector<Edge>& E, int edge, int after) {
  E[edge].prev = after;
  E[edge].next = E[after].next;
  E[E[after].next].prev = edge;
  E[after].next = edge;
}
static void backward_insert_edge_based_on_x(std::vector<Edge>& E, int edge) {
  Fixed x = E[edge].x;
  int prev = E[edge].prev;
  while (E[prev].prev >= 0 && E[prev].x > x) prev = E[prev].prev;
  if (E[prev].next != edge) {
    remove_edge(E, edge);
    insert_edge_after(E, edge, prev);
  }
}
static int backward_insert_start(std::vector<Edge>& E, int prev, Fixed x) {
  while (E[prev].prev >= 0 && E[prev].x > x) prev = E[prev].prev;
  return prev;
}
static void insert_new_edges(std::vector<Edge>& E, int newEdge, Fixed y,
                             Fixed* nny) {  // :207-247
  if (E[newEdge].upper_y > y) {
    update_next_next_y(E[newEdge].upper_y, y, nny);
    return;
  }
  int prev = E[newEdge].prev;
  if (E[prev].x <= E[newEdge].x) {
    while (E[newEdge].upper_y <= y) {
      check_intersection(E, newEdge, y, nny);
      update_next_next_y(E[newEdge].lower_y, y, nny);
      newEdge = E[newEdge].next;
    }
    update_next_next_y(E[newEdge].upper_y, y, nny);
    return;
  }
  int start = backward_insert_start(E, prev, E[newEdge].x);
  do {
    int next = E[newEdge].next;
    bool skip = false;
    while (true) {
      if (E[start].next == newEdge) {
        skip = true;
        break;
      }
      int after = E[start].next;
      if (E[after].x >= E[newEdge].x) break;
      start = after;
    }
    if (!skip) {
      remove_edge(E, newEdge);
      insert_edge_after(E, newEdge, start);
    }
    check_intersection(E, newEdge, y, nny);
    update_next_next_y(E[newEdge].lower_y, y, nny);
    start = newEdge;
    newEdge = next;
  } while (E[newEdge].upper_y <= y);
  update_next_next_y(E[newEdge].upper_y, y, nny);
}

static void WalkEdges(std::vector<Edge>& E, int head, int tail, bool even_odd,
                      SpanBuilder* sb, int start_y, int stop_y, Fixed left_clip,
                      Fixed right_clip) {  // :546-677
  E[head].x = E[head].upper_x = left_clip;
  E[tail].x = E[tail].upper_x = right_clip;
  Fixed y = std::max(E[E[head].next].upper_y, IntToFixed(start_y));
  Fixed nny = kMaxS32;
  {
    int edge;
    for (edge = E[head].next; E[edge].upper_y <= y; edge = E[edge].next) {
      GoY(&E[edge], y);
      update_next_next_y(E[edge].lower_y, y, &nny);
    }
    update_next_next_y(E[edge].upper_y, y, &nny);
  }
  int winding_mask = even_odd ? 1 : -1;
  while (true) {
    int w = 0;
    bool in_interval = false;
    Fixed prev_x = E[head].x;
    Fixed next_y = std::min(nny, FixedCeilToFixed(y + 1));
    int curr = E[head].next;
    int left_edge = head;
    Fixed left = left_clip;
    Fixed left_dy = 0;
    int prev_right = FixedFloorToInt(left_clip);
    nny = kMaxS32;
    int y_shift = 0;
    if ((next_y - y) & (kFixed1 >> 2)) {
      y_shift = 2;
      next_y = y + (kFixed1 >> 2);
    } else if ((next_y - y) & (kFixed1 >> 1)) {
      y_shift = 1;
    }
    uint8_t full = fixed_to_alpha(next_y - y);
    while (E[curr].upper_y <= y) {
      Edge& ce = E[curr];
      w += ce.winding;
      bool prev_in = in_interval;
      in_interval = (w & winding_mask) != 0;
      bool is_left = in_interval && !prev_in;
      bool is_right = !in_interval && prev_in;
      if (is_left) {
        left = std::max(ce.x, left_clip);
        left_dy = ce.dy;
        left_edge = curr;
        GoYShift(&ce, next_y, y_shift);
      } else if (is_right) {
        Fixed right = std::min(right_clip, ce.x);
        GoYShift(&ce, next_y, y_shift);
        Fixed next_left = std::max(left_clip, E[left_edge].x);
        Fixed next_right = std::min(right_clip, ce.x);
        Fixed right_dy = ce.dy;
        bool no_real = full == 0xFF &&
                       (edges_too_close_r(prev_right, left, E[left_edge].x) ||
                        edges_too_close_e(E, curr, ce.next, next_y, 0));
        blit_trapezoid_row(sb, y >> 16, left, right, next_left, next_right, left_dy,
                           right_dy, full, no_real);
        prev_right = FixedCeilToInt(std::max(right, ce.x));
      } else {
        GoYShift(&ce, next_y, y_shift);
      }
      int next = ce.next;
      while (E[curr].lower_y <= next_y) {
        if (E[curr].curve_count > 0) {
          KeepContinuous(&E[curr]);
          if (!UpdateQuad(&E[curr])) break;
        } else {
          break;
        }
      }
      if (E[curr].lower_y <= next_y) {
        remove_edge(E, curr);
      } else {
        update_next_next_y(E[curr].lower_y, next_y, &nny);
        Fixed new_x = E[curr].x;
        if (new_x < prev_x) {
          backward_insert_edge_based_on_x(E, curr);
        } else {
          prev_x = new_x;
        }
        check_intersection(E, curr, next_y, &nny);
      }
      curr = next;
    }
    if (in_interval) {
      bool no_real = full == 0xFF &&
                     edges_too_close_e(E, E[left_edge].prev, left_edge, next_y, 0);
      blit_trapezoid_row(sb, y >> 16, left, right_clip,
                         std::max(left_clip, E[left_edge].x), right_clip, left_dy, 0,
                         full, no_real);
    }
    y = next_y;
    if (y >= IntToFixed(stop_y)) break;
    insert_new_edges(E, curr, y, &nny);
  }
}

// SWRaster::RastePath (sw_raster.cc:731-786) with SortEdges/ProcessEdges
// (:679-729). Spans go to *spans in emission order; returns the number of
// edges built.
struct RasterStats {
  uint64_t edges = 0, tie_groups = 0;
};

// The canvas's global clip bounds in device space (Canvas::
// global_clip_bounds_stack_, canvas.cc:19-22,463-476): kMaxCullRect
// (include/skity/render/canvas.hpp:26) unless a ClipRect narrowed them.
struct Clip {
  float l = -1e9f, t = -1e9f, r = 1e9f, b = 1e9f;
};

static void RastePathQuads(const Path& quad, bool even_odd, std::vector<Span>* spans,
                           RasterStats* st, Clip clip = Clip()) {
  spans->clear();
  // bounds of the (identity-)transformed quad path (path.cc:1341-1360)
  size_t npts = quad.pts.size();
  if (quad.verbs.size() > 1 && quad.verbs.back() == kMove) npts--;
  if (npts == 0) return;
  float l = quad.pts[0].x, t = quad.pts[0].y, r = l, b = t;
  for (size_t i = 1; i < npts; ++i) {
    l = std::min(l, quad.pts[i].x);
    r = std::max(r, quad.pts[i].x);
    t = std::min(t, quad.pts[i].y);
    b = std::max(b, quad.pts[i].y);
  }
  float bl = std::floor(l), bt = std::floor(t), br = std::ceil(r), bb = std::ceil(b);
  // scan_bounds.Intersect(clip_bounds) (sw_raster.cc:746-748, rect.cc:160-172);
  // an empty intersection leaves nothing to scan
  float sl = std::max(l, clip.l), sr = std::min(r, clip.r);
  float stp = std::max(t, clip.t), sbm = std::min(b, clip.b);
  if (!(sl < sr && stp < sbm)) return;
  sl = std::floor(sl);
  stp = std::floor(stp);
  sr = std::ceil(sr);
  sbm = std::ceil(sbm);
  if (!(sl < sr && stp < sbm)) return;

  std::vector<Edge> E;
  BuildEdges(quad, stp, sbm, &E);
  if (E.empty()) return;
  size_t n = E.size();
  if (st) st->edges += n;
  // SortEdges: std::sort by (upper_y, x, dx) over the build order
  std::vector<int32_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = (int32_t)i;
  std::sort(order.begin(), order.end(), [&](int32_t ia, int32_t ib) {
    const Edge& a = E[ia];
    const Edge& c = E[ib];
    int va = a.upper_y, vb = c.upper_y;
    if (va == vb) {
      va = a.x;
      vb = c.x;
    }
    if (va == vb) {
      va = a.dx;
      vb = c.dx;
    }
    return va < vb;
  });
  if (st) {
    for (size_t i = 1; i < n; ++i) {
      const Edge& a = E[order[i - 1]];
      const Edge& c = E[order[i]];
      if (a.upper_y == c.upper_y && a.x == c.x && a.dx == c.dx) st->tie_groups++;
    }
  }
  std::vector<Edge> S(n + 2);
  for (size_t i = 0; i < n; ++i) S[i] = E[order[i]];
  int head = (int)n, tail = (int)n + 1;
  for (size_t i = 0; i < n; ++i) {
    S[i].prev = i == 0 ? head : (int)i - 1;
    S[i].next = i + 1 == n ? tail : (int)i + 1;
  }
  Edge& H = S[head];
  H = Edge{};
  H.prev = -1;
  H.next = 0;
  H.upper_y = H.lower_y = kMinS32;
  H.x = kMinS32;
  H.dx = 0;
  H.dy = kMaxS32;
  H.upper_x = kMinS32;
  Edge& T = S[tail];
  T = Edge{};
  T.prev = (int)n - 1;
  T.next = -1;
  T.upper_y = T.lower_y = kMaxS32;
  T.x = kMaxS32;
  T.dx = 0;
  T.dy = kMaxS32;
  T.upper_x = kMaxS32;

  SpanBuilder sb;
  sb.scan_top = stp;
  sb.left = (int)bl;
  sb.alphas.assign((size_t)(int)(br - bl), 0);
  sb.out = spans;
  int start_y = (int)bt;
  int stop_y = (int)sbm;
  // static_cast<uint32_t>(float) << 16 with x86-64 conversion semantics
  // (cvttss2si into a 64-bit register, low 32 bits kept)
  Fixed left_bound = (Fixed)((uint32_t)(int64_t)sl << 16);
  Fixed right_bound = (Fixed)((uint32_t)(int64_t)sr << 16);
  WalkEdges(S, head, tail, even_odd, &sb, start_y, stop_y, left_bound, right_bound);
  sb.Flush();
}

// ---------------------------------------------------------------------------
// Colour (src/graphic/color.cc:44-59, color_priv.hpp:20-72, color_priv.cc:97-108)
// ---------------------------------------------------------------------------
static inline uint32_t ColorSetARGB(uint32_t a, uint32_t r, uint32_t g, uint32_t b) {
  return (a << 24) | (r << 16) | (g << 8) | b;
}
static inline uint32_t GetA(uint32_t c) { return (c >> 24) & 0xFF; }
static inline uint32_t GetR(uint32_t c) { return (c >> 16) & 0xFF; }
static inline uint32_t GetG(uint32_t c) { return (c >> 8) & 0xFF; }
static inline uint32_t GetB(uint32_t c) { return c & 0xFF; }
static inline uint8_t ChannelToByte(float v) {
  float s = v * 255;
  s = std::min(std::max(s, 0.f), 255.f);
  return (uint8_t)s;
}
static inline uint32_t Color4fToColor(const float c[4]) {  // color.cc:53-59
  return ColorSetARGB(ChannelToByte(c[3]), ChannelToByte(c[0]), ChannelToByte(c[1]),
                      ChannelToByte(c[2]));
}
static inline uint32_t MulDiv255Round(uint32_t a, uint32_t b) {  // :31-47
  uint32_t prod = a * b + 128;
  return (prod + (prod >> 8)) >> 8;
}
static inline uint32_t ColorToPMColor(uint32_t c) {  // color_priv.cc:105-108
  uint32_t a = GetA(c), r = GetR(c), g = GetG(c), b = GetB(c);
  if (a != 255) {
    r = MulDiv255Round(r, a);
    g = MulDiv255Round(g, a);
    b = MulDiv255Round(b, a);
  }
  return (a << 24) | (r << 16) | (g << 8) | b;
}
static inline uint32_t AlphaMulQ(uint32_t c, uint32_t scale) {  // :62-68
  uint32_t mask = 0xFF00FF;
  uint32_t rb = ((c & mask) * scale) >> 8;
  uint32_t ag = ((c >> 8) & mask) * scale;
  return (rb & mask) | (ag & ~mask);
}
static inline uint32_t PMSrcOver(uint32_t src, uint32_t dst) {  // :70-72
  return src + AlphaMulQ(dst, 255 - GetA(src) + 1);
}
static inline uint32_t Alpha255To256(uint32_t a) { return a + 1; }  // :20-25
static inline uint32_t PMColorMul(uint32_t s, uint32_t d) {        // :74-79
  return (MulDiv255Round(GetA(s), GetA(d)) << 24) | (MulDiv255Round(GetR(s), GetR(d)) << 16) |
         (MulDiv255Round(GetG(s), GetG(d)) << 8) | MulDiv255Round(GetB(s), GetB(d));
}

// SoftLightComponent (blend_mode.cc:91-108); x = colour, y = alpha.
static float SoftLightComponent(float sx, float sy, float dx, float dy) {
  if (2.f * sx <= sy) return dx * dx * (sy - 2 * sx) / dy + (1 - dy) * sx + dx * (-sy + 2 * sx + 1);
  if (4.f * dx <= dy) {
    float dsq = dx * dx, dcub = dsq * dx, dasq = dy * dy, dacub = dasq * dy;
    return (dasq * (sx - dx * (3 * sy - 6 * sx - 1)) + 12 * dy * dsq * (sy - 2 * sx) -
            16 * dcub * (sy - 2 * sx) - dacub * sx) /
           dasq;
  }
  return dx * (sy - 2 * sx + 1) + sx - std::sqrt(dy * dx) * (sy - 2 * sx) - dy * sx;
}

// PorterDuffBlend (blend_mode.cc:123-191).  Modes past kScreen other than
// kSoftLight fall back to kDefault (kSrcOver).
static uint32_t PorterDuffBlend(uint32_t src, uint32_t dst, int mode) {
  if (mode > 14 && mode != 21) mode = 3;
  switch (mode) {
    case 0: return 0;
    case 1: return src;
    case 2: return dst;
    case 3:
      if (GetA(src) == 0) return dst;
      return PMSrcOver(src, dst);
    case 4:
      if (GetA(dst) == 255) return dst;
      return PMSrcOver(dst, src);
    case 5: return GetA(dst) == 255 ? src : AlphaMulQ(src, Alpha255To256(GetA(dst)));
    case 6:
      if (GetA(src) == 255) return dst;
      return AlphaMulQ(dst, Alpha255To256(GetA(src)));
    case 7: return GetA(dst) == 0 ? src : AlphaMulQ(src, Alpha255To256(255 - GetA(dst)));
    case 8:
      if (GetA(src) == 0) return dst;
      return AlphaMulQ(dst, Alpha255To256(255 - GetA(src)));
    case 9:
      return AlphaMulQ(src, Alpha255To256(GetA(dst))) +
             AlphaMulQ(dst, Alpha255To256(255 - GetA(src)));
    case 10:
      return AlphaMulQ(dst, Alpha255To256(GetA(src))) +
             AlphaMulQ(src, Alpha255To256(255 - GetA(dst)));
    case 11:
      return AlphaMulQ(src, Alpha255To256(255 - GetA(dst))) +
             AlphaMulQ(dst, Alpha255To256(255 - GetA(src)));
    case 12:
      return ColorSetARGB(std::min(GetA(src) + GetA(dst), 255u), std::min(GetR(src) + GetR(dst), 255u),
                          std::min(GetG(src) + GetG(dst), 255u), std::min(GetB(src) + GetB(dst), 255u));
    case 13: return PMColorMul(src, dst);
    case 14: return src + dst - PMColorMul(src, dst);
    default: {  // kSoftLight (:110-121)
      if (GetA(dst) == 0) return src;
      float s[4] = {GetR(src) / 255.f, GetG(src) / 255.f, GetB(src) / 255.f, GetA(src) / 255.f};
      float d[4] = {GetR(dst) / 255.f, GetG(dst) / 255.f, GetB(dst) / 255.f, GetA(dst) / 255.f};
      float out[4] = {SoftLightComponent(s[0], s[3], d[0], d[3]),
                      SoftLightComponent(s[1], s[3], d[1], d[3]),
                      SoftLightComponent(s[2], s[3], d[2], d[3]), s[3] + (1 - s[3]) * d[3]};
      return Color4fToColor(out);
    }
  }
}

// ---------------------------------------------------------------------------
// Brushes (src/render/sw/sw_span_brush.cc:66-383)
// ---------------------------------------------------------------------------
struct Mat {  // skity::Matrix, column-major e[col][row]
  float e[4][4];
  static Mat Identity() {
    Mat m{};
    for (int i = 0; i < 4; ++i) m.e[i][i] = 1.f;
    return m;
  }
  bool IsIdentity() const {  // glm::isIdentity(m, FLT_EPSILON)
    for (int c = 0; c < 4; ++c)
      for (int r = 0; r < 4; ++r) {
        float want = c == r ? 1.f : 0.f;
        if (!(std::fabs(e[c][r] - want) < 1.1920928955078125e-7f)) return false;
      }
    return true;
  }
};
static Mat MatMul(const Mat& a, const Mat& b) {  // matrix.cc:452-460
  if (a.IsIdentity()) return b;
  if (b.IsIdentity()) return a;
  Mat r{};
  for (int j = 0; j < 4; ++j)
    for (int k = 0; k < 4; ++k) {
      float v = a.e[0][k] * b.e[j][0];
      v = v + a.e[1][k] * b.e[j][1];
      v = v + a.e[2][k] * b.e[j][2];
      v = v + a.e[3][k] * b.e[j][3];
      r.e[j][k] = v;
    }
  return r;
}
static Mat MatScale(float sx, float sy) {
  Mat m = Mat::Identity();
  m.e[0][0] = sx;
  m.e[1][1] = sy;
  return m;
}
static Mat MatTranslate(float tx, float ty) {
  Mat m = Mat::Identity();
  m.e[3][0] = tx;
  m.e[3][1] = ty;
  return m;
}

struct Gradient {
  int type;  // 1 linear, 2 radial, 3 sweep, 4 two-point conical
  int tile;
  int count;
  bool has_offsets;
  const float* colors;   // 4 * count
  const float* offsets;  // count
  float p0[2], p1[2], radius[2];
};

// PointsToUnit (sw_span_brush.cc:164-200)
static Mat PointsToUnit(const Gradient& g) {
  if (g.type == 3) return MatTranslate(-g.p0[0], -g.p0[1]);
  if (g.type == 4) return Mat::Identity();  // the conical brush keeps its own
  if (g.type == 1) {
    float sx = g.p0[0], sy = g.p0[1];
    float ssx = g.p1[0] - sx, ssy = g.p1[1] - sy;
    float length = std::sqrt(ssx * ssx + ssy * ssy);
    float scale = length > 0 ? 1.0f / length : 0;
    float ux = ssx * scale, uy = ssy * scale;
    float sine = -uy, cosine = ux;
    Mat rot = Mat::Identity();
    rot.e[0][0] = cosine;
    rot.e[1][0] = -sine;
    rot.e[0][1] = sine;
    rot.e[1][1] = cosine;
    return MatMul(MatMul(rot, MatScale(scale, scale)), MatTranslate(-sx, -sy));
  }
  float radius = g.radius[0];
  float scale = radius > 0 ? 1.0f / radius : 0;
  return MatMul(MatScale(scale, scale), MatTranslate(-g.p0[0], -g.p0[1]));
}

static inline float RemapFloatTile(float t, int tile) {  // :21-32
  if (tile == 0) {
    t = std::min(std::max(t, 0.0f), 1.0f);
  } else if (tile == 1) {
    t = t - std::floor(t);
  } else if (tile == 2) {
    // float - 2 * std::floor(float * 0.5) - 1 evaluates in double
    float t1 = t - 1;
    float t2 = (float)((double)t1 - 2.0 * std::floor((double)t1 * 0.5) - 1.0);
    t = std::fabs(t2);
  }
  return t;
}

// GradientColorBrush::LerpColor (sw_span_brush.cc:232-296)
static void LerpColor(const Gradient& g, float current, float out[4]) {
  const float kNZ = 1.0f / (1 << 12);
  if (std::fabs(current) <= kNZ) {
    current = 0.0f;
  } else if (std::fabs(current - 1.0f) <= kNZ) {
    current = 1.0f;
  }
  if (g.tile == 3 && (current < 0.0 || current >= 1.0)) {
    out[0] = out[1] = out[2] = out[3] = 0;
    return;
  }
  current = RemapFloatTile(current, g.tile);
  int color_count = g.count;
  int stop_count = g.has_offsets ? g.count : 0;
  int si = 0, ei = 1;
  float step = 1.f / (color_count - 1);
  if (stop_count > 0 && current <= g.offsets[0]) {
    std::memcpy(out, g.colors, 16);
    return;
  }
  int i = 0;
  float start = 0.f, end = 0.f;
  for (i = 0; i < color_count - 1; i++) {
    if (stop_count > 0) {
      start = g.offsets[i];
      end = g.offsets[i + 1];
    } else {
      start = step * i;
      end = step * (i + 1);
    }
    if (current >= start && current <= end) {
      si = i;
      ei = i + 1;
      break;
    }
  }
  if (i == color_count - 1 && color_count > 0) {
    std::memcpy(out, g.colors + 4 * (color_count - 1), 16);
    return;
  }
  float total = end - start;
  float value = current - start;
  float mix = 0.5f;
  if (total > 0) mix = value / total;
  const float* c0 = g.colors + 4 * si;
  const float* c1 = g.colors + 4 * ei;
  for (int k = 0; k < 4; ++k) out[k] = c0[k] * (1 - mix) + c1[k] * mix;
}

// MapPoint (sw_span_brush.cc:224-227)
static inline void MapPoint(const Mat& m, float x, float y, float* ox, float* oy) {
  *ox = x * m.e[0][0] + y * m.e[1][0] + m.e[3][0];
  *oy = x * m.e[0][1] + y * m.e[1][1] + m.e[3][1];
}

// ConicalGradientColorBrush's state after OnPreBrush (sw_span_brush.cc:394-437)
struct Conical {
  float c0[4], c1[4];  // Points (z = 0, w = 1)
  float r0 = 0, r1 = 0, r1_square = 0;
  float delta_center = 0, delta_radius = 0;
  bool radial = false, strip = false, swap_01 = false;
  float scale = 0, scale_sign = 0, bias = 0, f = 0;
  Mat c0c1, cfc1;
};

static float Length4(const float a[4]) {  // Vec4::Length (vector.hpp:233-281)
  return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + a[3] * a[3]);
}

static Mat LineToUnit(const float p0[4], const float p1[4]) {  // PointsToUnit(p0, p1)
  Gradient g{};
  g.type = 1;
  g.p0[0] = p0[0];
  g.p0[1] = p0[1];
  g.p1[0] = p1[0];
  g.p1[1] = p1[1];
  return PointsToUnit(g);
}

static Conical ConicalPreBrush(const Gradient& g) {
  const float kNZ = 1.0f / (1 << 12);
  Conical c;
  c.c0[0] = g.p0[0], c.c0[1] = g.p0[1], c.c0[2] = 0.f, c.c0[3] = 1.f;
  c.c1[0] = g.p1[0], c.c1[1] = g.p1[1], c.c1[2] = 0.f, c.c1[3] = 1.f;
  c.r0 = g.radius[0];
  c.r1 = g.radius[1];
  float d[4];
  for (int i = 0; i < 4; ++i) d[i] = c.c1[i] - c.c0[i];
  c.delta_center = Length4(d);
  c.delta_radius = std::abs(c.r1 - c.r0);
  if (c.r0 < 0 || c.r1 < 0) return c;
  c.radial = c.delta_center < kNZ;
  c.strip = c.delta_radius < kNZ;
  if (c.radial) {
    if (!c.strip) {
      c.scale = 1.0 / c.delta_radius;
      c.scale_sign = c.delta_radius < 0 ? -1.f : 1.f;
      c.bias = c.r0 / c.delta_radius;
    }
  } else if (c.strip) {
    c.c0c1 = LineToUnit(c.c0, c.c1);
  } else {
    c.swap_01 = c.r1 < kNZ;
    if (c.swap_01) {
      for (int i = 0; i < 4; ++i) std::swap(c.c0[i], c.c1[i]);
      std::swap(c.r0, c.r1);
    }
    c.f = c.r0 / (c.r0 - c.r1);
    float cf[4], e[4];
    for (int i = 0; i < 4; ++i) cf[i] = c.c0[i] * (1.f - c.f) + c.c1[i] * c.f;
    for (int i = 0; i < 4; ++i) e[i] = c.c1[i] - cf[i];
    c.r1 = c.r1 / Length4(e);
    c.r1_square = c.r1 * c.r1;
    c.cfc1 = LineToUnit(cf, c.c1);
  }
  return c;
}

// CalculateConical (sw_span_brush.cc:441-507); false: transparent
static bool ConicalParam(const Conical& c, const Mat& d2l, int x, int y, float* out) {
  if (c.r0 < 0 || c.r1 < 0) return false;
  float px, py;
  MapPoint(d2l, x + 0.5f, y + 0.5f, &px, &py);
  float t = 0;
  if (c.radial) {
    if (c.strip) return false;
    float qx = (px - c.c0[0]) * c.scale, qy = (py - c.c0[1]) * c.scale;
    t = std::sqrt(qx * qx + qy * qy) * c.scale_sign - c.bias;
  } else if (c.strip) {
    float r = c.r0 / c.delta_center;
    float r_2 = r * r;
    float qx, qy;
    MapPoint(c.c0c1, px, py, &qx, &qy);
    t = r_2 - qy * qy;
    if (t < 0.0) return false;
    t = qx + ::sqrt(t);  // unqualified sqrt of a float: the C library's double sqrt
  } else {
    float qx, qy;
    MapPoint(c.cfc1, px, py, &qx, &qy);
    float xt = -1.f;
    if (std::abs(c.r1 - 1.f) < 1.0f / (1 << 12)) {
      xt = (qx * qx + qy * qy) / 2;
    } else if (c.r1 > 1.f) {
      float m = c.r1_square - 1.f;
      float delta = m * qy * qy + c.r1_square * qx * qx;
      xt = (std::sqrt(delta) - qx) / m;
    } else {
      float m = c.r1_square - 1.f;
      float delta = m * qy * qy + c.r1_square * qx * qx;
      if (delta > 0) {
        float xt1 = (std::sqrt(delta) - qx) / m;
        float xt2 = (-std::sqrt(delta) - qx) / m;
        xt = 1.f - c.f < 0 ? std::min(xt1, xt2) : std::max(xt1, xt2);
      }
    }
    if (xt < 0) return false;
    t = c.f + (1.f - c.f) * xt;
    if (c.swap_01) t = 1.0 - t;
  }
  *out = t;
  return true;
}

// A paint's colour filter (src/effect/color_filter.cc:56-186), as the
// stream records it: type 0 none, 1 blend, 2 matrix, 3 linear->sRGB,
// 4 sRGB->linear, 5 compose.
struct FilterRec {
  uint32_t type, mode, color, pad;
  float matrix[20];
};
static_assert(sizeof(FilterRec) == 96, "colour filter layout");

// UnPreMultiply::g_table_ (color_priv.cc:52-95): entry a is 255 * 2^24 / a,
// rounded to nearest.
static uint32_t UnpremulScale(uint32_t a) {
  return a == 0 ? 0u : (uint32_t)((((uint64_t)255 << 24) + a / 2) / a);
}
static uint32_t PMColorToColor(uint32_t c) {  // color_priv.cc:97-103
  uint32_t a = GetA(c), scale = UnpremulScale(a);
  auto apply = [&](uint32_t v) -> uint32_t { return (scale * v + (1u << 23)) >> 24; };
  return ColorSetARGB(a, apply(GetR(c)), apply(GetG(c)), apply(GetB(c)));
}

// The sRGB transfer tables of SRGBGammaColorFilter (color_filter.cc:121-166),
// rebuilt from the transfer functions: floor(255 * f(i / 255)), the argument
// and the product in float, f in double.
struct SRGBTables {
  uint8_t to_srgb[256], to_linear[256];
  SRGBTables() {
    for (int i = 0; i < 256; ++i) {
      float x = i / 255.f;
      double xd = x;
      double e = xd <= 0.0031308 ? 12.92 * xd : 1.055 * std::pow(xd, 1 / 2.4) - 0.055;
      double l = xd <= 0.04045 ? xd / 12.92 : std::pow((xd + 0.055) / 1.055, 2.4);
      to_srgb[i] = (uint8_t)std::floor((float)e * 255.f);
      to_linear[i] = (uint8_t)std::floor((float)l * 255.f);
    }
  }
};

static uint32_t ApplyColorFilter(const FilterRec* f, uint32_t c) {
  if (!f) return c;
  switch (f->type) {
    case 1:  // BlendColorFilter::OnFilterColor
      return PorterDuffBlend(ColorToPMColor(f->color), c, (int)f->mode);
    case 2: {  // MatrixColorFilter::OnFilterColor
      int16_t m[4][5];
      for (int i = 0; i < 20; ++i) m[i / 5][i % 5] = (int16_t)(f->matrix[i] * 255);
      uint32_t src = PMColorToColor(c);
      int32_t v[4] = {(int32_t)GetR(src), (int32_t)GetG(src), (int32_t)GetB(src), (int32_t)GetA(src)};
      uint8_t out[4];
      for (int i = 0; i < 4; ++i) {
        int32_t mul = v[0] * m[i][0] + v[1] * m[i][1] + v[2] * m[i][2] + v[3] * m[i][3];
        out[i] = (uint8_t)std::clamp(mul / 255 + m[i][4], 0, 255);
      }
      return ColorToPMColor(ColorSetARGB(out[3], out[0], out[1], out[2]));
    }
    case 3:
    case 4: {  // SRGBGammaColorFilter::OnFilterColor
      static const SRGBTables tables;
      const uint8_t* t = f->type == 3 ? tables.to_srgb : tables.to_linear;
      uint32_t src = PMColorToColor(c);
      return ColorToPMColor(ColorSetARGB(GetA(src), t[GetR(src)], t[GetG(src)], t[GetB(src)]));
    }
    default:  // none; ComposeColorFilter::OnFilterColor returns its input
      return c;
  }
}

// BitmapSampler (bitmap_sampler.cc:12-108) over an RGBA8 pixmap, and
// PixmapBrush::CalculateColor's premultiply of unpremultiplied pixels
// (sw_span_brush.cc:568-579).
struct Sampler {
  const uint8_t* px = nullptr;
  uint32_t w = 0, h = 0;
  int filter = 0;            // 0 nearest, else bilinear (cubic samples bilinearly)
  int tile_x = 0, tile_y = 0;  // TileMode: clamp, repeat, mirror, decal
  bool unpremul = false;

  static float Remap(float t, int mode) {  // RemapFloatTile
    switch (mode) {
      case 0: return std::clamp(t, 0.0f, 1.0f);
      case 1: return t - std::floor(t);  // FloatFract
      case 2: {
        float t1 = t - 1;
        float t2 = t1 - 2 * std::floor(t1 * 0.5) - 1;  // floor of a double
        return std::abs(t2);
      }
      default: return t;
    }
  }
  // glm::clamp<uint32_t>(v, 0, n - 1): the float argument converts to
  // uint32_t the way x86-64 builds of the reference convert it (through a
  // 64-bit signed integer: -1 becomes 0xFFFFFFFF, clamped to n - 1).
  static uint32_t Index(float v, uint32_t n) {
    uint32_t u = (uint32_t)(int64_t)v;
    return std::min(u, n - 1);
  }
  void Texel(float x, float y, float out[4]) const {  // SampleXY, Color4fFromColor
    const uint8_t* c = px + ((size_t)Index(y, h) * w + Index(x, w)) * 4;
    for (int i = 0; i < 4; ++i) out[i] = c[i] / 255.f;  // r, g, b, a
  }
  uint32_t Color(float u, float v) const {  // GetColor, then the brush's premultiply
    if ((tile_x == 3 && (u < 0.0 || u >= 1.0)) || (tile_y == 3 && (v < 0.0 || v >= 1.0)))
      return 0;
    u = Remap(u, tile_x);
    v = Remap(v, tile_y);
    float c[4];
    if (filter != 0) {  // SampleUnitLinear
      float fw = (float)w, fh = (float)h;
      float x = u * fw, y = v * fh;
      float i0 = std::floor(x - 0.5f), j0 = std::floor(y - 0.5f);
      if (tile_x == 1) i0 = i0 - fw * std::floor(i0 / fw);  // glm::mod
      if (tile_y == 1) j0 = j0 - fh * std::floor(j0 / fh);
      float i1 = i0 + 1.0f, j1 = j0 + 1.0f;
      if (tile_x == 1) i1 = i1 - fw * std::floor(i1 / fw);
      if (tile_y == 1) j1 = j1 - fh * std::floor(j1 / fh);
      float fx = x - 0.5f, fy = y - 0.5f;
      float a = fx - std::floor(fx), b = fy - std::floor(fy);  // glm::fract
      float t00[4], t10[4], t01[4], t11[4];
      Texel(i0, j0, t00);
      Texel(i1, j0, t10);
      Texel(i0, j1, t01);
      Texel(i1, j1, t11);
      float k00 = (1 - a) * (1 - b), k10 = a * (1 - b), k01 = (1 - a) * b, k11 = a * b;
      for (int i = 0; i < 4; ++i) c[i] = k00 * t00[i] + k10 * t10[i] + k01 * t01[i] + k11 * t11[i];
    } else {  // SampleUnitNearest
      Texel(u * (float)w, v * (float)h, c);
    }
    uint32_t col = Color4fToColor(c);
    return unpremul ? ColorToPMColor(col) : col;
  }
};

struct Brush {
  int kind = 0;  // 0 solid, 1 linear, 2 radial, 3 sweep, 4 two-point conical, 5 image shader
  Sampler img{};
  uint32_t solid = 0;
  Gradient g{};
  Mat m{};
  Mat d2l = Mat::Identity();  // conical: device_to_local, mapped before its own transforms
  Conical con{};
  uint8_t global_alpha = 255;
  const FilterRec* filter = nullptr;  // the paint's colour filter

  uint32_t ColorAt(int x, int y) const {
    if (kind == 0) return solid;
    float c[4];
    if (kind == 4) {
      float t;
      if (!ConicalParam(con, d2l, x, y, &t)) return 0;  // Colors::kTransparent
      LerpColor(g, t, c);
      return ColorToPMColor(Color4fToColor(c));
    }
    float mx, my;
    MapPoint(m, x + 0.5f, y + 0.5f, &mx, &my);
    if (kind == 5) return img.Color(mx, my);
    float t;
    if (kind == 1) {
      t = mx;
    } else if (kind == 2) {
      t = std::sqrt(mx * mx + my * my);
    } else {  // sweep (sw_span_brush.cc:336-349)
      float angle = std::atan2(-my, -mx);
      constexpr float k1Over2Pi = 0.1591549430918;
      t = (angle * k1Over2Pi + 0.5 + g.radius[0]) * g.radius[1];
    }
    LerpColor(g, t, c);
    return ColorToPMColor(Color4fToColor(c));
  }
};

struct Target {
  uint8_t* px;
  int w, h;
  int band0 = 0, band1 = 1 << 30;  // rows this target blends (banded replay)
  uint32_t Get(int x, int y) const {  // bitmap.cc:25-33 (RGBA)
    const uint8_t* c = px + ((size_t)y * w + x) * 4;
    return ColorSetARGB(c[3], c[0], c[1], c[2]);
  }
  void Set(int x, int y, uint32_t c) {  // bitmap.cc:52-64
    uint8_t* d = px + ((size_t)y * w + x) * 4;
    d[0] = (uint8_t)GetR(c);
    d[1] = (uint8_t)GetG(c);
    d[2] = (uint8_t)GetB(c);
    d[3] = (uint8_t)GetA(c);
  }
  // SWRenderTarget::BlendPixel with FastBlend (sw_render_target.cc:12-141)
  void Blend(int x, int y, uint32_t src, int mode) {
    if ((unsigned)x >= (unsigned)w || (unsigned)y >= (unsigned)h) return;
    if (mode == 0) {  // kClear
      Set(x, y, 0);
      return;
    }
    if (mode == 1) {  // kSrc
      Set(x, y, src);
      return;
    }
    if (mode == 2) return;  // kDst
    uint32_t a = GetA(src);
    if (mode == 3) {  // kSrcOver
      if (a == 0) return;
      if (a == 255) {
        Set(x, y, src);
        return;
      }
    } else if (mode == 4) {  // kDstOver over an opaque pixel
      if (GetA(Get(x, y)) == 255) return;
    } else if (mode == 6) {  // kDstIn
      if (a == 255) return;
      if (a == 0) {
        Set(x, y, 0);
        return;
      }
    } else if (mode == 8) {  // kDstOut
      if (a == 0) return;
      if (a == 255) {
        Set(x, y, 0);
        return;
      }
    }
    Set(x, y, PorterDuffBlend(src, Get(x, y), mode));
  }
};

// SWSpanBrush::Brush + BrushH (sw_span_brush.cc:66-138)
static uint64_t BrushSpans(const std::vector<Span>& spans, const Brush& br, int mode,
                           Target* t) {
  uint64_t frags = 0;
  for (const Span& s : spans) {
    int x = s.x, y = s.y, len = s.len;
    if (y < 0 || y >= t->h) continue;
    if (y < t->band0 || y >= t->band1) continue;
    if (x >= t->w || x + len < 0) continue;
    if (x < 0) {
      len += x;
      x = 0;
    }
    if (x + len >= t->w) len = t->w - x;
    if (len <= 0) continue;
    uint8_t alpha = (uint8_t)(s.cover & br.global_alpha);
    frags += (uint64_t)len;
    for (int i = 0; i < len; ++i) {
      uint32_t c = br.ColorAt(x + i, y);
      if (alpha != 255) c = AlphaMulQ(c, alpha);
      c = ApplyColorFilter(br.filter, c);
      t->Blend(x + i, y, c, mode);
    }
  }
  return frags;
}

// ---------------------------------------------------------------------------
// Scene stream (skity_gb300/scene.py layout) and the canvas replay
// ---------------------------------------------------------------------------
struct PaintRec {
  uint32_t style, cap, join, blend, fill_type;
  int32_t gradient;
  uint32_t blur_style;
  float blur_radius;
  float fill_color[4];
  float stroke_color[4];
  float stroke_width, miter;
  float translate[2];  // canvas translation of the draw
};
static_assert(sizeof(PaintRec) == 80, "paint layout");
struct GradRec {
  uint32_t type, tile_mode, stop_count, stop_start, has_offsets, reserved;
  float p0[2], p1[2], radius[2];
};
static_assert(sizeof(GradRec) == 48, "gradient layout");

struct SceneView {
  uint32_t width, height, has_clear;
  float clear[4];
  uint32_t nd;
  const uint32_t *vo, *po, *wo;
  const uint8_t* verbs;
  const float *pts, *wts;
  const PaintRec* paints;
  const GradRec* grads;
  const float *stop_colors, *stop_offsets;
  const float* clips;  // per draw (l, t, r, b) when the stream has the clip section
  const FilterRec* filters;  // per draw colour filter when the stream has that section
  // path clips (Canvas::ClipPath states), when the stream has that section
  struct ClipStateRec {
    uint32_t parent, op, fill_type, nv, np, nw;
    float translate[2], bounds[4];
  };
  uint32_t n_clip_states = 0;
  const ClipStateRec* clip_states = nullptr;
  const uint8_t* clip_verbs = nullptr;
  const float *clip_pts = nullptr, *clip_wts = nullptr;
  const uint32_t* draw_clip_state = nullptr;  // per draw, 1-based (0: none)
  const struct ClipStates* clip_cache = nullptr;  // the states' span lists (set per render)
  // images (header flag 8): records, pixel blob, per-draw image shaders
  struct ImageRec {
    uint32_t width, height, alpha_type, pad;
    uint64_t offset;
  };
  struct ImageShaderRec {
    uint32_t image, filter, tile_x, tile_y;
    float local[6];
    uint32_t rect, pad;
    float src[4], dst[4];
  };
  uint32_t n_images = 0;
  const ImageRec* images = nullptr;
  const uint8_t* image_pixels = nullptr;
  const ImageShaderRec* image_shaders = nullptr;
  // layers (header flag 16): Canvas::SaveLayer ... Restore, draws
  // [start, restore) inside (restore 0xFFFFFFFF: never restored)
  struct LayerRec {
    float bounds[4], translate[2], clip[4];
    uint32_t start, restore;
    float alpha;
    uint32_t blend, pad[2];
  };
  uint32_t n_layers = 0;
  const LayerRec* layers = nullptr;
  // per-draw canvas matrices (sx, kx, tx, ky, sy, ty), or null: the paints'
  // translations
  const float* matrices = nullptr;
  // per-clip-state canvas matrices, or null: the states' translations
  const float* clip_matrices = nullptr;
};

// The colour filter of the draw whose paint record is `p` (a record of s).
static const FilterRec* FilterOf(const SceneView& s, const PaintRec& p) {
  if (!s.filters) return nullptr;
  const size_t d = (size_t)(&p - s.paints);
  return d < s.nd && s.filters[d].type != 0 ? &s.filters[d] : nullptr;
}

static Clip ClipOf(const SceneView& s, uint32_t d) {
  Clip c;
  if (s.clips) {
    c.l = s.clips[4 * (size_t)d];
    c.t = s.clips[4 * (size_t)d + 1];
    c.r = s.clips[4 * (size_t)d + 2];
    c.b = s.clips[4 * (size_t)d + 3];
  }
  return c;
}

static bool ParseScene(const uint8_t* buf, size_t len, SceneView* s) {
  if (len < 72 || std::memcmp(buf, "SKSC", 4) != 0) return false;
  uint32_t hdr[7];
  std::memcpy(hdr, buf + 4, sizeof hdr);
  if (hdr[0] != 1) return false;
  s->width = hdr[1];
  s->height = hdr[2];
  s->has_clear = hdr[3];
  // 1: per-draw clip bounds, 2: per-draw colour filters, 4: path clips
  const uint32_t flags = hdr[4];
  if (flags & ~127u) return false;
  size_t o = 32;
  std::memcpy(s->clear, buf + o, 16);
  o += 16;
  uint32_t cnt[6];
  std::memcpy(cnt, buf + o, sizeof cnt);
  o += sizeof cnt;
  s->nd = cnt[0];
  auto at = [&](size_t bytes) {
    const uint8_t* p = buf + o;
    o += bytes;
    return p;
  };
  s->vo = (const uint32_t*)at(4 * (size_t)(s->nd + 1));
  s->po = (const uint32_t*)at(4 * (size_t)(s->nd + 1));
  s->wo = (const uint32_t*)at(4 * (size_t)(s->nd + 1));
  s->verbs = at(cnt[1]);
  o += (4 - cnt[1] % 4) % 4;
  s->pts = (const float*)at(8 * (size_t)cnt[2]);
  s->wts = (const float*)at(4 * (size_t)cnt[3]);
  s->paints = (const PaintRec*)at(sizeof(PaintRec) * s->nd);
  s->grads = (const GradRec*)at(sizeof(GradRec) * cnt[4]);
  s->stop_colors = (const float*)at(16 * (size_t)cnt[5]);
  s->stop_offsets = (const float*)at(4 * (size_t)cnt[5]);
  s->clips = (flags & 1) ? (const float*)at(16 * (size_t)s->nd) : nullptr;
  s->filters = (flags & 2) ? (const FilterRec*)at(sizeof(FilterRec) * s->nd) : nullptr;
  if (flags & 4) {
    if (o + 4 > len) return false;
    std::memcpy(&s->n_clip_states, buf + o, 4);
    o += 4;
    s->clip_states = (const SceneView::ClipStateRec*)at(sizeof(SceneView::ClipStateRec) *
                                                         (size_t)s->n_clip_states);
    if (o > len) return false;
    size_t tv = 0, tp = 0, tw = 0;
    for (uint32_t i = 0; i < s->n_clip_states; ++i) {
      tv += s->clip_states[i].nv;
      tp += s->clip_states[i].np;
      tw += s->clip_states[i].nw;
    }
    s->clip_verbs = at(tv);
    o += (4 - tv % 4) % 4;
    s->clip_pts = (const float*)at(8 * tp);
    s->clip_wts = (const float*)at(4 * tw);
    s->draw_clip_state = (const uint32_t*)at(4 * (size_t)s->nd);
  }
  if (flags & 8) {
    if (o + 4 > len) return false;
    std::memcpy(&s->n_images, buf + o, 4);
    o += 4;
    s->images = (const SceneView::ImageRec*)at(sizeof(SceneView::ImageRec) * (size_t)s->n_images);
    uint64_t nb = 0;
    if (o + 8 > len) return false;
    std::memcpy(&nb, buf + o, 8);
    o += 8;
    if (nb > len) return false;
    s->image_pixels = at(nb);
    o += (4 - nb % 4) % 4;
    s->image_shaders =
        (const SceneView::ImageShaderRec*)at(sizeof(SceneView::ImageShaderRec) * (size_t)s->nd);
  }
  if (flags & 16) {
    if (o + 4 > len) return false;
    std::memcpy(&s->n_layers, buf + o, 4);
    o += 4;
    s->layers = (const SceneView::LayerRec*)at(sizeof(SceneView::LayerRec) * (size_t)s->n_layers);
    if (o > len) return false;
    // one level: in start order, each restored before the next starts
    for (uint32_t i = 0; i < s->n_layers; ++i) {
      const SceneView::LayerRec& L = s->layers[i];
      const bool open = L.restore == 0xFFFFFFFFu;
      if (L.start > s->nd || (!open && (L.restore < L.start || L.restore > s->nd))) return false;
      if (i + 1 < s->n_layers && (open || s->layers[i + 1].start < L.restore)) return false;
    }
  }
  if (flags & 32) {
    s->matrices = (const float*)at(24 * (size_t)s->nd);
    for (uint32_t d = 0; d < s->nd && o <= len; ++d)
      if (s->paints[d].translate[0] != 0.f || s->paints[d].translate[1] != 0.f) return false;
  }
  if (flags & 64) s->clip_matrices = (const float*)at(24 * (size_t)s->n_clip_states);
  return o <= len;
}

// The canvas matrix of draw d as (sx, kx, tx, ky, sy, ty).
static void MatrixOf(const SceneView& s, uint32_t d, float m[6]) {
  if (s.matrices) {
    std::memcpy(m, s.matrices + 6 * (size_t)d, 24);
  } else {
    const float t[6] = {1.f, 0.f, s.paints[d].translate[0], 0.f, 1.f, s.paints[d].translate[1]};
    std::memcpy(m, t, 24);
  }
}
static bool IsTranslation(const float m[6]) {
  return m[0] == 1.f && m[1] == 0.f && m[3] == 0.f && m[4] == 1.f;
}

// Draws this restatement does not take under a canvas matrix that is more
// than a translation: layers, and shaders (a blur's filtered bitmap
// included) under a matrix with rotation or skew (their device_to_local
// needs the general 4x4 inverse).  The GPU path refuses the same draws.
static bool UnsupportedUnderMatrix(const SceneView& s) {
  if (!s.matrices) return false;
  for (uint32_t d = 0; d < s.nd; ++d) {
    const float* m = s.matrices + 6 * (size_t)d;
    const PaintRec& bp = s.paints[d];
    if (bp.blur_style != 0 && bp.blur_radius > 0.f && (m[1] != 0.f || m[3] != 0.f))
      return true;  // the blur's image draw under a rotation or skew
    if (IsTranslation(m)) continue;
    const PaintRec& p = s.paints[d];
    for (uint32_t i = 0; i < s.n_layers; ++i) {
      const uint32_t end = s.layers[i].restore == 0xFFFFFFFFu ? s.nd : s.layers[i].restore;
      if (d >= s.layers[i].start && d < end) return true;
    }
    const bool shaded = p.gradient >= 0 || (s.image_shaders && s.image_shaders[d].image);
    if (shaded && (m[1] != 0.f || m[3] != 0.f)) return true;
  }
  return false;
}

// A blurred or path-clipped draw inside a layer: not restated here (the GPU
// path refuses the same draws).
static bool BlurUnderClip(const SceneView& s) {
  for (uint32_t i = 0; i < s.n_layers; ++i) {
    const uint32_t end = s.layers[i].restore == 0xFFFFFFFFu ? s.nd : s.layers[i].restore;
    for (uint32_t d = s.layers[i].start; d < end; ++d)
      if ((s.paints[d].blur_style != 0 && s.paints[d].blur_radius > 0.f) ||
          (s.draw_clip_state && s.draw_clip_state[d] != 0))
        return true;
  }
  return false;
}

static Path BuildPath(const SceneView& s, uint32_t d) {
  Path path;
  const float* p = s.pts + 2 * (size_t)s.po[d];
  const float* w = s.wts + s.wo[d];
  for (uint32_t v = s.vo[d]; v < s.vo[d + 1]; ++v) {
    switch (s.verbs[v]) {
      case kMove: path.MoveTo(P{p[0], p[1]}); p += 2; break;
      case kLine: path.LineTo(P{p[0], p[1]}); p += 2; break;
      case kQuad: path.QuadTo(P{p[0], p[1]}, P{p[2], p[3]}); p += 4; break;
      case kConic: path.ConicTo(P{p[0], p[1]}, P{p[2], p[3]}, *w++); p += 4; break;
      case kCubic: path.CubicTo(P{p[0], p[1]}, P{p[2], p[3]}, P{p[4], p[5]}); p += 6; break;
      case kClose: path.Close(); break;
      default: break;
    }
  }
  return path;
}

// Stroke::StrokePath (stroke.cc:866-901); defined with the stroker below.
static void StrokePath(const Path& src, const PaintRec& paint, Path* dst);

struct Stats {
  uint64_t fragments = 0, spans = 0, edges = 0, tie_groups = 0;
};

// GenerateBrush (sw_canvas.cc:727-795) for the main canvas (identity CTM)
static Brush MakeBrush(const SceneView& s, const PaintRec& p, bool stroke) {
  Brush br;
  const size_t d = (size_t)(&p - s.paints);
  if (s.image_shaders && d < s.nd && s.image_shaders[d].image) {
    // GenerateBrush's pixmap branch (sw_canvas.cc:755-786): Scale(1/w, 1/h)
    // * inverse(local); the canvas translation is applied by the caller
    const SceneView::ImageShaderRec& r = s.image_shaders[d];
    const SceneView::ImageRec& im = s.images[r.image - 1];
    Mat inv = Mat::Identity();  // Matrix::InvertNonIdentity, scale + translate
    if (r.local[0] != 1.f || r.local[4] != 1.f) {
      float ix = 1.f / r.local[0], iy = 1.f / r.local[4];
      inv.e[0][0] = ix;
      inv.e[1][1] = iy;
      inv.e[3][0] = -r.local[2] * ix;
      inv.e[3][1] = -r.local[5] * iy;
    } else {
      inv.e[3][0] = -r.local[2];
      inv.e[3][1] = -r.local[5];
    }
    br.kind = 5;
    br.m = MatMul(MatScale(1.f / (float)im.width, 1.f / (float)im.height), inv);
    br.img.px = s.image_pixels + im.offset;
    br.img.w = im.width;
    br.img.h = im.height;
    br.img.filter = (int)r.filter;
    br.img.tile_x = (int)r.tile_x;
    br.img.tile_y = (int)r.tile_y;
    br.img.unpremul = im.alpha_type == 3;
    // SWSpanBrush's global alpha from Paint::GetAlphaF (paint.cc:96-98)
    br.global_alpha = (uint8_t)(255 * (p.style == 1 ? p.stroke_color[3] : p.fill_color[3]));
    br.filter = FilterOf(s, p);
    return br;
  }
  if (p.gradient >= 0) {
    const GradRec& g = s.grads[p.gradient];
    br.kind = (int)g.type;
    br.g.type = (int)g.type;
    br.g.tile = (int)g.tile_mode;
    br.g.count = (int)g.stop_count;
    br.g.has_offsets = g.has_offsets != 0;
    br.g.colors = s.stop_colors + 4 * (size_t)g.stop_start;
    br.g.offsets = s.stop_offsets + g.stop_start;
    std::memcpy(br.g.p0, g.p0, 8);
    std::memcpy(br.g.p1, g.p1, 8);
    std::memcpy(br.g.radius, g.radius, 8);
    br.m = PointsToUnit(br.g);
    if (br.kind == 4) br.con = ConicalPreBrush(br.g);
    br.filter = FilterOf(s, p);
    return br;
  }
  br.kind = 0;
  br.solid = ColorToPMColor(Color4fToColor(stroke ? p.stroke_color : p.fill_color));
  br.filter = FilterOf(s, p);
  return br;
}

// ---------------------------------------------------------------------------
// Path clips: SWCanvas::State's span algebra (sw_canvas.cc:42-265) and
// OnClipPath (:317-336)
// ---------------------------------------------------------------------------
// FindSpan (:218-262): the pieces of `s` under each clip span of its row,
// in clip-list order, covers min'd.
static void FindSubSpans(const Span& s, const std::vector<Span>& clip, std::vector<Span>* out) {
  for (const Span& c : clip) {
    if (c.y != s.y) continue;
    const int32_t cover = std::min(c.cover, s.cover);
    if (c.x < s.x) {
      if (c.x + c.len < s.x) continue;
      out->push_back(Span{s.x, s.y, std::min(c.x + c.len, s.x + s.len) - s.x, cover});
    } else if (c.x == s.x) {
      out->push_back(Span{s.x, s.y, std::min(s.len, c.len), cover});
    } else {
      if (s.x + s.len < c.x) continue;
      // the reference's + 1: the piece reaches one pixel past the span
      out->push_back(Span{c.x, s.y, std::min(s.x + s.len - c.x + 1, c.len), cover});
    }
  }
}

// spans_subtraction (:59-133): each span of `a` minus the spans of `b` on
// its row (those sorted by x with std::sort), pieces in x order.
static std::vector<Span> SubtractSpans(const std::vector<Span>& a, const std::vector<Span>& b) {
  std::vector<Span> out;
  for (const Span& sp : a) {
    std::vector<Span> ms;
    for (const Span& m : b)
      if (m.y == sp.y) ms.push_back(m);
    if (ms.empty()) {
      out.push_back(sp);
      continue;
    }
    std::sort(ms.begin(), ms.end(), [](const Span& p, const Span& q) { return p.x < q.x; });
    int32_t x = sp.x, len = sp.len;
    for (const Span& m : ms) {
      if (m.x + m.len < x || m.x > x + len) continue;
      if (m.x < x) {
        if (m.x + m.len > x + len) {  // all of it is subtracted
          len = 0;
          break;
        }
        const int32_t end = x + len, piece = m.x + m.len - x;
        if (piece == 0) continue;
        out.push_back(Span{x, sp.y, piece, sp.cover});
        x += piece;
        len = end - x;
      } else if (m.x + m.len < x + len) {
        const int32_t end = x + len;
        out.push_back(Span{x, sp.y, m.x - x, sp.cover});
        x = m.x + m.len;
        len = end - x;
      } else {
        out.push_back(Span{x, sp.y, m.x - x, sp.cover});
        len = 0;
      }
      if (len <= 0) break;
    }
    if (len > 0) out.push_back(Span{x, sp.y, len, sp.cover});
  }
  return out;
}

struct ClipState {  // SWCanvas::State: the clip's spans and op
  std::vector<Span> spans;
  uint32_t op = 1;  // Canvas::ClipOp: 0 kDifference, 1 kIntersect
  bool HasClip() const { return !spans.empty(); }
};

// State::PerformClip (:157-175)
static std::vector<Span> PerformClipOf(const ClipState& st, const std::vector<Span>& spans) {
  if (st.op == 0) return SubtractSpans(spans, st.spans);
  std::vector<Span> out;
  for (const Span& sp : spans) FindSubSpans(sp, st.spans, &out);
  return out;
}

// State::RecursiveClip (:177-193) and PerformMerge (:195-216)
static std::vector<Span> RecursiveClipOf(const ClipState& st, const std::vector<Span>& spans,
                                         uint32_t op) {
  if (st.op == op) {
    if (op == 1) return PerformClipOf(st, spans);
    std::vector<Span> all(spans);
    all.insert(all.end(), st.spans.begin(), st.spans.end());
    std::sort(all.begin(), all.end(), [](const Span& a, const Span& b) {
      if (a.y != b.y) return a.y < b.y;
      if (a.x != b.x) return a.x < b.x;
      return a.cover > b.cover;
    });
    return all;
  }
  return st.op == 0 ? SubtractSpans(spans, st.spans) : SubtractSpans(st.spans, spans);
}

struct ClipStates {
  std::vector<ClipState> states;  // index 0: no clip; k: after the k-th ClipPath
};

static Path BuildPathFrom(const uint8_t* verbs, uint32_t nv, const float* p, const float* w) {
  Path path;
  for (uint32_t v = 0; v < nv; ++v) {
    switch (verbs[v]) {
      case kMove: path.MoveTo(P{p[0], p[1]}); p += 2; break;
      case kLine: path.LineTo(P{p[0], p[1]}); p += 2; break;
      case kQuad: path.QuadTo(P{p[0], p[1]}, P{p[2], p[3]}); p += 4; break;
      case kConic: path.ConicTo(P{p[0], p[1]}, P{p[2], p[3]}, *w++); p += 4; break;
      case kCubic: path.CubicTo(P{p[0], p[1]}, P{p[2], p[3]}, P{p[4], p[5]}); p += 6; break;
      case kClose: path.Close(); break;
      default: break;
    }
  }
  return path;
}

// OnClipPath for every state of the stream, in order (a parent comes first).
static void ComputeClipStates(const SceneView& s, ClipStates* cs) {
  cs->states.assign(1, ClipState{});
  const uint8_t* v = s.clip_verbs;
  const float* p = s.clip_pts;
  const float* w = s.clip_wts;
  for (uint32_t i = 0; i < s.n_clip_states; ++i) {
    const SceneView::ClipStateRec& r = s.clip_states[i];
    Path path = BuildPathFrom(v, r.nv, p, w);
    v += r.nv;
    p += 2 * (size_t)r.np;
    w += r.nw;
    // RastePath(path, CurrentTransform(), GetScanClipBounds()); the points
    // mapped as CopyWithMatrix maps them (see DrawPathMatrix)
    const float* cm = s.clip_matrices ? s.clip_matrices + 6 * (size_t)i : nullptr;
    const float m[6] = {cm ? cm[0] : 1.f, cm ? cm[1] : 0.f, cm ? cm[2] : r.translate[0],
                        cm ? cm[3] : 0.f, cm ? cm[4] : 1.f, cm ? cm[5] : r.translate[1]};
    Path quad;
    QuadPath(path, &quad);
    for (auto& q : quad.pts) {
      const float x = q.x, y = q.y;
      q.x = (m[0] * x + m[1] * y) + (0.f * 0.f + m[2] * 1.f);
      q.y = (m[3] * x + m[4] * y) + (0.f * 0.f + m[5] * 1.f);
    }
    Clip bounds;
    bounds.l = r.bounds[0];
    bounds.t = r.bounds[1];
    bounds.r = r.bounds[2];
    bounds.b = r.bounds[3];
    std::vector<Span> raster;
    RastePathQuads(quad, r.fill_type == 1, &raster, nullptr, bounds);
    ClipState st = r.parent <= i ? cs->states[r.parent] : ClipState{};
    if (st.HasClip()) {
      st.spans = RecursiveClipOf(st, raster, r.op);
      if (st.op != r.op) st.op = 1;
    } else {
      st.spans = raster;
      st.op = r.op;
    }
    cs->states.push_back(std::move(st));
  }
}

// DoBrush's clip step (sw_canvas.cc:338-353): the spans a draw brushes;
// false when the clip leaves none.
static bool ClipDrawSpans(const SceneView& s, uint32_t d, std::vector<Span>* spans) {
  if (!s.draw_clip_state || !s.clip_cache) return true;
  const uint32_t k = s.draw_clip_state[d];
  if (k == 0 || k >= s.clip_cache->states.size()) return true;
  const ClipState& st = s.clip_cache->states[k];
  if (!st.HasClip()) return true;
  *spans = PerformClipOf(st, *spans);
  return !spans->empty();
}

// SWCanvas::OnDrawPath (sw_canvas.cc:357-411) for draws without filters
static void DrawPath(const SceneView& s, uint32_t d, Target* t, Stats* st,
                     std::vector<Span>* spans) {
  const PaintRec& paint = s.paints[d];
  Path path = BuildPath(s, d);
  bool even_odd = paint.fill_type == 1;
  bool need_fill = paint.style != 1;
  bool need_stroke = paint.style != 0;
  RasterStats rs;
  const Clip clip = ClipOf(s, d);
  auto draw_fill = [&]() {
    Path quad;
    QuadPath(path, &quad);
    RastePathQuads(quad, even_odd, spans, &rs, clip);
    if (!ClipDrawSpans(s, d, spans)) return;
    Brush br = MakeBrush(s, paint, false);
    st->fragments += BrushSpans(*spans, br, (int)paint.blend, t);
    st->spans += spans->size();
  };
  auto draw_stroke = [&]() {
    Path quad, outline, quad2;
    QuadPath(path, &quad);
    StrokePath(quad, paint, &outline);
    QuadPath(outline, &quad2);
    // RastePath reads the fill type of the path it is given: the stroke
    // outline is a fresh Path (kWinding), whatever the source's fill type
    // (sw_canvas.cc:388-407, sw_raster.cc:783-784)
    RastePathQuads(quad2, false, spans, &rs, clip);
    if (!ClipDrawSpans(s, d, spans)) return;
    Brush br = MakeBrush(s, paint, true);
    st->fragments += BrushSpans(*spans, br, (int)paint.blend, t);
    st->spans += spans->size();
  };
  if (paint.style == 3) {  // kStrokeThenFill (paint_order.hpp:12-31)
    if (need_stroke) draw_stroke();
    if (need_fill) draw_fill();
  } else {
    if (need_fill) draw_fill();
    if (need_stroke) draw_stroke();
  }
  st->edges += rs.edges;
  st->tie_groups += rs.tie_groups;
}

}  // namespace sko

// ---------------------------------------------------------------------------
// Stroker and conics live in their own translation unit section below.
// ---------------------------------------------------------------------------
#include "sw_oracle_stroke.inc"

// ---------------------------------------------------------------------------
// C ABI for the tests and the CPU baseline
// ---------------------------------------------------------------------------
extern "C" {

// BitmapSampler::GetColor (+ the pixmap brush's premultiply) of one RGBA8
// pixmap at unit coordinates (u, v): the checker of the sampler's own tests.
uint32_t sko_sample(const uint8_t* rgba, uint32_t w, uint32_t h, uint32_t alpha_type,
                    uint32_t filter, uint32_t tile_x, uint32_t tile_y, float u, float v) {
  sko::Sampler sm;
  sm.px = rgba;
  sm.w = w;
  sm.h = h;
  sm.filter = (int)filter;
  sm.tile_x = (int)tile_x;
  sm.tile_y = (int)tile_y;
  sm.unpremul = alpha_type == 3;
  return sm.Color(u, v);
}

int sko_render(const uint8_t* scene, size_t len, uint32_t first, uint32_t count,
               uint8_t* out_rgba, sko_stats* stats) {
  using namespace sko;
  SceneView s;
  if (!ParseScene(scene, len, &s)) return -2;
  if (BlurUnderClip(s)) return -3;
  if (UnsupportedUnderMatrix(s)) return -4;
  ClipStates clip_states;
  ComputeClipStates(s, &clip_states);
  s.clip_cache = &clip_states;
  Target t{out_rgba, (int)s.width, (int)s.height};
  auto t0 = std::chrono::steady_clock::now();
  if (s.has_clear) {
    // Canvas::Clear -> DrawColor(kSrc) -> OnDrawPaint: full-canvas rect of
    // coverage 255 blended with kSrc (sw_canvas.cc:413-439)
    uint32_t c = ColorToPMColor(Color4fToColor(s.clear));
    for (int y = 0; y < t.h; ++y)
      for (int x = 0; x < t.w; ++x) t.Set(x, y, c);
  } else {
    std::memset(out_rgba, 0, (size_t)t.w * t.h * 4);
  }
  Stats st;
  uint32_t last = std::min<uint32_t>(s.nd, first + count);
  ReplayDraws(s, first, last, &t, &st);
  auto t1 = std::chrono::steady_clock::now();
  if (stats) {
    stats->fragments = st.fragments;
    stats->spans = st.spans;
    stats->edges = st.edges;
    stats->tie_groups = st.tie_groups;
    stats->seconds = std::chrono::duration<double>(t1 - t0).count();
    stats->draws = last > first ? last - first : 0;
  }
  return 0;
}

// Banded replay on `threads` host threads: every thread rasterises every
// draw (the sweep is sequential per path) but blends only the spans of its
// own band of rows.  Blending is per pixel and in draw order, so the result
// equals the single-threaded replay; the brush work splits across threads.
int sko_render_mt(const uint8_t* scene, size_t len, uint32_t first, uint32_t count,
                  uint8_t* out_rgba, uint32_t threads, sko_stats* stats) {
  using namespace sko;
  SceneView s;
  if (!ParseScene(scene, len, &s)) return -2;
  if (BlurUnderClip(s)) return -3;
  if (UnsupportedUnderMatrix(s)) return -4;
  ClipStates clip_states;
  ComputeClipStates(s, &clip_states);
  s.clip_cache = &clip_states;
  if (threads == 0) threads = 1;
  auto t0 = std::chrono::steady_clock::now();
  uint32_t last = std::min<uint32_t>(s.nd, first + count);
  std::vector<Stats> st(threads);
  std::vector<std::thread> pool;
  int h = (int)s.height;
  for (uint32_t k = 0; k < threads; ++k) {
    pool.emplace_back([&, k]() {
      Target t{out_rgba, (int)s.width, (int)s.height};
      t.band0 = (int)((int64_t)h * k / threads);
      t.band1 = (int)((int64_t)h * (k + 1) / threads);
      uint32_t c = s.has_clear ? ColorToPMColor(Color4fToColor(s.clear)) : 0;
      for (int y = t.band0; y < t.band1; ++y)
        for (int x = 0; x < t.w; ++x) t.Set(x, y, c);
      ReplayDraws(s, first, last, &t, &st[k]);
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    for (auto& x : st) stats->fragments += x.fragments;
    stats->spans = st[0].spans;
    stats->edges = st[0].edges;
    stats->tie_groups = st[0].tie_groups;
    stats->seconds = std::chrono::duration<double>(t1 - t0).count();
    stats->draws = last > first ? last - first : 0;
  }
  return 0;
}

int sko_cubic_quad_count(const float pts[8]) {
  sko::P c[4] = {{pts[0], pts[1]}, {pts[2], pts[3]}, {pts[4], pts[5]}, {pts[6], pts[7]}};
  return sko::CubicQuadCount(c);
}

int sko_quad_edge(const float pts[6], int32_t out[4]) {
  sko::P q[3] = {{pts[0], pts[1]}, {pts[2], pts[3]}, {pts[4], pts[5]}};
  sko::Edge e{};
  // curve_count is consumed by the first UpdateQuad; report the shift instead
  if (!sko::SetQuad(&e, q)) return 0;
  out[0] = e.curve_shift + 1;
  out[1] = e.winding;
  out[2] = e.q_first_y;
  out[3] = e.q_last_y;
  return 1;
}

int sko_fill_quads(const uint8_t* scene, size_t len, uint32_t draw, uint8_t* verbs,
                   uint32_t vcap, float* pts, uint32_t pcap, uint32_t counts[2]) {
  using namespace sko;
  SceneView s;
  if (!ParseScene(scene, len, &s) || draw >= s.nd) return -2;
  Path path = BuildPath(s, draw);
  Path quad;
  QuadPath(path, &quad);
  // mapped by the draw's canvas matrix, as RastePath's CopyWithMatrix maps them
  float m[6];
  MatrixOf(s, draw, m);
  for (auto& q : quad.pts) {
    const float x = q.x, y = q.y;
    q.x = (m[0] * x + m[1] * y) + (0.f * 0.f + m[2] * 1.f);
    q.y = (m[3] * x + m[4] * y) + (0.f * 0.f + m[5] * 1.f);
  }
  counts[0] = (uint32_t)quad.verbs.size();
  counts[1] = (uint32_t)quad.pts.size();
  for (uint32_t i = 0; i < counts[0] && i < vcap; ++i) verbs[i] = (uint8_t)quad.verbs[i];
  for (uint32_t i = 0; i < counts[1] && i < pcap; ++i) {
    pts[2 * i] = quad.pts[i].x;
    pts[2 * i + 1] = quad.pts[i].y;
  }
  return 0;
}

int sko_path_spans(const uint8_t* scene, size_t len, uint32_t draw, int32_t* out,
                   uint32_t cap) {
  using namespace sko;
  SceneView s;
  if (!ParseScene(scene, len, &s) || draw >= s.nd) return -2;
  Path path = BuildPath(s, draw);
  Path quad;
  QuadPath(path, &quad);
  std::vector<Span> spans;
  RastePathQuads(quad, s.paints[draw].fill_type == 1, &spans, nullptr, ClipOf(s, draw));
  uint32_t n = (uint32_t)spans.size();
  for (uint32_t i = 0; i < n && i < cap; ++i) {
    out[4 * i] = spans[i].x;
    out[4 * i + 1] = spans[i].y;
    out[4 * i + 2] = spans[i].len;
    out[4 * i + 3] = spans[i].cover;
  }
  return (int)n;
}

}  // extern "C"
