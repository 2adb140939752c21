// Geometry of the raster path for one draw, written for one GPU thread:
// Path iteration, Stroke::QuadPath (cubic -> quads, conic -> 2 quads), the
// path stroker, fixed-point edge building and the edge sort.
//
// Every function restates the reference software backend's function of the
// same role (file:line cited), with the same float operation order; the
// translation unit is compiled with -fmad=false so no FMA contraction
// changes a rounding.  The code is host+device (SKC_HD) so tests can run it
// on the CPU against std::sort and the oracle.
#pragma once
#include <stdint.h>
#include <vector_types.h>  // float4 / uint2 on host builds too

// branch hints: SKC_COLD(c) for conditions that are rarely true on the hot
// path (keeps their blocks out of the straight-line code), SKC_LIKELY(c)
#define SKC_COLD(c) __builtin_expect(!!(c), 0)
#define SKC_LIKELY(c) __builtin_expect(!!(c), 1)

#ifdef __CUDACC__
#define SKC_HD __host__ __device__ __forceinline__
#define SKC_HDN inline __host__ __device__ __noinline__
#else
#include <cmath>
#define SKC_HD inline
#define SKC_HDN inline
#endif

namespace skc {

// ---------------------------------------------------------------------------
// math shims (same IEEE operations on host and device)
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
SKC_HD float fabs_(float x) { return fabsf(x); }
SKC_HD float sqrt_(float x) { return sqrtf(x); }
SKC_HD double sqrtd_(double x) { return sqrt(x); }
SKC_HD double atan2d_(double y, double x) { return atan2(y, x); }
SKC_HD float floor_(float x) { return floorf(x); }
SKC_HD float ceil_(float x) { return ceilf(x); }
SKC_HD double ceild_(double x) { return ceil(x); }
SKC_HD double pow_(double a, double b) { return pow(a, b); }
SKC_HD bool isfinite_(float x) { return isfinite(x); }
SKC_HD bool isinf_(float x) { return isinf(x); }
SKC_HD bool isnan_(float x) { return isnan(x); }
SKC_HD float round_(float x) { return roundf(x); }
#else
SKC_HD float fabs_(float x) { return std::fabs(x); }
SKC_HD float sqrt_(float x) { return std::sqrt(x); }
SKC_HD double sqrtd_(double x) { return std::sqrt(x); }
SKC_HD double atan2d_(double y, double x) { return std::atan2(y, x); }
SKC_HD float floor_(float x) { return std::floor(x); }
SKC_HD float ceil_(float x) { return std::ceil(x); }
SKC_HD double ceild_(double x) { return std::ceil(x); }
SKC_HD double pow_(double a, double b) { return std::pow(a, b); }
SKC_HD bool isfinite_(float x) { return std::isfinite(x); }
SKC_HD bool isinf_(float x) { return std::isinf(x); }
SKC_HD bool isnan_(float x) { return std::isnan(x); }
SKC_HD float round_(float x) { return std::round(x); }
#endif
template <typename T>
SKC_HD T min_(T a, T b) { return b < a ? b : a; }
template <typename T>
SKC_HD T max_(T a, T b) { return a < b ? b : a; }
template <typename T>
SKC_HD void swap_(T& a, T& b) { T t = a; a = b; b = t; }
SKC_HD int32_t iabs_(int32_t v) { return v < 0 ? -v : v; }
SKC_HD int clz_(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __clz((int)x);
#else
  return x ? __builtin_clz(x) : 32;
#endif
}

// ---------------------------------------------------------------------------
// fixed point (src/render/sw/sw_subpixel.hpp:18-97)
// ---------------------------------------------------------------------------
typedef int32_t Fixed;
typedef int32_t FDot6;
constexpr Fixed kFixed1 = 1 << 16;
constexpr Fixed kFixedHalf = 1 << 15;
constexpr int32_t kMaxS32 = 2147483647;
constexpr int32_t kMinS32 = -2147483647;
constexpr int32_t kNaN32 = (int32_t)0x80000000u;
constexpr int kAccuracy = 2;

SKC_HD int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
SKC_HD int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
SKC_HD int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
SKC_HD Fixed FixedMul(Fixed a, Fixed b) { return (Fixed)(((int64_t)a * b) >> 16); }
SKC_HD Fixed FDot6ToFixed(FDot6 x) { return (Fixed)((uint32_t)x << 10); }
SKC_HD int32_t LShift(int32_t v, int s) { return (int32_t)((uint32_t)v << s); }
SKC_HD Fixed FDot6ToFixedDiv2(FDot6 v) { return LShift(v, 16 - 6 - 1); }
// (numer << 16) / denom in 64 bits, truncated toward zero, clamped to
// [kMinS32, kMaxS32] (the reference's SkFixed-style FixedDiv).
SKC_HD Fixed FixedDivWide(int32_t numer, int32_t denom) {
  int64_t q = (int64_t)((uint64_t)(int64_t)numer << 16) / denom;
  if (q < kMinS32) q = kMinS32;
  if (q > kMaxS32) q = kMaxS32;
  return (Fixed)q;
}
// The same quotient without a 64-bit division (which the GPU runs as a long
// called routine): for |denom| < 2^24, floor(|numer| 2^16 / |denom|) is
// built from three 32-bit divisions giving 16 + 8 + 8 quotient bits
// (a = q1 b + r1, 2^8 r1 = q2 b + r2, 2^8 r2 = q3 b + r3, so the quotient
// is q1 2^16 + q2 2^8 + q3 and every partial dividend stays below 2^32),
// then signed as C's division truncates; larger divisors take the 64-bit
// path.  Equal to FixedDivWide for every input with denom != 0.
SKC_HD Fixed FixedDiv(int32_t numer, int32_t denom) {
  const uint32_t a = numer < 0 ? 0u - (uint32_t)numer : (uint32_t)numer;
  const uint32_t b = denom < 0 ? 0u - (uint32_t)denom : (uint32_t)denom;
  if (b >= (1u << 24)) return FixedDivWide(numer, denom);
  const uint32_t q1 = a / b, r1 = a - q1 * b;
  const uint32_t t2 = r1 << 8, q2 = t2 / b, r2 = t2 - q2 * b;
  const uint32_t q3 = (r2 << 8) / b;
  const uint64_t u = ((uint64_t)q1 << 16) + ((uint64_t)q2 << 8) + q3;
  int64_t q = ((numer < 0) != (denom < 0)) ? -(int64_t)u : (int64_t)u;
  if (q < kMinS32) q = kMinS32;
  if (q > kMaxS32) q = kMaxS32;
  return (Fixed)q;
}
SKC_HD int FDot6Round(FDot6 x) { return (x + 32) >> 6; }
SKC_HD FDot6 ScalarToFDot6(float x) { return (FDot6)(x * 64); }
SKC_HD FDot6 FixedToFDot6(Fixed x) { return x >> 10; }
SKC_HD Fixed FixedRoundToFixed(Fixed x) { return (Fixed)((uint32_t)(x + kFixedHalf) & 0xFFFF0000u); }
SKC_HD Fixed FixedCeilToFixed(Fixed x) { return (Fixed)((uint32_t)(x + kFixed1 - 1) & 0xFFFF0000u); }
SKC_HD Fixed FixedFloorToFixed(Fixed x) { return (Fixed)((uint32_t)x & 0xFFFF0000u); }
SKC_HD Fixed IntToFixed(int n) { return (Fixed)((uint32_t)n << 16); }
SKC_HD int FixedRoundToInt(Fixed x) { return (x + kFixedHalf) >> 16; }
SKC_HD int FixedCeilToInt(Fixed x) { return (x + kFixed1 - 1) >> 16; }
SKC_HD int FixedFloorToInt(Fixed x) { return x >> 16; }

struct P {
  float x, y;
};
SKC_HD P mkP(float x, float y) { P p; p.x = x; p.y = y; return p; }
SKC_HD bool PEq(P a, P b) { return a.x == b.x && a.y == b.y; }

enum : uint8_t { kMove = 0, kLine = 1, kQuad = 2, kConic = 3, kCubic = 4, kClose = 5, kDone = 6 };

// ---------------------------------------------------------------------------
// Read-only path view and a path builder over caller memory
// (src/graphic/path.cc:494-569, 837-860, 1042-1080, 1327-1339)
// ---------------------------------------------------------------------------
struct PathView {
  const uint8_t* verbs;
  const P* pts;
  const float* w;
  int nv, np, nw;
};

// DPath: skity::Path builder semantics over fixed buffers.  With cap_* = 0
// it only counts (the count pass); counts are always exact, values are
// stored while they fit.  Per-verb-type counts since the last MoveTo let a
// count-only path still size Path::ReversePathTo.
struct DPath {
  uint8_t* verbs;
  P* pts;
  float* w;
  int nv, np, nw;
  int cap_v, cap_p, cap_w;
  int last_move;
  uint8_t last_verb;  // kDone when empty
  int c_line, c_quad, c_conic, c_cubic;  // since the last MoveTo
  P last_pt;

  SKC_HD void init(uint8_t* v, int cv, P* p, int cp, float* ww, int cw) {
    verbs = v; pts = p; w = ww;
    cap_v = cv; cap_p = cp; cap_w = cw;
    reset();
  }
  SKC_HD void reset() {
    nv = np = nw = 0;
    last_move = ~0;
    last_verb = kDone;
    c_line = c_quad = c_conic = c_cubic = 0;
    last_pt = mkP(0, 0);
  }
  SKC_HD bool overflow() const { return nv > cap_v || np > cap_p || nw > cap_w; }
  SKC_HD PathView view() const {
    PathView v;
    v.verbs = verbs; v.pts = pts; v.w = w; v.nv = nv; v.np = np; v.nw = nw;
    return v;
  }
  SKC_HD void pushv(uint8_t v) {
    if (nv < cap_v) verbs[nv] = v;
    nv++;
    last_verb = v;
  }
  SKC_HD void pushp(P p) {
    if (np < cap_p) pts[np] = p;
    np++;
    last_pt = p;
  }
  SKC_HD void pushw(float x) {
    if (nw < cap_w) w[nw] = x;
    nw++;
  }
  SKC_HD P pt_at(int i) const { return (i >= 0 && i < np && i < cap_p) ? pts[i] : mkP(0, 0); }
  SKC_HD void MoveTo(P p) {
    if (nv > 0 && last_verb == kMove) {
      if (np - 1 < cap_p) pts[np - 1] = p;
      last_pt = p;
    } else {
      last_move = np;
      pushv(kMove);
      pushp(p);
    }
    c_line = c_quad = c_conic = c_cubic = 0;
  }
  SKC_HD void Inject() {
    if (last_move < 0) {
      P p = nv == 0 ? mkP(0, 0) : pt_at(~last_move);
      MoveTo(p);
    }
  }
  SKC_HD void LineTo(P p) {
    Inject();
    pushv(kLine);
    pushp(p);
    c_line++;
  }
  SKC_HD void QuadTo(P a, P b) {
    Inject();
    pushv(kQuad);
    pushp(a);
    pushp(b);
    c_quad++;
  }
  SKC_HD void ConicTo(P a, P b, float weight) {  // path.cc:533-555
    if (!(weight > 0)) {
      LineTo(b);
    } else if (isinf_(weight)) {
      LineTo(a);
      LineTo(b);
    } else if (weight == 1.0f) {
      QuadTo(a, b);
    } else {
      Inject();
      pushv(kConic);
      pushw(weight);
      pushp(a);
      pushp(b);
      c_conic++;
    }
  }
  SKC_HD void CubicTo(P a, P b, P c) {
    Inject();
    pushv(kCubic);
    pushp(a);
    pushp(b);
    pushp(c);
    c_cubic++;
  }
  SKC_HD void Close() {
    if (nv > 0 && last_verb != kClose) pushv(kClose);
    last_move ^= (~last_move >> 31);
  }
  SKC_HD P LastPt() const { return np > 0 ? last_pt : mkP(0, 0); }
};

// Path::Iter with forceClose = false (path.cc:234-397)
struct PathIter {
  PathView path;
  int v, p, wi;
  P move_to, last_pt;
  int seg_state;  // 0 empty contour, 1 after move, 2 after primitive
  float weight;
  SKC_HD void init(const PathView& src) {
    path = src;
    v = p = wi = 0;
    move_to = last_pt = mkP(0, 0);
    seg_state = 0;
    weight = 0;
  }
  SKC_HD P ConsMoveTo() {
    if (seg_state == 1) {
      seg_state = 2;
      return move_to;
    }
    return path.pts[p - 1];
  }
  SKC_HD uint8_t AutoClose(P* out) {  // path.cc:372-388
    if (!PEq(last_pt, move_to)) {
      if (isnan_(last_pt.x) || isnan_(last_pt.y) || isnan_(move_to.x) || isnan_(move_to.y))
        return kClose;
      out[0] = last_pt;
      out[1] = move_to;
      last_pt = move_to;
      return kLine;
    }
    out[0] = move_to;
    return kClose;
  }
  SKC_HD uint8_t Next(P out[4]) {
    if (v == path.nv) return kDone;
    uint8_t verb = path.verbs[v++];
    switch (verb) {
      case kMove:
        if (v == path.nv) return kDone;
        move_to = path.pts[p];
        out[0] = move_to;
        p += 1;
        seg_state = 1;
        last_pt = move_to;
        break;
      case kLine:
        out[0] = ConsMoveTo();
        out[1] = path.pts[p];
        last_pt = out[1];
        p += 1;
        break;
      case kConic:
        weight = path.w[wi++];
        out[0] = ConsMoveTo();
        out[1] = path.pts[p];
        out[2] = path.pts[p + 1];
        last_pt = out[2];
        p += 2;
        break;
      case kQuad:
        out[0] = ConsMoveTo();
        out[1] = path.pts[p];
        out[2] = path.pts[p + 1];
        last_pt = out[2];
        p += 2;
        break;
      case kCubic:
        out[0] = ConsMoveTo();
        out[1] = path.pts[p];
        out[2] = path.pts[p + 1];
        out[3] = path.pts[p + 2];
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
      default:
        return kDone;
    }
    return verb;
  }
};

// ---------------------------------------------------------------------------
// curves (src/geometry/geometry.cc:39-190, cubic.cc:29-61, conic.cc:18-59,168-197)
// ---------------------------------------------------------------------------
struct QuadCoeff {
  P A, B, C;
  SKC_HD void set(P p0, P p1, P p2) {
    C = p0;
    P d = mkP(p1.x - C.x, p1.y - C.y);
    B = mkP(d.x + d.x, d.y + d.y);
    P t2 = mkP(p1.x + p1.x, p1.y + p1.y);
    A = mkP((p2.x - t2.x) + C.x, (p2.y - t2.y) + C.y);
  }
  SKC_HD P eval(float t) const {
    return mkP((A.x * t + B.x) * t + C.x, (A.y * t + B.y) * t + C.y);
  }
};

struct CubicCoeff {
  P A, B, C, D;
  SKC_HD void set(P p0, P p1, P p2, P p3) {
    A = mkP((p3.x + 3.f * (p1.x - p2.x)) - p0.x, (p3.y + 3.f * (p1.y - p2.y)) - p0.y);
    P t = mkP(p1.x + p1.x, p1.y + p1.y);
    B = mkP(3.f * ((p2.x - t.x) + p0.x), 3.f * ((p2.y - t.y) + p0.y));
    C = mkP(3.f * (p1.x - p0.x), 3.f * (p1.y - p0.y));
    D = p0;
  }
  SKC_HD P eval(float t) const {
    return mkP(((A.x * t + B.x) * t + C.x) * t + D.x, ((A.y * t + B.y) * t + C.y) * t + D.y);
  }
};

// Cubic::ToQuads count (cubic.cc:29-38)
SKC_HD double CubicQuadCountD(const P c[4]) {
  float accuracy = 0.1f;
  double max_hypot2 = 432.0 * accuracy * accuracy;
  P p1x2 = mkP(c[1].x * 3.f - c[0].x, c[1].y * 3.f - c[0].y);
  P p2x2 = mkP(c[2].x * 3.f - c[3].x, c[2].y * 3.f - c[3].y);
  P d = mkP(p2x2.x - p1x2.x, p2x2.y - p1x2.y);
  float err = d.x * d.x + d.y * d.y;
  return max_(1., ceild_(pow_(err / max_hypot2, 1. / 6.0)));
}

// Cubic::ToQuads, quad i of quad_count (cubic.cc:42-61)
SKC_HD void CubicQuadAt(const P c[4], const CubicCoeff& cc, const QuadCoeff& qc,
                        double quad_count, int i, P out[3]) {
  double t0d = i / quad_count;
  double t1d = (i + 1) / quad_count;
  float t1 = (float)t0d, t2 = (float)t1d;
  P s0 = cc.eval(t1);
  P s3 = cc.eval(t2);
  float scale = (t2 - t1) * (1.f / 3.f);
  P q1 = qc.eval(t1), q2 = qc.eval(t2);
  P s1 = mkP(s0.x + q1.x * scale, s0.y + q1.y * scale);
  P s2 = mkP(s3.x - q2.x * scale, s3.y - q2.y * scale);
  P a = mkP(s1.x * 3.f - s0.x, s1.y * 3.f - s0.y);
  P b = mkP(s2.x * 3.f - s3.x, s2.y * 3.f - s3.y);
  out[0] = s0;
  out[1] = mkP((a.x + b.x) / 4.f, (a.y + b.y) / 4.f);
  out[2] = s3;
}

SKC_HD int valid_unit_divide(float number, float denom, float* ratio) {  // geometry.hpp:102-125
  if (number < 0) {
    number = -number;
    denom = -denom;
  }
  if (denom == 0 || number == 0 || number >= denom) return 0;
  float r = number / denom;
  if (isnan_(r)) return 0;
  if (r == 0) return 0;
  *ratio = r;
  return 1;
}

SKC_HD bool between_(float a, float b, float c) { return (a - b) * (c - b) <= 0; }

// Conic::ChopIntoQuadsPOW2(pts, 1) -> 5 points
SKC_HD void ConicTo2Quads(P p0, P p1, P p2, float w, P out[5]) {
  float scale = 1.0f / (w + 1.0f);
  P wp1 = mkP(w * p1.x, w * p1.y);
  P m = mkP(((p0.x + (wp1.x + wp1.x)) + p2.x) * scale * 0.5f,
            ((p0.y + (wp1.y + wp1.y)) + p2.y) * scale * 0.5f);
  if (!isfinite_(m.x) || !isfinite_(m.y)) {
    double w_d = w, w_2 = w_d * 2, scale_half = 1 / (1 + w_d) * 0.5;
    m.x = (float)((p0.x + w_2 * p1.x + p2.x) * scale_half);
    m.y = (float)((p0.y + w_2 * p1.y + p2.y) * scale_half);
  }
  P d0p1 = mkP((p0.x + wp1.x) * scale, (p0.y + wp1.y) * scale);
  P d0p2 = m, d1p0 = m;
  P d1p1 = mkP((wp1.x + p2.x) * scale, (wp1.y + p2.y) * scale);
  float startY = p0.y, endY = p2.y;
  if (between_(startY, p1.y, endY)) {
    float midY = d0p2.y;
    if (!between_(startY, midY, endY)) {
      float closerY = fabs_(midY - startY) < fabs_(midY - endY) ? startY : endY;
      d0p2.y = d1p0.y = closerY;
    }
    if (!between_(startY, d0p1.y, d0p2.y)) d0p1.y = startY;
    if (!between_(d1p0.y, d1p1.y, endY)) d1p1.y = endY;
  }
  out[0] = p0;
  out[1] = d0p1;
  out[2] = d0p2;
  out[3] = d1p1;
  out[4] = p2;
  float prod = 0;
  for (int i = 0; i < 5; ++i) prod *= (out[i].x * out[i].y);
  if (!(prod == 0)) {
    for (int i = 1; i < 4; ++i) out[i] = p1;
  }
}

// Stroke::QuadPath (stroke.cc:914-962)
SKC_HDN void QuadPath(const PathView& src, DPath* dst) {
  PathIter it;
  it.init(src);
  P pts[4];
  for (;;) {
    uint8_t verb = it.Next(pts);
    switch (verb) {
      case kMove: dst->MoveTo(pts[0]); break;
      case kLine: dst->LineTo(pts[1]); break;
      case kQuad: dst->QuadTo(pts[1], pts[2]); break;
      case kConic: {
        P q[5];
        ConicTo2Quads(pts[0], pts[1], pts[2], it.weight, q);
        dst->QuadTo(q[1], q[2]);
        dst->QuadTo(q[3], q[4]);
      } break;
      case kCubic: {
        double n = CubicQuadCountD(pts);
        CubicCoeff cc;
        cc.set(pts[0], pts[1], pts[2], pts[3]);
        QuadCoeff qc;
        qc.set(mkP(3.f * (pts[1].x - pts[0].x), 3.f * (pts[1].y - pts[0].y)),
               mkP(3.f * (pts[2].x - pts[1].x), 3.f * (pts[2].y - pts[1].y)),
               mkP(3.f * (pts[3].x - pts[2].x), 3.f * (pts[3].y - pts[2].y)));
        for (int i = 0; i < n; ++i) {
          P q[3];
          CubicQuadAt(pts, cc, qc, n, i, q);
          dst->QuadTo(q[1], q[2]);
        }
      } break;
      case kClose: dst->Close(); break;
      default: return;
    }
  }
}

}  // namespace skc
