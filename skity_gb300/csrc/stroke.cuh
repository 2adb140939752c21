// Stroke-to-fill expansion for one path on one GPU thread: a restatement of
// the reference PathStroker (src/geometry/stroke.cc:18-901) with its conic
// arcs (src/geometry/conic.cc:73-166) and the double-precision normalisation
// of PointSetLength (src/geometry/point_priv.hpp:81-108).
#pragma once
#include "geom.cuh"

namespace skc {

constexpr float kNearlyZero = 1.0f / (1 << 12);
constexpr float kRoot2Over2 = 0.707106781f;
constexpr float kSqrt2 = 1.41421356f;
SKC_HD bool NearlyZero(float x, float tol = kNearlyZero) { return fabs_(x) <= tol; }

SKC_HD bool PointSetLength(P* pt, float x, float y, float length) {
  double xx = x, yy = y;
  double dmag = sqrtd_(xx * xx + yy * yy);
  double dscale = length / dmag;
  x = (float)(x * dscale);
  y = (float)(y * dscale);
  if (!isfinite_(x) || !isfinite_(y) || (x == 0 && y == 0)) {
    pt->x = 0;
    pt->y = 0;
    return false;
  }
  pt->x = x;
  pt->y = y;
  return true;
}
SKC_HD bool CanNormalize(float dx, float dy) { return isfinite_(dx) && isfinite_(dy) && (dx || dy); }
SKC_HD bool PointCanNormalize(float dx, float dy) {
  return (!isinf_(dx) && !isinf_(dy)) && (dx || dy);
}
SKC_HD float DistSqd(P a, P b) {
  float dx = a.x - b.x, dy = a.y - b.y;
  return dx * dx + dy * dy;
}

// skity::Matrix as used by round joins: column-major 4x4, glm products
struct Mat4 {
  float e[4][4];
  SKC_HD void identity() {
    for (int c = 0; c < 4; ++c)
      for (int r = 0; r < 4; ++r) e[c][r] = c == r ? 1.f : 0.f;
  }
  SKC_HD bool is_identity() const {
    for (int c = 0; c < 4; ++c)
      for (int r = 0; r < 4; ++r) {
        float want = c == r ? 1.f : 0.f;
        if (!(fabs_(e[c][r] - want) < 1.1920928955078125e-7f)) return false;
      }
    return true;
  }
};
SKC_HD Mat4 MatMul(const Mat4& a, const Mat4& b) {  // src/geometry/matrix.cc:452-460
  if (a.is_identity()) return b;
  if (b.is_identity()) return a;
  Mat4 r;
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
SKC_HD Mat4 MatScale(float sx, float sy) {
  Mat4 m;
  m.identity();
  m.e[0][0] = sx;
  m.e[1][1] = sy;
  return m;
}
SKC_HD Mat4 MatTranslate(float tx, float ty) {
  Mat4 m;
  m.identity();
  m.e[3][0] = tx;
  m.e[3][1] = ty;
  return m;
}
// Matrix::Skew(sx, sy) (include/skity/geometry/matrix.hpp:30-35)
SKC_HD Mat4 MatSkew(float kx, float ky) {
  Mat4 m;
  m.identity();
  m.e[1][0] = kx;
  m.e[0][1] = ky;
  return m;
}
// Matrix::Set9 (matrix.cc:96-104): a row-major 3x3 (scale x, skew x,
// translate x, skew y, scale y, translate y, perspective 0, 1, 2) into the
// column-major 4x4.
SKC_HD Mat4 MatFrom9(const float b[9]) {
  Mat4 m;
  m.identity();
  m.e[0][0] = b[0];
  m.e[0][1] = b[3];
  m.e[0][3] = b[6];
  m.e[1][0] = b[1];
  m.e[1][1] = b[4];
  m.e[1][3] = b[7];
  m.e[3][0] = b[2];
  m.e[3][1] = b[5];
  m.e[3][3] = b[8];
  return m;
}
// Matrix(16 floats), column-major: e[c][r] = m[4c + r] (the CONCAT44 /
// SET_M44 records of a picture, module/io/src/picture.cc:431-460,991-1011).
SKC_HD Mat4 MatFrom16(const float m[16]) {
  Mat4 r;
  for (int c = 0; c < 4; ++c)
    for (int k = 0; k < 4; ++k) r.e[c][k] = m[4 * c + k];
  return r;
}
// glm's mat4 product with no identity shortcut (what glm::rotate(...) * d1
// computes: columns summed left to right).
SKC_HD Mat4 MatMulPlain(const Mat4& a, const Mat4& b) {
  Mat4 r;
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
// Matrix::RotateDeg(deg, (px, py)) (matrix.cc:28-53): radians = deg times
// pi / 180 in float (FloatDegreesToRadians, scalar.hpp:101-103), then
// glm::rotate(Translate(px, py), rad, (0, 0, 1)) * Translate(-px, -py).
// glm::rotate builds the rotation about the normalised axis from cos and
// sin and right-multiplies its upper 3x3 into the matrix's first three
// columns, keeping the fourth.
SKC_HD Mat4 MatRotateDeg(float deg, float px, float py) {
  const float rad = deg * (float)0.01745329251994329576923690768489;
  const float c = cosf(rad), s = sinf(rad);
  const float ax[3] = {0.f, 0.f, 1.f};  // (0, 0, 1) normalised is itself
  const float tmp[3] = {(1.f - c) * ax[0], (1.f - c) * ax[1], (1.f - c) * ax[2]};
  float rot[3][3];
  rot[0][0] = c + tmp[0] * ax[0];
  rot[0][1] = tmp[0] * ax[1] + s * ax[2];
  rot[0][2] = tmp[0] * ax[2] - s * ax[1];
  rot[1][0] = tmp[1] * ax[0] - s * ax[2];
  rot[1][1] = c + tmp[1] * ax[1];
  rot[1][2] = tmp[1] * ax[2] + s * ax[0];
  rot[2][0] = tmp[2] * ax[0] + s * ax[1];
  rot[2][1] = tmp[2] * ax[1] - s * ax[0];
  rot[2][2] = c + tmp[2] * ax[2];
  const Mat4 d2 = MatTranslate(px, py);
  Mat4 r;
  for (int j = 0; j < 3; ++j)
    for (int k = 0; k < 4; ++k)
      r.e[j][k] = (d2.e[0][k] * rot[j][0] + d2.e[1][k] * rot[j][1]) + d2.e[2][k] * rot[j][2];
  for (int k = 0; k < 4; ++k) r.e[3][k] = d2.e[3][k];
  return MatMulPlain(r, MatTranslate(-px, -py));
}
SKC_HD P MatMapPoint(const Mat4& m, P p) {  // mat4 * (x, y, 0, 1)
  float rx = (m.e[0][0] * p.x + m.e[1][0] * p.y) + (m.e[2][0] * 0.f + m.e[3][0] * 1.f);
  float ry = (m.e[0][1] * p.x + m.e[1][1] * p.y) + (m.e[2][1] * 0.f + m.e[3][1] * 1.f);
  return mkP(rx, ry);
}

struct Conic {
  P pts[3];
  float w;
};

// Conic::BuildUnitArc (conic.cc:73-166)
SKC_HDN int BuildUnitArc(P start, P stop, bool ccw, const Mat4* user, Conic dst[5]) {
  float x = start.x * stop.x + start.y * stop.y;
  float y = start.x * stop.y - start.y * stop.x;
  float absY = fabs_(y);
  if (absY <= kNearlyZero && x > 0 && ((y >= 0 && !ccw) || (y <= 0 && ccw))) return 0;
  if (ccw) y = -y;
  int quadrant = 0;
  if (NearlyZero(y)) {
    quadrant = 2;
  } else if (NearlyZero(x)) {
    quadrant = y > 0 ? 1 : 3;
  } else {
    if (y < 0) quadrant += 2;
    if ((x < 0) != (y < 0)) quadrant += 1;
  }
  const float qx[8] = {1, 1, 0, -1, -1, -1, 0, 1};
  const float qy[8] = {0, 1, 1, 1, 0, -1, -1, -1};
  int count = quadrant;
  for (int i = 0; i < count; i++) {
    for (int j = 0; j < 3; ++j) dst[i].pts[j] = mkP(qx[i * 2 + j], qy[i * 2 + j]);
    dst[i].w = kRoot2Over2;
  }
  P finalP = mkP(x, y);
  P lastQ = mkP(qx[quadrant * 2], qy[quadrant * 2]);
  float dot = lastQ.x * finalP.x + lastQ.y * finalP.y;
  if (dot < 1) {
    P off = mkP(lastQ.x + x, lastQ.y + y);
    float cosThetaOver2 = sqrt_((1 + dot) / 2);
    PointSetLength(&off, off.x, off.y, 1.0f / cosThetaOver2);
    if (PointCanNormalize(lastQ.x - off.x, lastQ.y - off.y)) {
      dst[count].pts[0] = lastQ;
      dst[count].pts[1] = off;
      dst[count].pts[2] = finalP;
      dst[count].w = cosThetaOver2;
      count += 1;
    }
  }
  Mat4 m;
  m.identity();
  m.e[0][0] = start.x;
  m.e[0][1] = start.y;
  m.e[1][0] = -start.y;
  m.e[1][1] = start.x;
  if (ccw) m = MatMul(m, MatScale(1.0f, -1.0f));
  if (user) m = MatMul(*user, m);
  for (int i = 0; i < count; i++)
    for (int j = 0; j < 3; j++) dst[i].pts[j] = MatMapPoint(m, dst[i].pts[j]);
  return count;
}

SKC_HD P EvalQuadAt(const P q[3], float t) {
  QuadCoeff c;
  c.set(q[0], q[1], q[2]);
  return c.eval(t);
}
SKC_HD P EvalQuadTangentAt(const P q[3], float t) {  // geometry.cc:78-95
  if ((t == 0 && PEq(q[0], q[1])) || (t == 1 && PEq(q[1], q[2]))) {
    return mkP(q[2].x - q[0].x, q[2].y - q[0].y);
  }
  P B = mkP(q[1].x - q[0].x, q[1].y - q[0].y);
  P A = mkP((q[2].x - q[1].x) - B.x, (q[2].y - q[1].y) - B.y);
  P T = mkP(A.x * t + B.x, A.y * t + B.y);
  return mkP(T.x + T.x, T.y + T.y);
}
SKC_HD void EvalQuadAtClamped(const P q[3], float t, P* pt, P* tangent) {
  if (t < 0) t = 0;
  if (t > 1.0f) t = 1.0f;
  if (pt) *pt = EvalQuadAt(q, t);
  if (tangent) *tangent = EvalQuadTangentAt(q, t);
}
SKC_HD float pt_to_line(P pt, P a, P b) {  // geometry.cc:257-274
  P dxy = mkP(b.x - a.x, b.y - a.y);
  P ab0 = mkP(pt.x - a.x, pt.y - a.y);
  float number = dxy.x * ab0.x + dxy.y * ab0.y;
  float denom = dxy.x * dxy.x + dxy.y * dxy.y;
  float t = number / denom;
  if (t >= 0 && t <= 1) {
    P hit = mkP(a.x * (1 - t) + b.x * t, a.y * (1 - t) + b.y * t);
    return DistSqd(hit, pt);
  }
  return DistSqd(pt, a);
}
SKC_HD int FindUnitQuadRoots(float A, float B, float C, float roots[2]) {  // :128-160
  if (A == 0) return valid_unit_divide(-C, B, roots);
  int n = 0;
  double dr = (double)B * B - 4 * (double)A * C;
  if (dr < 0) return 0;
  dr = sqrtd_(dr);
  float R = (float)dr;
  if (isinf_(R)) return 0;
  float Q = (B < 0) ? -(B - R) / 2 : -(B + R) / 2;
  n += valid_unit_divide(Q, A, roots + n);
  n += valid_unit_divide(C, Q, roots + n);
  if (n == 2) {
    if (roots[0] > roots[1]) {
      float t = roots[0];
      roots[0] = roots[1];
      roots[1] = t;
    } else if (roots[0] == roots[1]) {
      n -= 1;
    }
  }
  return n;
}

struct QuadConstruct {  // stroke.cc:332-372
  P quad[3];
  P tangent_start, tangent_end;
  float start_t, mid_t, end_t;
  bool start_set, end_set;
  SKC_HD bool init(float start, float end) {
    start_t = start;
    mid_t = (start + end) * 0.5f;
    end_t = end;
    start_set = end_set = false;
    return start_t < mid_t && mid_t < end_t;
  }
  SKC_HD bool initWithStart(const QuadConstruct* parent) {
    if (!init(parent->start_t, parent->mid_t)) return false;
    quad[0] = parent->quad[0];
    tangent_start = parent->tangent_start;
    start_set = true;
    return true;
  }
  SKC_HD bool initWithEnd(const QuadConstruct* parent) {
    if (!init(parent->mid_t, parent->end_t)) return false;
    quad[2] = parent->quad[2];
    tangent_end = parent->tangent_end;
    end_set = true;
    return true;
  }
};

enum { kButtCap = 0, kRoundCap = 1, kSquareCap = 2 };
enum { kMiterJoin = 0, kRoundJoin = 1, kBevelJoin = 2 };

struct Stroker {
  float radius, scale, miter_limit, inv_res_scale, inv_res_scale_sq;
  DPath* outer;
  DPath* inner;
  P first_normal, prev_normal, first_unit_normal, prev_unit_normal;
  P first_pt, prev_pt, first_outer_pt;
  int segment_count;
  bool join_completed;
  int cap, join;
  int recursion_depth;
  int stroke_type;
  int inner_max_v, inner_max_p, inner_max_w;  // largest inner contour seen

  SKC_HD void init(float r, float miter, int cap_, int join_, DPath* o, DPath* in) {
    radius = r;
    scale = 1.f;
    miter_limit = miter;
    cap = cap_;
    join = join_;
    inv_res_scale = 1.f / (scale * 4);
    inv_res_scale_sq = inv_res_scale * inv_res_scale;
    if (join == kMiterJoin && miter <= 1.f) join = kBevelJoin;
    outer = o;
    inner = in;
    segment_count = -1;
    join_completed = false;
    recursion_depth = 0;
    stroke_type = 1;
    inner_max_v = inner_max_p = inner_max_w = 0;
    first_normal = prev_normal = first_unit_normal = prev_unit_normal = mkP(0, 0);
    first_pt = prev_pt = first_outer_pt = mkP(0, 0);
  }

  SKC_HD void Cap(DPath* path, P pivot, P normal, P stop) {  // stroke.cc:163-194
    if (cap == kButtCap) {
      path->LineTo(stop);
    } else if (cap == kSquareCap) {
      P par = mkP(-normal.y, normal.x);
      path->LineTo(mkP(pivot.x + normal.x + par.x, pivot.y + normal.y + par.y));
      path->LineTo(mkP(pivot.x - normal.x + par.x, pivot.y - normal.y + par.y));
      path->LineTo(stop);
    } else {
      P par = mkP(-normal.y, normal.x);
      P pc = mkP(pivot.x + par.x, pivot.y + par.y);
      path->ConicTo(mkP(pc.x + normal.x, pc.y + normal.y), pc, kRoot2Over2);
      path->ConicTo(mkP(pc.x - normal.x, pc.y - normal.y), stop, kRoot2Over2);
    }
  }
  static SKC_HD bool is_clockwise(P b, P a) { return b.x * a.y > b.y * a.x; }
  static SKC_HD void inner_join(DPath* in, P pivot, P after) {
    in->LineTo(pivot);
    in->LineTo(mkP(pivot.x - after.x, pivot.y - after.y));
  }
  static SKC_HD int AngleType(float dot) {  // 0 nearly 180, 1 sharp, 2 shallow, 3 nearly line
    if (dot >= 0) return NearlyZero(1.f - dot) ? 3 : 2;
    return NearlyZero(1.f + dot) ? 0 : 1;
  }
  SKC_HDN void Join(int kind, DPath* o, DPath* in, P bun, P pivot, P aun) {  // :196-330
    if (kind == kBevelJoin) {
      P after = mkP(aun.x * radius, aun.y * radius);
      if (!is_clockwise(bun, aun)) {
        swap_(o, in);
        after = mkP(-after.x, -after.y);
      }
      o->LineTo(mkP(pivot.x + after.x, pivot.y + after.y));
      inner_join(in, pivot, after);
    } else if (kind == kRoundJoin) {
      float dotProd = bun.x * aun.x + bun.y * aun.y;
      if (AngleType(dotProd) == 3) return;
      P before = bun, after = aun;
      bool ccw = false;
      if (!is_clockwise(before, after)) {
        swap_(o, in);
        before = mkP(-before.x, -before.y);
        after = mkP(-after.x, -after.y);
        ccw = true;
      }
      Mat4 m = MatMul(MatTranslate(pivot.x, pivot.y), MatScale(radius, radius));
      Conic conics[5];
      int count = BuildUnitArc(before, after, ccw, &m, conics);
      if (count > 0) {
        for (int i = 0; i < count; ++i) o->ConicTo(conics[i].pts[1], conics[i].pts[2], conics[i].w);
        after = mkP(after.x * radius, after.y * radius);
        inner_join(in, pivot, after);
      }
    } else {
      float dotProd = bun.x * aun.x + bun.y * aun.y;
      int angleType = AngleType(dotProd);
      P before = bun, after = aun, mid;
      if (angleType == 3) return;
      if (angleType == 0) {
        after = mkP(after.x * radius, after.y * radius);
        o->LineTo(mkP(pivot.x + after.x, pivot.y + after.y));
        inner_join(in, pivot, after);
        return;
      }
      if (!is_clockwise(before, after)) {
        swap_(o, in);
        before = mkP(-before.x, -before.y);
        after = mkP(-after.x, -after.y);
      }
      if (0 == dotProd && miter_limit >= kSqrt2) {
        mid = mkP((before.x + after.x) * radius, (before.y + after.y) * radius);
      } else {
        P od = mkP(before.x + after.x, before.y + after.y);
        float k = 2.f / (od.x * od.x + od.y * od.y);
        mid = mkP(k * od.x * radius, k * od.y * radius);
        if (sqrt_(mid.x * mid.x + mid.y * mid.y) >= miter_limit * radius) {
          after = mkP(after.x * radius, after.y * radius);
          o->LineTo(mkP(pivot.x + after.x, pivot.y + after.y));
          inner_join(in, pivot, after);
          return;
        }
      }
      o->LineTo(mkP(pivot.x + mid.x, pivot.y + mid.y));
      after = mkP(after.x * radius, after.y * radius);
      o->LineTo(mkP(pivot.x + after.x, pivot.y + after.y));
      inner_join(in, pivot, after);
    }
  }

  // Path::ReversePathTo(inner) appended to outer (path.cc:1042-1080)
  SKC_HD void ReverseInnerInto(DPath* dst) {
    if (inner->nv == 0) return;
    bool have = inner->cap_v >= inner->nv && inner->cap_p >= inner->np && inner->cap_w >= inner->nw;
    if (!have) {
      // count-only pass: the reversed contour adds exactly the segments
      // recorded since the inner path's MoveTo
      for (int i = 0; i < inner->c_line; ++i) dst->LineTo(mkP(0, 0));
      for (int i = 0; i < inner->c_quad; ++i) dst->QuadTo(mkP(0, 0), mkP(0, 0));
      for (int i = 0; i < inner->c_conic; ++i) dst->ConicTo(mkP(0, 0), mkP(0, 0), 0.5f);
      for (int i = 0; i < inner->c_cubic; ++i) dst->CubicTo(mkP(0, 0), mkP(0, 0), mkP(0, 0));
      return;
    }
    int vi = inner->nv;
    int pi = inner->np - 1;
    int wi = inner->nw;
    while (vi > 0) {
      uint8_t v = inner->verbs[--vi];
      int n = (v == kMove || v == kLine) ? 1 : ((v == kQuad || v == kConic) ? 2 : (v == kCubic ? 3 : 0));
      pi -= n;
      const P* pts = inner->pts + pi;
      switch (v) {
        case kMove: return;
        case kLine: dst->LineTo(pts[0]); break;
        case kQuad: dst->QuadTo(pts[1], pts[0]); break;
        case kConic: dst->ConicTo(pts[1], pts[0], inner->w[--wi]); break;
        case kCubic: dst->CubicTo(pts[2], pts[1], pts[0]); break;
        default: break;
      }
    }
  }

  SKC_HD void MoveTo(P pt) {  // stroke.cc:457-463
    if (segment_count > 0) FinishContour(false);
    segment_count = 0;
    first_pt = prev_pt = pt;
    join_completed = false;
  }
  SKC_HDN void FinishContour(bool close) {  // stroke.cc:733-769
    if (segment_count > 0) {
      if (close) {
        Join(join, outer, inner, prev_unit_normal, prev_pt, first_unit_normal);
        outer->Close();
        P pt = inner->LastPt();
        outer->MoveTo(pt);
        ReverseInnerInto(outer);
        outer->Close();
      } else {
        P pt = inner->LastPt();
        Cap(outer, prev_pt, prev_normal, pt);
        ReverseInnerInto(outer);
        Cap(outer, first_pt, mkP(-first_normal.x, -first_normal.y), first_outer_pt);
        outer->Close();
      }
    }
    inner_max_v = max_(inner_max_v, inner->nv);
    inner_max_p = max_(inner_max_p, inner->np);
    inner_max_w = max_(inner_max_w, inner->nw);
    inner->reset();
    segment_count = -1;
  }
  SKC_HD bool set_normal_unitnormal(P before, P after, P* normal, P* unit) {  // :100-110
    if (!PointSetLength(unit, (after.x - before.x) * scale, (after.y - before.y) * scale, 1.0f))
      return false;
    float tmp = unit->x;
    unit->x = unit->y;
    unit->y = -tmp;
    *normal = mkP(unit->x * radius, unit->y * radius);
    return true;
  }
  SKC_HD bool PreJoinTo(P curr, P* normal, P* unit) {  // :795-823
    float prevX = prev_pt.x, prevY = prev_pt.y;
    if (!set_normal_unitnormal(prev_pt, curr, normal, unit)) {
      if (cap == kButtCap) return false;
      *normal = mkP(radius, 0);
      *unit = mkP(1, 0);
    }
    if (segment_count == 0) {
      first_normal = *normal;
      first_unit_normal = *unit;
      first_outer_pt = mkP(prevX + normal->x, prevY + normal->y);
      outer->MoveTo(first_outer_pt);
      inner->MoveTo(mkP(prevX - normal->x, prevY - normal->y));
    } else {
      Join(join, outer, inner, prev_unit_normal, prev_pt, *unit);
    }
    return true;
  }
  SKC_HD void PostJoinTo(P curr, P normal, P unit) {
    join_completed = true;
    prev_pt = curr;
    prev_unit_normal = unit;
    prev_normal = normal;
    segment_count += 1;
  }
  SKC_HD void LineTo(P curr) {  // :472-488
    bool teeny = NearlyZero(prev_pt.x - curr.x, kNearlyZero * inv_res_scale) &&
                 NearlyZero(prev_pt.y - curr.y, kNearlyZero * inv_res_scale);
    if (teeny && cap == kButtCap) return;
    if (teeny && join_completed) return;
    P normal, unit;
    if (!PreJoinTo(curr, &normal, &unit)) return;
    outer->LineTo(mkP(curr.x + normal.x, curr.y + normal.y));
    inner->LineTo(mkP(curr.x - normal.x, curr.y - normal.y));
    PostJoinTo(curr, normal, unit);
  }

  // ---- quads
  SKC_HD static bool quad_in_line(const P q[3]) {  // :53-76
    float ptMax = -1;
    int outer1 = 0, outer2 = 0;
    for (int index = 0; index < 2; ++index) {
      for (int inner_ = index + 1; inner_ < 3; ++inner_) {
        float dx = q[inner_].x - q[index].x, dy = q[inner_].y - q[index].y;
        float testMax = max_(fabs_(dx), fabs_(dy));
        if (ptMax < testMax) {
          outer1 = index;
          outer2 = inner_;
          ptMax = testMax;
        }
      }
    }
    int mid = outer1 ^ outer2 ^ 3;
    const float kCurvatureSlop = 0.000005f;
    float lineSlop = ptMax * ptMax * kCurvatureSlop;
    return pt_to_line(q[mid], q[outer1], q[outer2]) <= lineSlop;
  }
  SKC_HD static float find_quad_max_curvature(const P src[3]) {  // :78-98
    float Ax = src[1].x - src[0].x;
    float Ay = src[1].y - src[0].y;
    float Bx = src[0].x - src[1].x - src[1].x + src[2].x;
    float By = src[0].y - src[1].y - src[1].y + src[2].y;
    float numer = -(Ax * Bx + Ay * By);
    float denom = Bx * Bx + By * By;
    if (denom < 0) {
      numer = -numer;
      denom = -denom;
    }
    if (numer <= 0) return 0;
    if (numer >= denom) return 1;
    return numer / denom;
  }
  SKC_HD static int CheckQuadLinear(const P q[3], P* reduction) {  // :836-858
    P p1c = mkP(q[1].x - q[0].x, q[1].y - q[0].y);
    bool d1 = !CanNormalize(p1c.x, p1c.y);
    P cp2 = mkP(q[2].x - q[1].x, q[2].y - q[1].y);
    bool d2 = !CanNormalize(cp2.x, cp2.y);
    if (d1 & d2) return 0;
    if (d1 | d2) return 1;
    if (!quad_in_line(q)) return 2;
    float t = find_quad_max_curvature(q);
    if (t == 0 || t == 1) return 1;
    EvalQuadAtClamped(q, t, reduction, nullptr);
    return 3;
  }
  SKC_HD void SetRayPts(P tPt, P* dxy, P* onPt, P* tangent) const {
    if (!PointSetLength(dxy, dxy->x, dxy->y, radius)) {
      dxy->x = radius;
      dxy->y = 0;
    }
    float axisFlip = (float)stroke_type;
    onPt->x = tPt.x + axisFlip * dxy->y;
    onPt->y = tPt.y - axisFlip * dxy->x;
    if (tangent) {
      tangent->x = onPt->x + dxy->x;
      tangent->y = onPt->y + dxy->y;
    }
  }
  SKC_HD void QuadPerpRay(const P q[3], float t, P* tPt, P* onPt, P* tangent) const {
    P dxy;
    EvalQuadAtClamped(q, t, tPt, &dxy);
    if (dxy.x == 0 && dxy.y == 0) dxy = mkP(q[2].x - q[0].x, q[2].y - q[0].y);
    SetRayPts(*tPt, &dxy, onPt, tangent);
  }
  enum { kSplit = 0, kDegenerate = 1, kQuadResult = 2 };
  SKC_HD int IntersectRay(QuadConstruct* qp) const {  // :625-671
    P start = qp->quad[0], end = qp->quad[2];
    P aLen = mkP(qp->tangent_start.x - start.x, qp->tangent_start.y - start.y);
    P bLen = mkP(qp->tangent_end.x - end.x, qp->tangent_end.y - end.y);
    float denom = aLen.x * bLen.y - aLen.y * bLen.x;
    if (denom == 0 || isinf_(denom) && denom > 0) return kDegenerate;
    P ab0 = mkP(start.x - end.x, start.y - end.y);
    float numerA = bLen.x * ab0.y - bLen.y * ab0.x;
    float numerB = aLen.x * ab0.y - aLen.y * ab0.x;
    if ((numerA >= 0) == (numerB >= 0)) {
      float dist1 = pt_to_line(start, end, qp->tangent_end);
      float dist2 = pt_to_line(end, start, qp->tangent_start);
      if (max_(dist1, dist2) <= inv_res_scale_sq) return kDegenerate;
      return kSplit;
    }
    numerA /= denom;
    bool valid = numerA > numerA - 1;
    if (valid) {
      qp->quad[1].x = start.x * (1 - numerA) + qp->tangent_start.x * numerA;
      qp->quad[1].y = start.y * (1 - numerA) + qp->tangent_start.y * numerA;
      return kQuadResult;
    }
    return kDegenerate;
  }
  SKC_HD bool PtInQuadBounds(const P q[3], P pt) const {  // :713-731
    float xMin = min_(min_(q[0].x, q[1].x), q[2].x);
    if (pt.x + inv_res_scale < xMin) return false;
    float xMax = max_(max_(q[0].x, q[1].x), q[2].x);
    if (pt.x - inv_res_scale > xMax) return false;
    float yMin = min_(min_(q[0].y, q[1].y), q[2].y);
    if (pt.y + inv_res_scale < yMin) return false;
    float yMax = max_(max_(q[0].y, q[1].y), q[2].y);
    if (pt.y - inv_res_scale > yMax) return false;
    return true;
  }
  SKC_HD static bool sharp_angle(const P quad[3]) {  // :134-149
    P smaller = mkP(quad[1].x - quad[0].x, quad[1].y - quad[0].y);
    P larger = mkP(quad[1].x - quad[2].x, quad[1].y - quad[2].y);
    float smallerLen = smaller.x * smaller.x + smaller.y * smaller.y;
    float largerLen = larger.x * larger.x + larger.y * larger.y;
    if (smallerLen > largerLen) {
      swap_(smaller, larger);
      largerLen = smallerLen;
    }
    if (!PointSetLength(&smaller, smaller.x, smaller.y, largerLen)) return false;
    float dot = smaller.x * larger.x + smaller.y * larger.y;
    return dot > 0;
  }
  SKC_HD static int intersect_quad_ray(const P line[2], const P quad[3], float roots[2]) {
    P vec = mkP(line[1].x - line[0].x, line[1].y - line[0].y);
    float r[3];
    for (int n = 0; n < 3; ++n) r[n] = (quad[n].y - line[0].y) * vec.x - (quad[n].x - line[0].x) * vec.y;
    float A = r[2], B = r[1], C = r[0];
    A += C - 2 * B;
    B -= C;
    return FindUnitQuadRoots(A, 2 * B, C, roots);
  }
  SKC_HD int StrokeCloseEnough(const P stroke[3], const P ray[2], QuadConstruct* qp) const {
    P strokeMid = EvalQuadAt(stroke, 0.5f);
    if (DistSqd(ray[0], strokeMid) <= inv_res_scale * inv_res_scale) {
      return sharp_angle(qp->quad) ? kSplit : kQuadResult;
    }
    if (!PtInQuadBounds(stroke, ray[0])) return kSplit;
    float roots[2];
    int rootCount = intersect_quad_ray(ray, stroke, roots);
    if (rootCount != 1) return kSplit;
    P quadPt = EvalQuadAt(stroke, roots[0]);
    float error = inv_res_scale * (1.f - fabs_(roots[0] - 0.5f) * 2);
    if (DistSqd(ray[0], quadPt) <= error * error) {
      return sharp_angle(qp->quad) ? kSplit : kQuadResult;
    }
    return kSplit;
  }
  SKC_HD int CompareQuadQuad(const P q[3], QuadConstruct* qp) {  // :568-591
    if (!qp->start_set) {
      P startPt;
      QuadPerpRay(q, qp->start_t, &startPt, &qp->quad[0], &qp->tangent_start);
      qp->start_set = true;
    }
    if (!qp->end_set) {
      P endPt;
      QuadPerpRay(q, qp->end_t, &endPt, &qp->quad[2], &qp->tangent_end);
      qp->end_set = true;
    }
    int rt = IntersectRay(qp);
    if (rt != kQuadResult) return rt;
    P ray[2];
    QuadPerpRay(q, qp->mid_t, &ray[1], &ray[0], nullptr);
    return StrokeCloseEnough(qp->quad, ray, qp);
  }
  // QuadStroke (stroke.cc:539-566) without recursion: an explicit stack of
  // pending halves reproduces the recursive visiting order, including the
  // abort on exceeding the depth limit (33) and the depth counter left
  // raised by an abort.
  SKC_HDN bool QuadStroke(const P q[3], QuadConstruct* root) {
    QuadConstruct stack[36];
    unsigned char state[36];  // 0: evaluate, 1: left half done, 2: both done
    int sp = 0;
    stack[0] = *root;
    state[0] = 0;
    bool ok = true;
    while (sp >= 0) {
      QuadConstruct* qp = &stack[sp];
      if (state[sp] == 0) {
        int rt = CompareQuadQuad(q, qp);
        if (rt == kQuadResult) {
          DPath* path = stroke_type == 1 ? outer : inner;
          path->QuadTo(qp->quad[1], qp->quad[2]);
          ok = true;
          sp--;
          continue;
        }
        if (rt == kDegenerate) {
          ok = true;
          sp--;
          continue;
        }
        if (++recursion_depth > 33) {
          ok = false;
          sp--;
          continue;
        }
        state[sp] = 1;
        stack[sp + 1].initWithStart(qp);
        state[sp + 1] = 0;
        sp++;
        continue;
      }
      if (state[sp] == 1) {
        if (!ok) {
          sp--;
          continue;
        }
        state[sp] = 2;
        stack[sp + 1].initWithEnd(qp);
        state[sp + 1] = 0;
        sp++;
        continue;
      }
      // state 2: right half returned
      if (ok) --recursion_depth;
      sp--;
    }
    return ok;
  }
  SKC_HDN void QuadTo(P c, P p2) {  // :490-527
    const P quad[3] = {prev_pt, c, p2};
    P reduction;
    int rt = CheckQuadLinear(quad, &reduction);
    if (rt == 0 || rt == 1) {
      LineTo(p2);
      return;
    }
    if (rt == 3) {
      LineTo(reduction);
      int save = join;
      join = kRoundJoin;
      LineTo(p2);
      join = save;
      return;
    }
    P normalAB, unitAB, normalBC, unitBC;
    if (!PreJoinTo(c, &normalAB, &unitAB)) {
      LineTo(p2);
      return;
    }
    QuadConstruct qp;
    stroke_type = 1;
    qp.init(0, 1);
    (void)QuadStroke(quad, &qp);
    stroke_type = -1;
    qp.init(0, 1);
    (void)QuadStroke(quad, &qp);
    if (!set_normal_unitnormal(quad[1], quad[2], &normalBC, &unitBC)) {
      normalBC = normalAB;
      unitBC = unitAB;
    }
    PostJoinTo(p2, normalBC, unitBC);
  }
};

// Stroke::StrokePath (stroke.cc:866-901); src has been through QuadPath
SKC_HDN void StrokePath(const PathView& src, float width, float miter, int cap, int join,
                        DPath* outer, DPath* inner, int inner_max[3]) {
  Stroker s;
  s.init(width * 0.5f, miter, cap, join, outer, inner);
  PathIter it;
  it.init(src);
  P pts[4];
  for (;;) {
    uint8_t verb = it.Next(pts);
    if (verb == kDone) break;
    switch (verb) {
      case kMove: s.MoveTo(pts[0]); break;
      case kLine: s.LineTo(pts[1]); break;
      case kQuad: s.QuadTo(pts[1], pts[2]); break;
      case kClose: s.FinishContour(true); break;
      default: break;
    }
  }
  s.FinishContour(false);
  inner_max[0] = s.inner_max_v;
  inner_max[1] = s.inner_max_p;
  inner_max[2] = s.inner_max_w;
}

}  // namespace skc
