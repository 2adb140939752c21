// Fixed-point edges, the edge sort and the analytic-AA scanline sweep for
// one draw on one GPU thread.  Restates src/render/sw/sw_edge.{hpp,cc} and
// src/render/sw/sw_raster.cc of the reference; spans go to a sink instead of
// a std::vector.
#pragma once
#include "geom.cuh"

namespace skc {

// SWEdge / SWQuadEdge (sw_edge.hpp:18-81), list links as indices
struct Edge {
  int32_t prev, next;
  Fixed x, y, dx, dy, upper_x, upper_y, lower_y;
  int8_t curve_count;
  uint8_t curve_shift;
  int8_t winding;
  uint8_t pad;
  Fixed qx, qy, qdx, qdy, qddx, qddy, q_first_y, q_last_x, q_last_y;
  Fixed snapped_x, snapped_y;
};

SKC_HD Fixed SnapY(Fixed y) {  // sw_edge.hpp:36-41
  return (Fixed)((((uint32_t)y + (uint32_t)(kFixed1 >> (kAccuracy + 1))) >> (16 - kAccuracy))
                 << (16 - kAccuracy));
}
SKC_HD void GoYShift(Edge* e, Fixed dst_y, int y_shift) {  // :55-58
  e->y = dst_y;
  e->x = wadd(e->x, e->dx >> y_shift);
}
SKC_HD void GoY(Edge* e, Fixed dst_y) {  // :43-51
  if (dst_y == wadd(e->y, kFixed1)) {
    e->x = wadd(e->x, e->dx);
    e->y = dst_y;
  } else if (e->y != dst_y) {
    e->x = wadd(e->upper_x, FixedMul(e->dx, wsub(e->y, e->upper_y)));
    e->y = dst_y;
  }
}
SKC_HD bool UpdateLine(Edge* e, Fixed x0, Fixed y0, Fixed x1, Fixed y1, Fixed slope) {  // sw_edge.cc:45-70
  if (y0 > y1) {
    swap_(x0, x1);
    swap_(y0, y1);
    e->winding = (int8_t)-e->winding;
  }
  FDot6 x0x1 = FixedToFDot6(wsub(x1, x0));
  FDot6 y0y1 = FixedToFDot6(wsub(y1, y0));
  if (y0y1 == 0) return false;
  e->x = x0;
  e->y = y0;
  e->dx = slope;
  e->dy = (x0x1 == 0 || slope == 0) ? kMaxS32 : iabs_(FixedDiv(y0y1, x0x1));
  e->upper_x = x0;
  e->upper_y = y0;
  e->lower_y = y1;
  return true;
}
SKC_HD bool SetLine(Edge* e, P p0, P p1) {  // sw_edge.cc:18-43
  const int mul = 1 << kAccuracy;
  Fixed x0 = FDot6ToFixed(ScalarToFDot6(p0.x * mul)) >> kAccuracy;
  Fixed y0 = SnapY(FDot6ToFixed(ScalarToFDot6(p0.y * mul)) >> kAccuracy);
  Fixed x1 = FDot6ToFixed(ScalarToFDot6(p1.x * mul)) >> kAccuracy;
  Fixed y1 = SnapY(FDot6ToFixed(ScalarToFDot6(p1.y * mul)) >> kAccuracy);
  e->winding = 1;
  FDot6 y0y1 = FixedToFDot6(wsub(y1, y0));
  if (y0y1 == 0) return false;
  FDot6 x0x1 = FixedToFDot6(wsub(x1, x0));
  Fixed slope = FixedDiv(x0x1, y0y1);
  e->curve_count = 0;
  e->curve_shift = 0;
  return UpdateLine(e, x0, y0, x1, y1, slope);
}
SKC_HD bool CanBeIgnored(float top, float bottom, Fixed y0, Fixed y1) {  // :72-88
  const int mul = 1 << kAccuracy;
  Fixed start_y = SnapY(FDot6ToFixed(ScalarToFDot6(top * mul)) >> kAccuracy);
  Fixed stop_y = SnapY(FDot6ToFixed(ScalarToFDot6(bottom * mul)) >> kAccuracy);
  return y0 >= stop_y || y1 <= start_y;
}
SKC_HD int diff_to_shift(FDot6 dx, FDot6 dy, int shiftAA) {  // :97-119
  dx = iabs_(dx);
  dy = iabs_(dy);
  FDot6 dist = max_(dx, dy) + (min_(dx, dy) >> 1);
  dist = (dist + (1 << (2 + shiftAA))) >> (3 + shiftAA);
  return (32 - clz_((uint32_t)dist)) >> 1;
}
SKC_HD bool UpdateQuad(Edge* e) {  // sw_edge.cc:233-292
  int success = 0;
  int count = e->curve_count;
  Fixed oldx = e->qx, oldy = e->qy;
  Fixed dx = e->qdx, dy = e->qdy;
  Fixed newx = 0, newy = 0, nsx = 0, nsy = 0;
  int shift = e->curve_shift;
  do {
    Fixed slope;
    if (--count > 0) {
      newx = wadd(oldx, dx >> shift);
      newy = wadd(oldy, dy >> shift);
      if (iabs_(dy >> shift) >= kFixed1 * 2) {
        FDot6 diffY = FixedToFDot6(wsub(newy, e->snapped_y));
        slope = diffY ? FixedDiv(FixedToFDot6(wsub(newx, e->snapped_x)), diffY) : kMaxS32;
        nsy = min_<Fixed>(e->q_last_y, FixedRoundToFixed(newy));
        nsx = wsub(newx, FixedMul(slope, wsub(newy, nsy)));
      } else {
        nsy = min_<Fixed>(e->q_last_y, SnapY(newy));
        nsx = newx;
        FDot6 diffY = FixedToFDot6(wsub(nsy, e->snapped_y));
        slope = diffY ? FixedDiv(FixedToFDot6(wsub(newx, e->snapped_x)), diffY) : kMaxS32;
      }
      dx = wadd(dx, e->qddx);
      dy = wadd(dy, e->qddy);
    } else {
      newx = e->q_last_x;
      newy = e->q_last_y;
      nsy = newy;
      nsx = newx;
      FDot6 diffY = wsub(newy, e->snapped_y) >> 10;
      slope = diffY ? FixedDiv(wsub(newx, e->snapped_x) >> 10, diffY) : kMaxS32;
    }
    if (slope < kMaxS32) success = UpdateLine(e, e->snapped_x, e->snapped_y, nsx, nsy, slope);
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
SKC_HD bool SetQuad(Edge* e, const P pts[3]) {  // sw_edge.cc:121-231
  float scale = (float)(1 << (kAccuracy + 6));
  FDot6 x0 = (int)(pts[0].x * scale), y0 = (int)(pts[0].y * scale);
  FDot6 x1 = (int)(pts[1].x * scale), y1 = (int)(pts[1].y * scale);
  FDot6 x2 = (int)(pts[2].x * scale), y2 = (int)(pts[2].y * scale);
  int w = 1;
  if (y0 > y2) {
    swap_(x0, x2);
    swap_(y0, y2);
    w = -1;
  }
  if (FDot6Round(y0) == FDot6Round(y2)) return false;
  FDot6 dx = (LShift(x1, 1) - x0 - x2) >> 2;
  FDot6 dy = (LShift(y1, 1) - y0 - y2) >> 2;
  int shift = diff_to_shift(dx, dy, kAccuracy);
  if (shift == 0) {
    shift = 1;
  } else if (shift > 6) {
    shift = 6;
  }
  e->winding = (int8_t)w;
  e->curve_count = (int8_t)(1 << shift);
  e->curve_shift = (uint8_t)(shift - 1);
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

// ChopQuadAtYExtrema (src/geometry/geometry.cc:311-349)
SKC_HD int ChopQuadAtYExtrema(const P src[3], P dst[5]) {
  float a = src[0].y, b = src[1].y, c = src[2].y;
  float ab = a - b, bc = b - c;
  if (ab < 0) bc = -bc;
  if (ab == 0 || bc < 0) {
    float t;
    if (valid_unit_divide(a - b, a - b - b + c, &t)) {
      P p01 = mkP(src[0].x + (src[1].x - src[0].x) * t, src[0].y + (src[1].y - src[0].y) * t);
      P p12 = mkP(src[1].x + (src[2].x - src[1].x) * t, src[1].y + (src[2].y - src[1].y) * t);
      dst[0] = src[0];
      dst[1] = p01;
      dst[2] = mkP(p01.x + (p12.x - p01.x) * t, p01.y + (p12.y - p01.y) * t);
      dst[3] = p12;
      dst[4] = src[2];
      dst[1].y = dst[3].y = dst[2].y;
      return 1;
    }
    b = fabs_(a - b) < fabs_(b - c) ? a : c;
  }
  dst[0] = src[0];
  dst[1] = src[1];
  dst[2] = src[2];
  dst[1].y = b;
  return 0;
}

// Pixel-space bounds of a (translated) quad path and the scan bounds
// derived from them (sw_raster.cc:731-754, path.cc:1341-1360).
struct RasterBounds {
  bool empty;
  float l, t, r, b;      // floor/ceil of the path bounds (bounds_)
  float sl, st, sr, sb;  // scan bounds
};
// The canvas matrix RastePath maps the quadified path by
// (Path::CopyWithMatrix, path.cc:1274-1294, sw_raster.cc:740): glm's
// mat4 * vec4 sums the columns as (m0 x + m1 y) + (m2 0 + m3 1), which is
// (sx x + kx y) + tx in each row.  A translation (lin false) maps
// x -> x + tx: its (1 x + 0 y) is x exactly.
struct Xform {
  float tx, ty;
  float sx, kx, ky, sy;  // the linear part (lin)
  bool lin;
  SKC_HD P map(P p) const {
    if (!lin) return mkP(p.x + tx, p.y + ty);
    return mkP((sx * p.x + kx * p.y) + tx, (ky * p.x + sy * p.y) + ty);
  }
};

// The clip bounds (cl, ct, cr, cb) are the canvas's global clip bounds:
// kMaxCullRect (+-1e9, include/skity/render/canvas.hpp:26) unless a
// ClipRect narrowed them.
SKC_HD RasterBounds ComputeBounds(const PathView& q, const Xform& xf, float cl = -1e9f,
                                  float ct = -1e9f, float cr = 1e9f, float cb = 1e9f) {
  RasterBounds rb;
  rb.empty = true;
  rb.l = rb.t = rb.r = rb.b = rb.sl = rb.st = rb.sr = rb.sb = 0;
  int n = q.np;
  if (q.nv > 1 && q.verbs[q.nv - 1] == kMove) n--;
  if (n <= 0) return rb;
  const P p0 = xf.map(q.pts[0]);
  float l = p0.x, t = p0.y, r = l, b = t;
  for (int i = 1; i < n; ++i) {
    const P pi = xf.map(q.pts[i]);
    const float x = pi.x, y = pi.y;
    l = min_(l, x);
    r = max_(r, x);
    t = min_(t, y);
    b = max_(b, y);
  }
  rb.l = floor_(l);
  rb.t = floor_(t);
  rb.r = ceil_(r);
  rb.b = ceil_(b);
  // scan_bounds.Intersect(clip_bounds) (sw_raster.cc:746-748, rect.cc:160-172)
  float sl = max_(l, cl), sr = min_(r, cr), st = max_(t, ct), sb = min_(b, cb);
  if (!(sl < sr && st < sb)) return rb;
  sl = floor_(sl);
  st = floor_(st);
  sr = ceil_(sr);
  sb = ceil_(sb);
  if (!(sl < sr && st < sb)) return rb;
  rb.empty = false;
  rb.sl = sl;
  rb.st = st;
  rb.sr = sr;
  rb.sb = sb;
  return rb;
}

// SWEdgeBuilder::BuildEdges over PathEdgeIter (sw_edge.cc:299-336,
// src/graphic/path_priv.hpp:75-170).  Points are mapped by the canvas
// matrix first (Xform).  Returns the number of edges (may exceed cap: only
// cap are stored).
SKC_HDN int BuildEdges(const PathView& q, const Xform& xf, float top, float bottom,
                       Edge* out, int cap) {
  int n = 0;
  int vi = 0, pi = 0, move_to = 0;
  bool needs_close = false;
  auto T = [&](int i) { return xf.map(q.pts[i]); };
  auto add_line = [&](P a, P b) {
    Edge e;
    if (SetLine(&e, a, b) && !CanBeIgnored(top, bottom, e.upper_y, e.lower_y)) {
      if (n < cap) out[n] = e;
      n++;
    }
  };
  auto add_quad = [&](const P* qq) {
    Edge e;
    if (SetQuad(&e, qq) && !CanBeIgnored(top, bottom, e.q_first_y, e.q_last_y)) {
      if (n < cap) out[n] = e;
      n++;
    }
  };
  for (;;) {
    if (vi == q.nv) {
      if (needs_close) add_line(T(pi - 1), T(move_to));
      return n;
    }
    uint8_t v = q.verbs[vi++];
    if (v == kMove) {
      if (needs_close) {
        add_line(T(pi - 1), T(move_to));
        needs_close = false;
      }
      move_to = pi++;
    } else if (v == kClose) {
      if (needs_close) {
        add_line(T(pi - 1), T(move_to));
        needs_close = false;
      }
    } else {
      int k = (v + 2) / 2;
      needs_close = true;
      pi += k;
      int s = pi - (k + 1);
      if (v == kLine) {
        add_line(T(s), T(s + 1));
      } else if (v == kQuad) {
        P seg[3] = {T(s), T(s + 1), T(s + 2)};
        P mono[5];
        int c = ChopQuadAtYExtrema(seg, mono);
        for (int i = 0; i <= c; i++) add_quad(&mono[i * 2]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Edge sort: the reference sorts with std::sort (sw_raster.cc:679-704), whose
// order among fully tied edges is that of introsort as the C++ runtime
// implements it (Musser's introsort: median-of-three Hoare partitioning down
// to blocks of 16, heapsort past a depth of 2*floor(log2 n), then insertion
// sort).  Tied edges must keep that order for pixel parity, so the same
// published algorithm is restated here over edge indices; tests compare its
// permutation with std::sort.
// ---------------------------------------------------------------------------
struct EdgeLess {
  const Edge* e;
  SKC_HD bool operator()(int32_t ia, int32_t ib) const {
    int va = e[ia].upper_y, vb = e[ib].upper_y;
    if (va == vb) {
      va = e[ia].x;
      vb = e[ib].x;
    }
    if (va == vb) {
      va = e[ia].dx;
      vb = e[ib].dx;
    }
    return va < vb;
  }
};

template <typename Less>
SKC_HD void heap_sift(int32_t* a, int hole, int len, int32_t value, Less less) {
  // move the hole down to a leaf along larger children, then sift value up
  const int top = hole;
  int child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (less(a[child], a[child - 1])) child--;
    a[hole] = a[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    a[hole] = a[child - 1];
    hole = child - 1;
  }
  int parent = (hole - 1) / 2;
  while (hole > top && less(a[parent], value)) {
    a[hole] = a[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  a[hole] = value;
}
template <typename Less>
SKC_HD void heap_sort_range(int32_t* a, int len, Less less) {
  if (len < 2) return;
  for (int parent = (len - 2) / 2;; --parent) {
    heap_sift(a, parent, len, a[parent], less);
    if (parent == 0) break;
  }
  for (int last = len - 1; last > 0; --last) {
    int32_t v = a[last];
    a[last] = a[0];
    heap_sift(a, 0, last, v, less);
  }
}
template <typename Less>
SKC_HD void median_to_first(int32_t* a, int r, int x, int y, int z, Less less) {
  if (less(a[x], a[y])) {
    if (less(a[y], a[z])) swap_(a[r], a[y]);
    else if (less(a[x], a[z])) swap_(a[r], a[z]);
    else swap_(a[r], a[x]);
  } else if (less(a[x], a[z])) {
    swap_(a[r], a[x]);
  } else if (less(a[y], a[z])) {
    swap_(a[r], a[z]);
  } else {
    swap_(a[r], a[y]);
  }
}
template <typename Less>
SKC_HD int partition_pivot(int32_t* a, int first, int last, Less less) {
  int mid = first + (last - first) / 2;
  median_to_first(a, first, first + 1, mid, last - 1, less);
  int lo = first + 1, hi = last;
  const int32_t pivot = a[first];
  for (;;) {
    while (less(a[lo], pivot)) ++lo;
    --hi;
    while (less(pivot, a[hi])) --hi;
    if (!(lo < hi)) return lo;
    swap_(a[lo], a[hi]);
    ++lo;
  }
}
template <typename Less>
SKC_HD void insertion_sort(int32_t* a, int first, int last, Less less) {
  if (first == last) return;
  for (int i = first + 1; i < last; ++i) {
    int32_t v = a[i];
    if (less(v, a[first])) {
      for (int k = i; k > first; --k) a[k] = a[k - 1];
      a[first] = v;
    } else {
      int k = i;
      while (less(v, a[k - 1])) {
        a[k] = a[k - 1];
        --k;
      }
      a[k] = v;
    }
  }
}
template <typename Less>
SKC_HD void unguarded_insertion_sort(int32_t* a, int first, int last, Less less) {
  for (int i = first; i < last; ++i) {
    int32_t v = a[i];
    int k = i;
    while (less(v, a[k - 1])) {
      a[k] = a[k - 1];
      --k;
    }
    a[k] = v;
  }
}
struct IntLess {
  SKC_HD bool operator()(int32_t a, int32_t b) const { return a < b; }
};

template <typename Less>
SKC_HDN void introsort(int32_t* a, int n, Less less) {
  if (n < 2) return;
  // explicit stack of [first, last, depth] ranges (right part recursed
  // first, left part looped), same visiting order as the recursive form
  struct Range { int first, last, depth; };
  Range stack[64];
  int sp = 0;
  int lg = 31 - clz_((uint32_t)n);
  stack[sp++] = Range{0, n, 2 * lg};
  while (sp > 0) {
    Range r = stack[--sp];
    int first = r.first, last = r.last, depth = r.depth;
    while (last - first > 16) {
      if (depth == 0) {
        heap_sort_range(a + first, last - first, less);
        break;
      }
      --depth;
      int cut = partition_pivot(a, first, last, less);
      // the recursive form sorts [cut, last) before continuing with
      // [first, cut); both orders give the same result since the ranges are
      // disjoint, but keep the reference's order for clarity
      stack[sp++] = Range{first, cut, depth};
      first = cut;
      if (sp >= 63) break;  // cannot happen: depth <= 2*log2(n) < 62
    }
    if (last - first > 16 && depth != 0 && sp >= 63) {
      heap_sort_range(a + first, last - first, less);
    }
  }
  if (n > 16) {
    insertion_sort(a, 0, 16, less);
    unguarded_insertion_sort(a, 16, n, less);
  } else {
    insertion_sort(a, 0, n, less);
  }
}

// ---------------------------------------------------------------------------
// Execution width of a sweep: a whole warp on the GPU (the sequential sweep
// logic runs warp-uniformly -- every lane computes the same values -- and the
// per-pixel loops are split across lanes), one thread on the CPU.
// ---------------------------------------------------------------------------
// SKC_WARP_LANES: the lanes of a sweep are the 32 threads of a warp.  A
// translation unit that defines SKC_SOLO_LANES before its includes compiles
// the sweep for one thread per pass instead (the form the CPU runs).
#if defined(__CUDA_ARCH__) && !defined(SKC_SOLO_LANES)
#define SKC_WARP_LANES 1
#endif
struct Lanes {
#ifdef SKC_WARP_LANES
  static constexpr int n = 32;
  int lane;
  __device__ unsigned ballot(bool p) const { return __ballot_sync(0xffffffffu, p); }
  __device__ void sync() const { __syncwarp(); }
  __device__ uint32_t shfl(uint32_t v, int src) const { return __shfl_sync(0xffffffffu, v, src); }
  __device__ unsigned lt_mask() const { return (1u << lane) - 1u; }
  __device__ static int popc(unsigned m) { return __popc(m); }
  __device__ static int ffs(unsigned m) { return __ffs((int)m); }
#else
  static constexpr int n = 1;
  int lane = 0;
  SKC_HD unsigned ballot(bool p) const { return p ? 1u : 0u; }
  SKC_HD void sync() const {}
  SKC_HD uint32_t shfl(uint32_t v, int) const { return v; }
  SKC_HD unsigned lt_mask() const { return 0u; }
#ifdef __CUDA_ARCH__
  __device__ static int popc(unsigned m) { return __popc(m); }
  __device__ static int ffs(unsigned m) { return __ffs((int)m); }
#else
  static int popc(unsigned m) { return __builtin_popcount(m); }
  static int ffs(unsigned m) { return __builtin_ffs((int)m); }
#endif
#endif
  SKC_HD bool leader() const { return lane == 0; }
};

// Runs of equal nonzero alphas in acc[lo, hi), in increasing x
// (SpanBuilder::Flush, sw_raster.cc:103-136); emit(start, width, alpha) is
// called warp-uniformly, one call per run.
template <typename F>
SKC_HD void acc_runs_lanes(const Lanes& L, const uint8_t* acc, int lo, int hi, F&& emit) {
  int open_start = -1;
  uint8_t open_v = 0;
  for (int base = lo; base < hi; base += Lanes::n) {
    int i = base + L.lane;
    uint8_t v = i < hi ? acc[i] : 0;
    uint8_t pv = (i > lo && i < hi) ? acc[i - 1] : 0;
    unsigned mask = L.ballot(i < hi && v != pv);
    while (mask) {
      int bit = Lanes::ffs(mask) - 1;
      mask &= mask - 1;
      int pos = base + bit;
      uint8_t bv = (uint8_t)L.shfl(v, bit);
      if (open_start >= 0) {
        emit(open_start, pos - open_start, open_v);
        open_start = -1;
      }
      if (bv != 0) {
        open_start = pos;
        open_v = bv;
      }
    }
  }
  if (open_start >= 0) emit(open_start, hi - open_start, open_v);
}

// ---------------------------------------------------------------------------
// AAA scanline sweep (sw_raster.cc:19-677) with a span sink
// ---------------------------------------------------------------------------
// Sink interface (Sink::real(x, y, len, alpha), Sink::acc_row(y, alphas,
// left, lo, hi) is called at flush with the accumulated row).
SKC_HD uint8_t partial_alpha_h(uint8_t alpha, Fixed h) {
  return (uint8_t)FixedRoundToInt(wmul(alpha, h));
}
SKC_HD uint8_t partial_alpha_a(uint8_t alpha, uint8_t full) { return (uint8_t)((alpha * full) >> 8); }
SKC_HD Fixed approximate_intersection(Fixed l1, Fixed r1, Fixed l2, Fixed r2) {
  if (l1 > r1) swap_(l1, r1);
  if (l2 > r2) swap_(l2, r2);
  return wadd(max_(l1, l2), min_(r1, r2)) / 2;
}
SKC_HD uint8_t trapezoid_to_alpha(Fixed l1, Fixed l2) {
  Fixed area = wadd(l1, l2) / 2;
  return (uint8_t)(area >> 8);
}
SKC_HD uint8_t partial_triangle_to_alpha(Fixed a, Fixed b) {
  Fixed area = wmul(wmul(a >> 11, a >> 11), b >> 11);
  return (uint8_t)((area >> 8) & 0xFF);
}

// Entry i of compute_alpha_below_line (below = true) or
// compute_alpha_above_line (sw_raster.cc:314-370) over R = ceil(r) pixels;
// the reference fills the entries with a running sum, re-derived here per
// entry so any subset can be computed.
SKC_HD uint8_t triangle_entry(bool below, Fixed l, Fixed r, Fixed dY, uint8_t full, int i) {
  int R = FixedCeilToInt(r);
  if (R == 1) {
    return below ? partial_alpha_a(trapezoid_to_alpha(l, r), full)
                 : partial_alpha_a((uint8_t)(wsub(wsub(R << 17, l), r) >> 9), full);
  }
  Fixed first = kFixed1 - l;
  Fixed last = r - ((R - 1) << 16);
  if (below) {
    Fixed lastH = FixedMul(last, dY);
    if (i == R - 1) return (uint8_t)(FixedMul(last, lastH) >> 9);
    if (i == 0) return (uint8_t)(full - partial_triangle_to_alpha(first, dY));
    Fixed a16 = wadd(wadd(lastH, dY >> 1), wmul(R - 2 - i, dY));
    return (uint8_t)((a16 >> 8) & 0xFF);
  }
  Fixed firstH = FixedMul(first, dY);
  if (i == 0) return (uint8_t)(FixedMul(first, firstH) >> 9);
  if (i == R - 1) return (uint8_t)(full - partial_triangle_to_alpha(last, dY));
  Fixed a16 = wadd(wadd(firstH, dY >> 1), wmul(i - 1, dY));
  return (uint8_t)(a16 >> 8);
}

}  // namespace skc
