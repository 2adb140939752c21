// FP64 exact-area coverage of a filled path -- test infrastructure, an
// independent yardstick, not a restatement of the reference.
//
// The reference rasteriser (src/render/sw/sw_raster.cc) is an analytic-AA
// approximation in 16.16 fixed point; this computes what it approximates:
// for every pixel, the area of the pixel square covered by the path's fill
// region (nonzero or even-odd), in double precision.
//
// Input: the path after QuadPath (moves, lines, quads, closes; contours are
// closed implicitly, as PathEdgeIter closes them, path_priv.hpp:121-170).
// Quads are flattened into `n` uniform pieces with the chord error bound
// |p0 - 2 p1 + p2| / (8 n^2) <= tol.  For each pixel row the piece ends and
// the pairwise crossings of pieces inside the row cut it into slabs where the
// pieces keep their x order; in a slab the fill region is a union of
// trapezoids between consecutive pieces where the winding is inside, and a
// trapezoid's area over each pixel column is integrated exactly (the
// integrand, clamp(x(y) - column, 0, 1), is piecewise linear in y).
// Result: exact for polygons, within tol per unit length for curves.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

struct Seg {
  double x0, y0, x1, y1;  // y0 < y1 after orientation
  int w;                  // +1 for a downward piece, -1 upward
};

// Integral over [ya, yb] of clamp(x(y) - c, 0, 1) for x linear from xa (at
// ya) to xb (at yb).
double ColumnIntegral(double xa, double xb, double ya, double yb, double c) {
  const double h = yb - ya;
  if (h <= 0) return 0;
  auto g = [&](double t) { return xa + (xb - xa) * t - c; };  // t in [0, 1]
  // breakpoints where g crosses 0 or 1
  double ts[4] = {0, 1, 0, 0};
  int n = 2;
  const double d = xb - xa;
  if (d != 0) {
    for (double level : {0.0, 1.0}) {
      const double t = (c + level - xa) / d;
      if (t > 0 && t < 1) ts[n++] = t;
    }
  }
  for (int i = 1; i < n; ++i)  // insertion sort of at most 4 values
    for (int j = i; j > 0 && ts[j] < ts[j - 1]; --j) std::swap(ts[j], ts[j - 1]);
  double area = 0;
  for (int i = 0; i + 1 < n; ++i) {
    const double t0 = ts[i], t1 = ts[i + 1];
    if (t1 <= t0) continue;
    const double v0 = std::min(1.0, std::max(0.0, g(t0)));
    const double v1 = std::min(1.0, std::max(0.0, g(t1)));
    area += 0.5 * (v0 + v1) * (t1 - t0);
  }
  return area * h;
}

void AddPiece(std::vector<Seg>& out, double x0, double y0, double x1, double y1) {
  if (y0 == y1) return;
  if (y0 < y1) {
    out.push_back({x0, y0, x1, y1, 1});
  } else {
    out.push_back({x1, y1, x0, y0, -1});
  }
}

double XAt(const Seg& s, double y) {
  if (s.y1 == s.y0) return s.x0;
  return s.x0 + (s.x1 - s.x0) * ((y - s.y0) / (s.y1 - s.y0));
}

}  // namespace

extern "C" {

// verbs: 0 move, 1 line, 2 quad, 5 close (a QuadPath); pts: x, y pairs.
// Writes width*height coverages in [0, 1] to cov. Returns 0, or -2 for a
// verb it does not take.
int ska_exact_coverage(const uint8_t* verbs, uint32_t nv, const float* pts, uint32_t np,
                       int even_odd, int width, int height, double tol, double* cov) {
  std::vector<Seg> segs;
  double sx = 0, sy = 0, cx = 0, cy = 0;
  bool open = false;
  uint32_t pi = 0;
  auto close = [&]() {
    if (open && (cx != sx || cy != sy)) AddPiece(segs, cx, cy, sx, sy);
    open = false;
  };
  for (uint32_t i = 0; i < nv; ++i) {
    switch (verbs[i]) {
      case 0:
        close();
        if (pi >= np) return -2;
        sx = cx = pts[2 * pi];
        sy = cy = pts[2 * pi + 1];
        pi += 1;
        open = true;
        break;
      case 1: {
        if (pi >= np) return -2;
        const double x = pts[2 * pi], y = pts[2 * pi + 1];
        pi += 1;
        AddPiece(segs, cx, cy, x, y);
        cx = x;
        cy = y;
        break;
      }
      case 2: {
        if (pi + 1 >= np) return -2;
        const double x1 = pts[2 * pi], y1 = pts[2 * pi + 1];
        const double x2 = pts[2 * pi + 2], y2 = pts[2 * pi + 3];
        pi += 2;
        const double ddx = cx - 2 * x1 + x2, ddy = cy - 2 * y1 + y2;
        const double dd = std::sqrt(ddx * ddx + ddy * ddy);
        int n = (int)std::ceil(std::sqrt(dd / (8 * tol)));
        n = std::max(1, std::min(n, 1 << 16));
        double px = cx, py = cy;
        for (int k = 1; k <= n; ++k) {
          const double t = (double)k / n, u = 1 - t;
          const double x = u * u * cx + 2 * u * t * x1 + t * t * x2;
          const double y = u * u * cy + 2 * u * t * y1 + t * t * y2;
          AddPiece(segs, px, py, x, y);
          px = x;
          py = y;
        }
        cx = x2;
        cy = y2;
        break;
      }
      case 5:
        close();
        cx = sx;
        cy = sy;
        break;
      default:
        return -2;
    }
  }
  close();
  std::fill(cov, cov + (size_t)width * height, 0.0);
  // pieces by the rows they touch
  std::vector<std::vector<int>> by_row(height);
  for (size_t i = 0; i < segs.size(); ++i) {
    const int r0 = std::max(0, (int)std::floor(segs[i].y0));
    const int r1 = std::min(height - 1, (int)std::ceil(segs[i].y1) - 1);
    for (int r = r0; r <= r1; ++r) by_row[r].push_back((int)i);
  }
  std::vector<double> full(width + 1), part(width);
  std::vector<Seg> row;
  std::vector<double> cuts;
  std::vector<std::pair<double, int>> act;
  for (int r = 0; r < height; ++r) {
    if (by_row[r].empty()) continue;
    const double top = r, bot = r + 1;
    row.clear();
    for (int i : by_row[r]) {
      const Seg& s = segs[i];
      const double ya = std::max(top, s.y0), yb = std::min(bot, s.y1);
      if (yb <= ya) continue;
      row.push_back({XAt(s, ya), ya, XAt(s, yb), yb, s.w});
    }
    if (row.empty()) continue;
    cuts.clear();
    cuts.push_back(top);
    cuts.push_back(bot);
    for (const Seg& s : row) {
      cuts.push_back(s.y0);
      cuts.push_back(s.y1);
    }
    // crossings: pieces whose x ranges overlap, found by a sweep in x
    std::vector<int> ord(row.size());
    for (size_t i = 0; i < row.size(); ++i) ord[i] = (int)i;
    auto xmin = [&](int i) { return std::min(row[i].x0, row[i].x1); };
    auto xmax = [&](int i) { return std::max(row[i].x0, row[i].x1); };
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return xmin(a) < xmin(b); });
    for (size_t a = 0; a < ord.size(); ++a) {
      const Seg& p = row[ord[a]];
      const double pmax = xmax(ord[a]);
      for (size_t b = a + 1; b < ord.size() && xmin(ord[b]) <= pmax; ++b) {
        const Seg& q = row[ord[b]];
        const double lo = std::max(p.y0, q.y0), hi = std::min(p.y1, q.y1);
        if (hi <= lo) continue;
        const double d0 = XAt(p, lo) - XAt(q, lo), d1 = XAt(p, hi) - XAt(q, hi);
        if ((d0 < 0 && d1 > 0) || (d0 > 0 && d1 < 0))
          cuts.push_back(lo + (hi - lo) * (d0 / (d0 - d1)));
      }
    }
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    std::fill(full.begin(), full.end(), 0.0);
    std::fill(part.begin(), part.end(), 0.0);
    // adds sign * (area left of the piece within each column) over [y0, y1]
    auto add_edge = [&](const Seg& s, double y0, double y1, double sign) {
      const double xa = XAt(s, y0), xb = XAt(s, y1);
      const double lo = std::min(xa, xb), hi = std::max(xa, xb);
      const double h = y1 - y0;
      int c0 = (int)std::floor(lo), c1 = (int)std::ceil(hi);
      if (c1 == c0) c1 = c0 + 1;
      // columns left of c0 are covered for the full slab height
      const int f = std::min(std::max(c0, 0), width);
      full[0] += sign * h;
      full[f] -= sign * h;
      for (int c = std::max(c0, 0); c < std::min(c1, width); ++c)
        part[c] += sign * ColumnIntegral(xa, xb, y0, y1, c);
    };
    for (size_t k = 0; k + 1 < cuts.size(); ++k) {
      const double y0 = cuts[k], y1 = cuts[k + 1];
      if (y1 - y0 <= 0) continue;
      const double ym = 0.5 * (y0 + y1);
      act.clear();
      for (size_t i = 0; i < row.size(); ++i) {
        if (row[i].y0 <= y0 && row[i].y1 >= y1) act.push_back({XAt(row[i], ym), (int)i});
      }
      if (act.size() < 2) continue;
      std::sort(act.begin(), act.end());
      int w = 0;
      for (size_t i = 0; i < act.size(); ++i) {
        const int prev = w;
        w += row[act[i].second].w;
        const bool in_before = even_odd ? (prev & 1) : prev != 0;
        const bool in_after = even_odd ? (w & 1) : w != 0;
        if (!in_before && in_after) add_edge(row[act[i].second], y0, y1, -1.0);
        if (in_before && !in_after) add_edge(row[act[i].second], y0, y1, 1.0);
      }
    }
    double run = 0;
    for (int c = 0; c < width; ++c) {
      run += full[c];
      const double v = run + part[c];
      cov[(size_t)r * width + c] = std::min(1.0, std::max(0.0, v));
    }
  }
  return 0;
}

}  // extern "C"
