// The sweep of sweep.cuh with the active edges held in registers.
//
// Same per-step restatement of WalkEdges (src/render/sw/sw_raster.cc:546-677)
// as LaneSweep, but the state that the generic form keeps in per-pass global
// arrays lives on chip:
//   * list position p of the active list is slot p / 32 of lane p % 32; a
//     slot holds the edge's index, x, dx, dy, lower_y, winding and curve
//     count in registers, and in the 32-edge form its quad-piece state too
//     (the larger forms keep that in the pass's edge copy in global memory,
//     touched only when a piece ends);
//   * the per-position values an interval reads (x before the step, after
//     GoY and after the update, dx, dy) and the interval endpoints are
//     exchanged through a per-warp shared-memory block;
//   * the reorder of the survivors is a compaction when their new x are
//     already non-decreasing in list order (no crossing in the step), and
//     the rank computation of LaneSweep otherwise;
//   * each step's intervals, the one left open by a culled right edge
//     included, are blitted in one pass after the reorder has been decided.
// A path whose active list would exceed M edges (the form's size) is not swept here
// (RegWalk returns 0 before touching its sink's output for the first time
// at that size) and goes to LaneSweep.
#pragma once
#include "sweep.cuh"

namespace skc {

constexpr int kRegMaxM = 128;  // the largest active list held in registers
// intervals of one step with at most M active edges: one per pair of them,
// plus the one left open by a culled right edge
SKC_HD constexpr int RegIntervals(int M) { return M / 2 + 4; }

// TrapRow set-ups of a step's intervals, one array per field.
template <int N>
struct TrapRowSoA {
  int32_t ul[N], ur[N], ll[N], lr[N], ldy[N], rdy[N];
  uint32_t meta[N];  // full | real << 8
  SKC_HD void put(int i, const TrapRow& t) {
    ul[i] = t.ul;
    ur[i] = t.ur;
    ll[i] = t.ll;
    lr[i] = t.lr;
    ldy[i] = t.lDY;
    rdy[i] = t.rDY;
    meta[i] = (uint32_t)t.full | (t.real ? 0x100u : 0u);
  }
  SKC_HD TrapRow get(int i) const {
    TrapRow t;
    t.ul = ul[i];
    t.ur = ur[i];
    t.ll = ll[i];
    t.lr = lr[i];
    t.lDY = ldy[i];
    t.rDY = rdy[i];
    t.full = (uint8_t)(meta[i] & 0xFF);
    t.real = (meta[i] & 0x100u) != 0;
    return t;
  }
};

// The quad-piece state of an active edge that UpdateQuad reads besides the
// edge's line (x, dx, dy, lower_y, winding, curve count): forward-difference
// position, steps and second differences, the last point, the shift.  The
// 32-edge form holds it in registers beside the rest of the edge (one slot
// per lane), so a piece change is a register update; the larger forms, with
// two or four slots per lane, keep it in the pass's edge copy in memory.
constexpr int kRegQuadWords = 9;
SKC_HD constexpr bool RegQuadHeld(int M) { return M == 32; }
struct RegQuad {
  int32_t w[kRegQuadWords];  // qx, qy, qdx, qdy, qddx, qddy, q_last_x, q_last_y, curve_shift
  SKC_HD void load(const Edge& e) {
    w[0] = e.qx;
    w[1] = e.qy;
    w[2] = e.qdx;
    w[3] = e.qdy;
    w[4] = e.qddx;
    w[5] = e.qddy;
    w[6] = e.q_last_x;
    w[7] = e.q_last_y;
    w[8] = e.curve_shift;
  }
  SKC_HD void put(Edge& e) const {
    e.qx = w[0];
    e.qy = w[1];
    e.qdx = w[2];
    e.qdy = w[3];
    e.qddx = w[4];
    e.qddy = w[5];
    e.q_last_x = w[6];
    e.q_last_y = w[7];
    e.curve_shift = (uint8_t)w[8];
  }
};

// Per-warp shared block of the register sweep for active lists of up to
// M edges.
template <int M>
struct RegSharedT {
  static constexpr int kIntervals = RegIntervals(M);
  static constexpr int kFlushEvents = 2 * M;  // nonzero accumulator entries a flush gathers
  int32_t xo[M];   // x before the step, by list position
  int32_t xg[M];   //   after GoY
  int32_t xf[M];   //   after the quad-piece update
  int32_t dxo[M];  // dx before the step
  int32_t dyo[M];  // dy before the step
  int32_t dxf[M];  // dx after the update
  int32_t ia[M];   // interval k: left position
  int32_t ib[M];   //   right position
  int32_t ax[M];   // active x at insertion; new rank by list position in the reorder
  // edge state by new list position (reorder and insertion)
  int32_t p_idx[M], p_x[M], p_dx[M], p_dy[M];
  int32_t p_low[M], p_wc[M];
  // the quad-piece state of the edges (RegQuad) by new list position, for
  // the forms that keep it in registers
  int32_t p_q[RegQuadHeld(M) ? kRegQuadWords : 1][M];
  union {
    struct {
      // the step's intervals (blit_trapezoid_row set-ups) and their first span
      TrapRowSoA<kIntervals> iv;
      int32_t iv_start[kIntervals + 4];
    } b;
    // accumulator flush scratch (used between steps, never during a blit)
    int32_t ev[2 * kFlushEvents];
  } u;
  uint8_t surv[M];  // 1: survives the step
};
// Host and device must agree on these sizes (the host sizes the launch).
static_assert(sizeof(RegSharedT<32>) % 16 == 0, "RegSharedT keeps 16-byte alignment");
static_assert(sizeof(RegSharedT<64>) % 16 == 0, "RegSharedT keeps 16-byte alignment");
static_assert(sizeof(RegSharedT<128>) % 16 == 0, "RegSharedT keeps 16-byte alignment");

SKC_HD int32_t MakeWc(int winding, int count) { return (winding & 0xFF) | ((count & 0xFF) << 8); }
SKC_HD int WcWinding(int32_t wc) { return (int8_t)(wc & 0xFF); }
SKC_HD int WcCount(int32_t wc) { return (int8_t)((wc >> 8) & 0xFF); }

SKC_HD long long LaneMax64(const Lanes& L, long long v) {
#ifdef SKC_WARP_LANES
  for (int o = 16; o > 0; o >>= 1) {
    long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
#endif
  return v;
}

// Row accumulator of the sweep (the difference array and its touched range).
struct AccState {
  int32_t* diff;
  int left, width;
  int y;       // row being accumulated (kNaN32: none yet)
  int lo, hi;  // touched entries [lo, hi] (this lane's adds; reduced at the flush)
  int32_t* ev; // flush scratch: (position, value) of nonzero entries
  int ev_cap;
};

template <typename Sink>
SKC_HD void AccFlush(const Lanes& L, AccState& a, Sink* sink) {
  if (a.y == kNaN32) return;
  a.lo = LaneMin(L, a.lo);
  a.hi = LaneMax(L, a.hi);
  if (a.lo <= a.hi) {
    const bool read = sink->acc_row(L, a.y, a.diff, a.left, a.lo, a.hi, a.ev, a.ev_cap);
    L.sync();
    if (SKC_LIKELY(read)) {
      if (L.leader()) a.diff[a.hi] = 0;
    } else {
      for (int i = a.lo + L.lane; i <= a.hi; i += Lanes::n) a.diff[i] = 0;
    }
    L.sync();
  }
  a.lo = 0x7fffffff;
  a.hi = -1;
}

template <typename Sink>
SKC_HD void AccFlushIfNeed(const Lanes& L, AccState& a, Sink* sink, int row) {
  if (a.y == row) return;
  if (a.y != kNaN32) AccFlush(L, a, sink);
  a.y = row;
}

// Trapezoid rows of a row's steps waiting for their spans: the set-ups of
// intervals [0, n) in the shared interval block, `total` spans, canvas row y.
struct BlitPending {
  int n, total, y;
};

// The spans of the pending intervals, numbered in interval order, spread
// over the lanes (span g on lane g mod 32), so a long partial row does not
// hold one lane while the others wait.  Direct spans are written in that
// order, the others go to the row accumulator.
template <int M, typename Sink>
SKC_HD void RegBlitFlush(const Lanes& L, RegSharedT<M>& sh, Sink* sink, AccState& as,
                         BlitPending& pend) {
  constexpr int NL = Lanes::n;
  if (pend.n == 0) return;
  sink->row_begin(L, pend.y);
  if (L.leader()) sh.u.b.iv_start[pend.n] = pend.total;
  L.sync();
  const int T = pend.total;
  const int y = pend.y;
  uint32_t run = 0;
  unsigned long long frags = 0;
  int lo = 0x7fffffff, hi = -1;
  int iv = 0;
  for (int gb = 0; gb < T; gb += NL) {
    const int g = gb + L.lane;
    bool kept = false;
    uint2 v = make_uint2(0, 0);
    if (g < T) {
      while (sh.u.b.iv_start[iv + 1] <= g) ++iv;
      const TrapRow t = sh.u.b.iv.get(iv);
      int x = 0, len = 0;
      uint8_t a = 0;
      TrapSpan(t, g - sh.u.b.iv_start[iv], x, len, a);
      if (t.real) {
        if (sink->keep(x, y, len, a)) {
          kept = true;
          v = sink->pack(x, len, a);
          frags += (unsigned)len;
        }
      } else {
        int o0 = x - as.left, o1 = o0 + len;
        o0 = max_(o0, 0);
        o1 = min_(o1, as.width);
        if (o0 < o1) {
          lo = min_(lo, o0);
          hi = max_(hi, o1);
          if (a != 0) {
            AtomicAddI32(&as.diff[o0], (int32_t)a);
            AtomicAddI32(&as.diff[o1], -(int32_t)a);
          }
        }
      }
    }
    const unsigned km = L.ballot(kept);
    const uint32_t cnt = (uint32_t)Lanes::popc(km);
    if (cnt) {
      const uint64_t at = sink->reserve(L, run, cnt);
      uint2* dst = sink->span_ptr(at + run + (uint32_t)Lanes::popc(km & L.lt_mask()));
      if (kept && dst) *dst = v;
      run += cnt;
    }
  }
  // the fragment count and the accumulator's touched range stay per lane
  // (summed at the pass's end, reduced at the row's flush)
  as.lo = min_(as.lo, lo);
  as.hi = max_(as.hi, hi);
  sink->commit(L, run, frags);
  pend.n = 0;
  pend.total = 0;
  L.sync();
}

// The intervals [0, K) of a step, then (trailing_a >= 0) the interval left
// open by the last left edge: blit_trapezoid_row for each.  One lane per
// interval does the row's set-up and counts its spans; the set-ups wait in
// the interval block, with those of the row's earlier steps, until the row
// ends or the block is full (a row's partial steps all go to the
// accumulator, whose sums do not depend on order; a full step is the only
// step of its row), and their spans are then made in one pass.
template <int M, typename Sink>
SKC_HD void RegBlit(const Lanes& L, RegSharedT<M>& sh, Sink* sink, AccState& as,
                    BlitPending& pend, const Edge* W, int n, int y, Fixed next_y, int K, int m,
                    int k, uint8_t full, Fixed left_clip, Fixed right_clip, int trailing_a,
                    bool trailing_nr) {
  constexpr int NL = Lanes::n;
  const int total = K + (trailing_a >= 0 ? 1 : 0);
  if (pend.n > 0 && (pend.y != y || pend.n + total > RegSharedT<M>::kIntervals))
    RegBlitFlush(L, sh, sink, as, pend);
  AccFlushIfNeed(L, as, sink, y);
  int carry = 0;
  for (int kb = 0; kb < total; kb += NL) {
    const int ki = kb + L.lane;
    int cnt = 0;
    if (ki < total) {
      Fixed ul, ur, ll, lr, lDY, rDY;
      bool nr;
      if (ki < K) {
        const int a = sh.ia[ki], b = sh.ib[ki];
        ul = max_(sh.xo[a], left_clip);
        lDY = sh.dyo[a];
        ur = min_(right_clip, sh.xo[b]);
        ll = max_(left_clip, sh.xf[a]);
        lr = min_(right_clip, sh.xg[b]);
        rDY = sh.dyo[b];
        int prev_right;
        if (ki == 0) {
          prev_right = FixedFloorToInt(left_clip);
        } else {
          const int pb = sh.ib[ki - 1];
          prev_right = FixedCeilToInt(max_(min_(right_clip, sh.xo[pb]), sh.xg[pb]));
        }
        bool tc = prev_right > FixedFloorToInt(ul) || prev_right > FixedFloorToInt(sh.xf[a]);
        if (!tc) {
          // edges_too_close(right edge, its successor before the step)
          int32_t nxo, ndx;
          Fixed nup;
          if (b + 1 < m) {
            nxo = sh.xo[b + 1];
            ndx = sh.dxo[b + 1];
            nup = kMinS32;  // active: upper_y <= y < next_y
          } else if (k < n) {
            nxo = W[k].x;
            ndx = W[k].dx;
            nup = W[k].upper_y;
          } else {
            nxo = kMaxS32;
            ndx = 0;
            nup = kMaxS32;
          }
          tc = nup < next_y && wadd(sh.xg[b], kFixed1) >= wsub(nxo, iabs_(ndx));
        }
        nr = tc;
      } else {
        const int a = trailing_a;
        ul = max_(sh.xo[a], left_clip);
        lDY = sh.dyo[a];
        ur = right_clip;
        ll = max_(left_clip, sh.xf[a]);
        lr = right_clip;
        rDY = 0;
        nr = trailing_nr;
      }
      TrapRow t;
      if (TrapPrepare(t, ul, ur, ll, lr, lDY, rDY, full, nr)) {
        cnt = TrapCount(t);
        sh.u.b.iv.put(pend.n + ki, t);
      }
    }
    const int32_t incl = LaneScanIncl(L, cnt);
    if (ki < total) sh.u.b.iv_start[pend.n + ki] = pend.total + carry + incl - cnt;
    carry += LaneBcast(L, incl, NL - 1);
  }
  pend.y = y;
  pend.n += total;
  pend.total += carry;
  L.sync();
}

// WalkEdges over the pass's sorted edges W[0, n) (modified in place: quad
// pieces).  Returns 0 if the active list would exceed M edges.
template <int M, typename Sink>
SKC_HD int RegWalk(const Lanes& L, RegSharedT<M>& sh, Edge* W, int n, Sink* sink, AccState& as,
                   float scan_top, bool even_odd, int start_y, int stop_y, Fixed left_clip,
                   Fixed right_clip) {
  constexpr int NL = Lanes::n;
  constexpr int S = M / NL;
  constexpr unsigned kFull = NL == 32 ? 0xffffffffu : 1u;
  const int winding_mask = even_odd ? 1 : -1;
  int32_t r_idx[S], r_x[S], r_dx[S], r_dy[S], r_low[S], r_wc[S];
  constexpr bool kQ = RegQuadHeld(M);
  RegQuad r_q[kQ ? S : 1];

  BlitPending pend;
  pend.n = pend.total = 0;
  pend.y = kNaN32;
  Fixed y = max_(W[0].upper_y, IntToFixed(start_y));
  // initial activation: the edges with upper_y <= y, in their sorted order
  int k = 0;
  for (int base = 0; base < n; base += NL) {
    const int i = base + L.lane;
    const unsigned mask = L.ballot(i < n && W[i].upper_y <= y);
    k += Lanes::popc(mask);
    if (mask != kFull) break;
  }
  if (k > M) return 0;
  int m = k;
  Fixed nny = kMaxS32;
  {
    int32_t lmin = kMaxS32;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const int p = s * NL + L.lane;
      r_idx[s] = r_x[s] = r_dx[s] = r_dy[s] = r_low[s] = r_wc[s] = 0;
      if (p < m) {
        Edge e = W[p];
        GoY(&e, y);
        if (kQ) r_q[s].load(e);
        r_idx[s] = p;
        r_x[s] = e.x;
        r_dx[s] = e.dx;
        r_dy[s] = e.dy;
        r_low[s] = e.lower_y;
        r_wc[s] = MakeWc(e.winding, e.curve_count);
        if (e.lower_y > y) lmin = min_(lmin, e.lower_y);
      }
    }
    lmin = LaneMin(L, lmin);
    nny = min_(nny, lmin);
    if (k < n && W[k].upper_y > y) nny = min_(nny, W[k].upper_y);
  }

  for (;;) {
    Fixed next_y = min_(nny, FixedCeilToFixed(y + 1));
    int y_shift = 0;
    if ((next_y - y) & (kFixed1 >> 2)) {
      y_shift = 2;
      next_y = y + (kFixed1 >> 2);
    } else if ((next_y - y) & (kFixed1 >> 1)) {
      y_shift = 1;
    }
    const uint8_t full = partial_alpha_h(0xFF, next_y - y);
    nny = kMaxS32;
    const int ns = (m + NL - 1) / NL;

    // ---- A: advance every active edge
    int32_t wcarry = 0;
    int nl = 0, nr = 0;
    unsigned smask[S];
    int32_t lmin = kMaxS32;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      smask[s] = 0;
      if (s < ns) {
        const int p = s * NL + L.lane;
        const bool valid = p < m;
        const int32_t wv = valid ? (int32_t)WcWinding(r_wc[s]) : 0;
        const int32_t incl = LaneScanIncl(L, wv) + wcarry;
        const int32_t excl = incl - wv;
        const bool in = (incl & winding_mask) != 0;
        const bool pin = (excl & winding_mask) != 0;
        const bool is_left = valid && in && !pin;
        const bool is_right = valid && !in && pin;
        const unsigned lm = L.ballot(is_left), rm = L.ballot(is_right);
        bool surv = false;
        if (valid) {
          const int32_t xo = r_x[s], dxo = r_dx[s], dyo = r_dy[s];
          int32_t x = wadd(xo, dxo >> y_shift);  // GoYShift
          const int32_t xg = x;
          if (SKC_COLD(r_low[s] <= next_y && WcCount(r_wc[s]) > 0)) {
            Edge e;
            if (kQ) {
              r_q[s].put(e);
            } else {
              e = W[r_idx[s]];
            }
            e.x = x;
            e.y = next_y;
            e.dx = dxo;
            e.dy = dyo;
            e.lower_y = r_low[s];
            e.winding = (int8_t)WcWinding(r_wc[s]);
            e.curve_count = (int8_t)WcCount(r_wc[s]);
            while (e.lower_y <= next_y && e.curve_count > 0) {
              e.snapped_x = e.x;  // KeepContinuous (sw_edge.cc:294-297)
              e.snapped_y = e.y;
              if (!UpdateQuad(&e)) break;
            }
            if (kQ) {
              r_q[s].load(e);
            } else {
              W[r_idx[s]] = e;
            }
            x = e.x;
            r_dx[s] = e.dx;
            r_dy[s] = e.dy;
            r_low[s] = e.lower_y;
            r_wc[s] = MakeWc(e.winding, e.curve_count);
          }
          r_x[s] = x;
          surv = r_low[s] > next_y;
          if (surv) lmin = min_(lmin, r_low[s]);
          sh.xo[p] = xo;
          sh.xg[p] = xg;
          sh.xf[p] = x;
          sh.dxo[p] = dxo;
          sh.dyo[p] = dyo;
          sh.dxf[p] = r_dx[s];
          sh.surv[p] = surv ? 1 : 0;
          if (is_left) sh.ia[nl + Lanes::popc(lm & L.lt_mask())] = p;
          if (is_right) sh.ib[nr + Lanes::popc(rm & L.lt_mask())] = p;
        }
        smask[s] = L.ballot(surv);
        nl += Lanes::popc(lm);
        nr += Lanes::popc(rm);
        wcarry = LaneBcast(L, incl, min_(NL, m - s * NL) - 1);
      }
    }
    const bool final_in = (wcarry & winding_mask) != 0;
    L.sync();

    // ---- C: survivors in stable order of their new x; intersections
    int m2 = 0;
    int r_rank[S];
    bool cross = false, inv = false;
    {
      int last = -1, before = 0;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        r_rank[s] = 0;
        if (s < ns) {
          const unsigned below = smask[s] & L.lt_mask();
          const bool surv = (smask[s] >> (NL == 32 ? L.lane : 0)) & 1u;
          const int q = below ? s * NL + (31 - clz_(below)) : last;
          r_rank[s] = before + Lanes::popc(below);
          if (surv && q >= 0) {
            const int32_t xq = sh.xf[q];
            if (xq > r_x[s]) inv = true;
            if (wadd(xq, sh.dxf[q]) > wadd(r_x[s], r_dx[s])) cross = true;
          }
          before += Lanes::popc(smask[s]);
          if (smask[s]) last = s * NL + (31 - clz_(smask[s]));
        }
      }
      m2 = before;
    }
    const bool any_inv = L.ballot(inv) != 0;
    if (SKC_COLD(any_inv)) {
      // Some survivor moved left of an earlier one.  The reference ripples
      // each such edge backwards (backward_insert_edge_based_on_x), which
      // leaves the survivors stably sorted by new x; its crossing check then
      // compares an edge with its predecessor at that moment: the latest
      // (in sorted order) earlier-listed survivor whose x is not greater.
      // Sort the survivors' (x, list position) keys in place by odd-even
      // transposition (the list is nearly sorted, so few phases run), then
      // find each one's predecessor by a short backward scan.
      int32_t* kx = sh.p_x;
      int32_t* kp = sh.p_idx;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (s < ns && p < m && sh.surv[p]) {
          kx[r_rank[s]] = r_x[s];
          kp[r_rank[s]] = p;
        }
      }
      L.sync();
      bool dirty_prev = true;
      for (int phase = 0; phase < m2 + 2; ++phase) {
        bool swapped = false;
        for (int i = 2 * L.lane + (phase & 1); i + 1 < m2; i += 2 * NL) {
          const int32_t xa = kx[i], xb = kx[i + 1];
          const int32_t pa = kp[i], pb = kp[i + 1];
          if (xb < xa || (xb == xa && pb < pa)) {
            kx[i] = xb;
            kx[i + 1] = xa;
            kp[i] = pb;
            kp[i + 1] = pa;
            swapped = true;
          }
        }
        L.sync();
        const bool dirty = L.ballot(swapped) != 0;
        if (!dirty && !dirty_prev) break;
        dirty_prev = dirty;
      }
      cross = false;
      for (int r = L.lane; r < m2; r += NL) {
        const int pr = kp[r];
        sh.ax[pr] = r;
        int q = r - 1;
        while (q >= 0 && kp[q] > pr) --q;
        if (q >= 0 && wadd(kx[q], sh.dxf[kp[q]]) > wadd(kx[r], sh.dxf[pr])) cross = true;
      }
      L.sync();
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (s < ns && p < m && sh.surv[p]) r_rank[s] = sh.ax[p];
      }
      L.sync();
    }
    lmin = LaneMin(L, lmin);
    nny = min_(nny, lmin);
    if (L.ballot(cross)) nny = min_(nny, next_y + (kFixed1 >> kAccuracy));

    // ---- the interval left open by the last left edge (its right edge was
    // culled): too-close test against the left edge's predecessor after the
    // reorder (its new predecessor if it survives, else the last processed
    // survivor before it)
    int trailing_a = -1;
    bool trailing_nr = false;
    if (SKC_COLD(final_in)) {
      const int a = sh.ia[nr];
      const bool a_surv = sh.surv[a] != 0;
      const int32_t xa = sh.xf[a];
      long long key = 0;
      bool found = false;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (s < ns && p < m && sh.surv[p]) {
          const int32_t xi = r_x[s];
          const bool cand = a_surv ? (p != a && (xi < xa || (xi == xa && p < a))) : p < a;
          if (cand) {
            const long long kk = ((long long)xi << 32) | (unsigned)p;
            if (!found || kk > key) key = kk;
            found = true;
          }
        }
      }
      const bool any = L.ballot(found) != 0;
      if (!found) key = (long long)kMinS32 << 32;
      key = LaneMax64(L, key);
      const int32_t pred_x = any ? (int32_t)(key >> 32) : left_clip;
      const bool tc = wadd(pred_x, kFixed1) >= wsub(xa, iabs_(sh.dxf[a]));
      trailing_a = a;
      trailing_nr = full == 0xFF && tc;
    }

    // ---- B: coverage of the step's intervals, in list order
    const int row = y >> 16;
    if (nr + (final_in ? 1 : 0) > 0 && !(row < scan_top)) {
      RegBlit(L, sh, sink, as, pend, W, n, row, next_y, nr, m, k, full, left_clip, right_clip,
              trailing_a, trailing_nr);
    }

    // ---- reorder the survivors into the new list (nothing moves when every
    // edge survives in order: the rank of position p is then p)
    if (SKC_COLD(m2 != m || any_inv)) {
#pragma unroll
      for (int s = 0; s < S; ++s) {
        if (s < ns && ((smask[s] >> (NL == 32 ? L.lane : 0)) & 1u)) {
          const int r = r_rank[s];
          sh.p_idx[r] = r_idx[s];
          sh.p_x[r] = r_x[s];
          sh.p_dx[r] = r_dx[s];
          sh.p_dy[r] = r_dy[s];
          sh.p_low[r] = r_low[s];
          sh.p_wc[r] = r_wc[s];
          if (kQ) {
#pragma unroll
            for (int j = 0; j < kRegQuadWords; ++j) sh.p_q[j][r] = r_q[s].w[j];
          }
        }
      }
      L.sync();
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (p < m2) {
          r_idx[s] = sh.p_idx[p];
          r_x[s] = sh.p_x[p];
          r_dx[s] = sh.p_dx[p];
          r_dy[s] = sh.p_dy[p];
          r_low[s] = sh.p_low[p];
          r_wc[s] = sh.p_wc[p];
          if (kQ) {
#pragma unroll
            for (int j = 0; j < kRegQuadWords; ++j) r_q[s].w[j] = sh.p_q[j][p];
          }
        }
      }
      L.sync();
    }
    m = m2;
    y = next_y;
    if (y >= IntToFixed(stop_y)) break;

    // ---- D: insert_new_edges (sw_raster.cc:207-247) as a merge
    if (SKC_COLD(k < n && W[k].upper_y <= y)) {
      int c = 0;
      for (int base = k; base < n; base += NL) {
        const int i = base + L.lane;
        const unsigned mask = L.ballot(i < n && W[i].upper_y <= y);
        c += Lanes::popc(mask);
        if (mask != kFull) break;
      }
      if (SKC_COLD(m + c > M)) return 0;
      const int32_t x0 = W[k].x;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (p < m) sh.ax[p] = r_x[s];
      }
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (p < m) {
          const int32_t xa = r_x[s];
          int before = 0;
          if (xa > x0) {
            before = 1;
            for (int t = 1; t < c; ++t) before += W[k + t].x <= xa ? 1 : 0;
          }
          const int np = p + before;
          sh.p_idx[np] = r_idx[s];
          sh.p_x[np] = r_x[s];
          sh.p_dx[np] = r_dx[s];
          sh.p_dy[np] = r_dy[s];
          sh.p_low[np] = r_low[s];
          sh.p_wc[np] = r_wc[s];
          if (kQ) {
#pragma unroll
            for (int j = 0; j < kRegQuadWords; ++j) sh.p_q[j][np] = r_q[s].w[j];
          }
        }
      }
      L.sync();
      int32_t lmin2 = kMaxS32;
      for (int tb = 0; tb < c; tb += NL) {
        const int t = tb + L.lane;
        if (t < c) {
          const Edge e = W[k + t];
          const int32_t xt = e.x;
          int cnt = 0;
          for (int i = 0; i < m; ++i) {
            const int32_t xa = sh.ax[i];
            cnt += (xa <= x0 || (t >= 1 && xa < xt)) ? 1 : 0;
          }
          const int np = t + cnt;
          sh.p_idx[np] = k + t;
          sh.p_x[np] = e.x;
          sh.p_dx[np] = e.dx;
          sh.p_dy[np] = e.dy;
          sh.p_low[np] = e.lower_y;
          sh.p_wc[np] = MakeWc(e.winding, e.curve_count);
          if (kQ) {
            RegQuad q;
            q.load(e);
#pragma unroll
            for (int j = 0; j < kRegQuadWords; ++j) sh.p_q[j][np] = q.w[j];
          }
          if (e.lower_y > y) lmin2 = min_(lmin2, e.lower_y);
        }
      }
      L.sync();
      const int mm = m + c;
      bool cross2 = false;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int p = s * NL + L.lane;
        if (p < mm) {
          r_idx[s] = sh.p_idx[p];
          r_x[s] = sh.p_x[p];
          r_dx[s] = sh.p_dx[p];
          r_dy[s] = sh.p_dy[p];
          r_low[s] = sh.p_low[p];
          r_wc[s] = sh.p_wc[p];
          if (kQ) {
#pragma unroll
            for (int j = 0; j < kRegQuadWords; ++j) r_q[s].w[j] = sh.p_q[j][p];
          }
          if (r_idx[s] >= k && p > 0 &&
              wadd(sh.p_x[p - 1], sh.p_dx[p - 1]) > wadd(r_x[s], r_dx[s]))
            cross2 = true;
        }
      }
      L.sync();
      lmin2 = LaneMin(L, lmin2);
      nny = min_(nny, lmin2);
      if (L.ballot(cross2)) nny = min_(nny, y + (kFixed1 >> kAccuracy));
      m = mm;
      k += c;
    }
    if (k < n && W[k].upper_y > y) nny = min_(nny, W[k].upper_y);
  }
  RegBlitFlush(L, sh, sink, as, pend);
  return 1;
}

}  // namespace skc
