// The analytic-AA scanline sweep of one path (WalkEdges and its helpers,
// src/render/sw/sw_raster.cc:19-677), executed by one warp with the lanes
// working on different active edges and different coverage intervals.
//
// The reference walks a doubly linked list of edges one edge at a time.
// Its per-step effects are restated here in a form whose parts are
// independent per edge / per interval, with results identical to the
// sequential walk:
//   * winding and the interval pairing are a prefix scan over the list
//     order; every interval's trapezoid parameters come from the left and
//     right edges' x before the step, after GoY and after the quad-piece
//     update, exactly as the sequential loop reads them;
//   * the backward insertions that keep the list x-sorted leave the
//     surviving edges in a stable sort by their new x; check_intersection
//     compares each edge with the last processed survivor whose new x is
//     not greater than its own, i.e. its predecessor at insertion time;
//   * insert_new_edges is a merge: the first new edge goes after every
//     active edge with x <= its x, each later one after the previous new
//     edge and after the active edges with smaller x;
//   * SpanBuilder's saturating per-pixel sums are min(255, sum) of
//     non-negative alphas, so the row accumulator is a difference array of
//     int32 (range adds are O(1), lanes add atomically) saturated at flush.
// Spans of a row keep the reference's order: the direct spans of its
// intervals in list order, then the accumulated runs in x order.
#pragma once
#include "raster.cuh"

namespace skc {

// ---- warp-level helpers -----------------------------------------------------
SKC_HD int32_t LaneScanIncl(const Lanes& L, int32_t v) {
#ifdef SKC_WARP_LANES
  for (int o = 1; o < 32; o <<= 1) {
    int32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (L.lane >= o) v += t;
  }
#endif
  return v;
}
SKC_HD int32_t LaneBcast(const Lanes& L, int32_t v, int src) {
#ifdef SKC_WARP_LANES
  return __shfl_sync(0xffffffffu, v, src);
#else
  return v;
#endif
}
SKC_HD int32_t LaneMin(const Lanes& L, int32_t v) {
#ifdef SKC_WARP_LANES
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
#endif
  return v;
}
SKC_HD int32_t LaneMax(const Lanes& L, int32_t v) {
#ifdef SKC_WARP_LANES
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
#endif
  return v;
}
SKC_HD unsigned long long LaneSum64(const Lanes& L, unsigned long long v) {
#ifdef SKC_WARP_LANES
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
#endif
  return v;
}
SKC_HD void FlagError(uint32_t* err, uint32_t code) {
  if (!err) return;
#ifdef __CUDA_ARCH__
  atomicOr(err, code);
#else
  *err |= code;
#endif
}
// An add to the row accumulator, which the lanes of a warp share.
SKC_HD void AtomicAddI32(int32_t* p, int32_t v) {
#ifdef SKC_WARP_LANES
  atomicAdd(p, v);
#else
  *p += v;
#endif
}

// Runs of equal nonzero saturated sums of diff[lo, hi) (prefix sums,
// min 255), in increasing x; emit(start, width, alpha) is called
// warp-uniformly, one call per run (SpanBuilder::Flush, sw_raster.cc:103-136).
// Each lane takes V consecutive entries per chunk; every entry read is reset
// to zero, so the accumulator is clean for the next row except diff[hi].
template <typename F>
SKC_HD void DiffRuns(const Lanes& L, int32_t* diff, int lo, int hi, F&& emit) {
  constexpr int V = Lanes::n == 32 ? 4 : 1;
  int open_start = -1;
  int32_t open_v = 0;
  int32_t carry = 0;      // prefix sum before this chunk
  int32_t prev_sat = 0;   // saturated value of the entry before this chunk
  for (int base = lo; base < hi; base += Lanes::n * V) {
    const int i0 = base + L.lane * V;
    int32_t sat[V];
    int32_t run = 0;
#pragma unroll
    for (int j = 0; j < V; ++j) {
      int32_t d = 0;
      if (i0 + j < hi) {
        d = diff[i0 + j];
        diff[i0 + j] = 0;
      }
      run += d;
      sat[j] = run;
    }
    const int32_t incl = LaneScanIncl(L, run);
    const int32_t pre = incl - run + carry;
#pragma unroll
    for (int j = 0; j < V; ++j) {
      const int32_t v = sat[j] + pre;
      sat[j] = v > 255 ? 255 : v;
    }
    int32_t before = LaneBcast(L, sat[V - 1], L.lane > 0 ? L.lane - 1 : 0);
    if (L.lane == 0) before = prev_sat;
    unsigned bits = 0;
#pragma unroll
    for (int j = 0; j < V; ++j) {
      const int32_t b = j == 0 ? before : sat[j - 1];
      if (i0 + j < hi && sat[j] != b) bits |= 1u << j;
    }
    unsigned mask = L.ballot(bits != 0);
    while (mask) {
      const int src = Lanes::ffs(mask) - 1;
      mask &= mask - 1;
      const unsigned sb = (unsigned)LaneBcast(L, (int32_t)bits, src);
#pragma unroll
      for (int j = 0; j < V; ++j) {
        const int32_t bv = LaneBcast(L, sat[j], src);
        if (sb & (1u << j)) {
          const int pos = base + src * V + j;
          if (open_start >= 0) {
            emit(open_start, pos - open_start, (uint8_t)open_v);
            open_start = -1;
          }
          if (bv != 0) {
            open_start = pos;
            open_v = bv;
          }
        }
      }
    }
    carry += LaneBcast(L, incl, Lanes::n - 1);
    prev_sat = LaneBcast(L, sat[V - 1], Lanes::n - 1);
  }
  if (open_start >= 0) emit(open_start, hi - open_start, (uint8_t)open_v);
}

// ---- one coverage interval of a step, on one lane ----------------------------
// blit_trapezoid_row (sw_raster.cc:457-544) with its helpers
// (blit_single_alpha, blit_two_alphas, blit_full_alpha, blit_aaa_trapezoid_row,
// :281-455).  Out::real(x, len, a) receives direct spans in order,
// Out::acc(x, len, a) accumulator adds.
template <typename Out>
SKC_HD void AaaRow(Out& out, Fixed ul, Fixed ur, Fixed ll, Fixed lr, Fixed lDY, Fixed rDY,
                   uint8_t full, bool real) {
  int L0 = FixedFloorToInt(ul), R = FixedCeilToInt(lr);
  int len = R - L0;
  if (len == 1) {
    uint8_t a = trapezoid_to_alpha(ur - ul, lr - ll);
    if (real) out.real(L0, 1, a);
    else out.acc(L0, 1, partial_alpha_a(a, full));
    return;
  }
  int uL = FixedFloorToInt(ul), lL = FixedCeilToInt(ll);
  int uR = FixedFloorToInt(ur), lR = FixedCeilToInt(lr);
  bool two_left = uL + 2 == lL, two_right = uR + 2 == lR;
  uint8_t la1 = 0, la2 = 0, ra1 = 0, ra2 = 0;
  if (two_left) {
    Fixed first = IntToFixed(uL) + kFixed1 - ul;
    Fixed second = ll - ul - first;
    la1 = (uint8_t)(full - partial_triangle_to_alpha(first, lDY));
    la2 = partial_triangle_to_alpha(second, lDY);
  }
  if (two_right) {
    Fixed first = IntToFixed(uR) + kFixed1 - ur;
    Fixed second = lr - ur - first;
    ra1 = partial_triangle_to_alpha(first, rDY);
    ra2 = (uint8_t)(full - partial_triangle_to_alpha(second, rDY));
  }
  for (int i = 0; i < len; ++i) {
    int px = L0 + i;
    uint8_t a = full;
    if (two_left) {
      if (i == 0) a = a > la1 ? (uint8_t)(a - la1) : 0;
      if (i == 1) a = a > la2 ? (uint8_t)(a - la2) : 0;
    } else if (px >= uL && px < lL) {
      uint8_t t = triangle_entry(true, ul - IntToFixed(uL), ll - IntToFixed(uL), lDY, full, px - uL);
      a = a > t ? (uint8_t)(a - t) : 0;
    }
    if (two_right) {
      if (i == len - 2) a = a > ra1 ? (uint8_t)(a - ra1) : 0;
      if (i == len - 1) a = a > ra2 ? (uint8_t)(a - ra2) : 0;
    } else if (px >= uR && px < lR) {
      uint8_t t = triangle_entry(false, ur - IntToFixed(uR), lr - IntToFixed(uR), rDY, full, px - uR);
      a = a > t ? (uint8_t)(a - t) : 0;
    }
    if (real) out.real(px, 1, a);
    else out.acc(px, 1, a);
  }
}

template <typename Out>
SKC_HD void TrapezoidRow(Out& out, Fixed ul, Fixed ur, Fixed ll, Fixed lr, Fixed lDY, Fixed rDY,
                         uint8_t full, bool no_real) {
  if (ul > ur) return;
  if (ll > lr) ll = lr = approximate_intersection(ul, ll, ur, lr);
  if (ul == ur && ll == lr) return;
  if (ul > ll) swap_(ul, ll);
  if (ur > lr) swap_(ur, lr);
  const bool real = full == 0xFF && !no_real;
  Fixed joinLeft = FixedCeilToFixed(ll);
  Fixed joinRite = FixedFloorToFixed(ur);
  if (joinLeft <= joinRite) {
    if (ul < joinLeft) {
      int len = FixedCeilToInt(joinLeft - ul);
      if (len == 1) {
        uint8_t a = trapezoid_to_alpha(joinLeft - ul, joinLeft - ll);
        if (real) out.real(ul >> 16, 1, a);
        else out.acc(ul >> 16, 1, partial_alpha_a(a, full));
      } else if (len == 2) {
        Fixed first = joinLeft - kFixed1 - ul;
        Fixed second = ll - ul - first;
        uint8_t a1 = partial_triangle_to_alpha(first, lDY);
        uint8_t a2 = (uint8_t)(full - partial_triangle_to_alpha(second, lDY));
        if (real) {
          out.real(ul >> 16, 1, a1);
          out.real((ul >> 16) + 1, 1, a2);
        } else {
          out.acc(ul >> 16, 1, a1);
          out.acc((ul >> 16) + 1, 1, a2);
        }
      } else {
        AaaRow(out, ul, joinLeft, ll, joinLeft, lDY, kMaxS32, full, real);
      }
    }
    if (joinLeft < joinRite) {
      int x = FixedFloorToInt(joinLeft), len = FixedFloorToInt(joinRite - joinLeft);
      if (real) out.real(x, len, full);
      else out.acc(x, len, full);
    }
    if (lr > joinRite) {
      int len = FixedCeilToInt(lr - joinRite);
      if (len == 1) {
        uint8_t a = trapezoid_to_alpha(ur - joinRite, lr - joinRite);
        if (real) out.real(joinRite >> 16, 1, a);
        else out.acc(joinRite >> 16, 1, partial_alpha_a(a, full));
      } else if (len == 2) {
        Fixed first = joinRite + kFixed1 - ur;
        Fixed second = lr - ur - first;
        uint8_t a1 = (uint8_t)(full - partial_triangle_to_alpha(first, rDY));
        uint8_t a2 = partial_triangle_to_alpha(second, rDY);
        if (real) {
          out.real(joinRite >> 16, 1, a1);
          out.real((joinRite >> 16) + 1, 1, a2);
        } else {
          out.acc(joinRite >> 16, 1, a1);
          out.acc((joinRite >> 16) + 1, 1, a2);
        }
      } else {
        AaaRow(out, joinRite, ur, joinRite, lr, kMaxS32, rDY, full, real);
      }
    }
  } else {
    AaaRow(out, ul, ur, ll, lr, lDY, rDY, full, real);
  }
}

// The same row in indexed form, for span-parallel blits: TrapPrepare does
// blit_trapezoid_row's set-up (false: the row emits nothing), TrapCount the
// number of out.real / out.acc calls it makes, TrapSpan the k-th of them
// (x, len, alpha; direct when `real`, an accumulator add otherwise), in the
// order TrapezoidRow makes them.
struct TrapRow {
  Fixed ul, ur, ll, lr, lDY, rDY;
  uint8_t full;
  bool real;
};

SKC_HD bool TrapPrepare(TrapRow& t, Fixed ul, Fixed ur, Fixed ll, Fixed lr, Fixed lDY, Fixed rDY,
                        uint8_t full, bool no_real) {
  if (ul > ur) return false;
  if (ll > lr) ll = lr = approximate_intersection(ul, ll, ur, lr);
  if (ul == ur && ll == lr) return false;
  if (ul > ll) swap_(ul, ll);
  if (ur > lr) swap_(ur, lr);
  t.ul = ul;
  t.ur = ur;
  t.ll = ll;
  t.lr = lr;
  t.lDY = lDY;
  t.rDY = rDY;
  t.full = full;
  t.real = full == 0xFF && !no_real;
  return true;
}

SKC_HD int AaaCount(Fixed ul, Fixed lr) {
  const int len = FixedCeilToInt(lr) - FixedFloorToInt(ul);
  return len > 0 ? len : 0;
}

SKC_HD int TrapCount(const TrapRow& t) {
  const Fixed joinLeft = FixedCeilToFixed(t.ll);
  const Fixed joinRite = FixedFloorToFixed(t.ur);
  if (joinLeft > joinRite) return AaaCount(t.ul, t.lr);
  int c = 0;
  if (t.ul < joinLeft) {
    const int len = FixedCeilToInt(joinLeft - t.ul);
    c += len <= 2 ? len : AaaCount(t.ul, joinLeft);
  }
  if (joinLeft < joinRite) c += 1;
  if (t.lr > joinRite) {
    const int len = FixedCeilToInt(t.lr - joinRite);
    c += len <= 2 ? len : AaaCount(joinRite, t.lr);
  }
  return c;
}

// Pixel i of blit_aaa_trapezoid_row (AaaRow above).
SKC_HD void AaaSpan(Fixed ul, Fixed ur, Fixed ll, Fixed lr, Fixed lDY, Fixed rDY, uint8_t full,
                    bool real, int i, int& x, int& len, uint8_t& a) {
  const int L0 = FixedFloorToInt(ul), R = FixedCeilToInt(lr);
  len = 1;
  if (R - L0 == 1) {
    const uint8_t t = trapezoid_to_alpha(ur - ul, lr - ll);
    x = L0;
    a = real ? t : partial_alpha_a(t, full);
    return;
  }
  const int uL = FixedFloorToInt(ul), lL = FixedCeilToInt(ll);
  const int uR = FixedFloorToInt(ur), lR = FixedCeilToInt(lr);
  const bool two_left = uL + 2 == lL, two_right = uR + 2 == lR;
  const int px = L0 + i;
  const int n = R - L0;
  uint8_t v = full;
  if (two_left) {
    if (i <= 1) {
      const Fixed first = IntToFixed(uL) + kFixed1 - ul;
      const uint8_t la = i == 0 ? (uint8_t)(full - partial_triangle_to_alpha(first, lDY))
                                : partial_triangle_to_alpha(ll - ul - first, lDY);
      v = v > la ? (uint8_t)(v - la) : 0;
    }
  } else if (px >= uL && px < lL) {
    const uint8_t t = triangle_entry(true, ul - IntToFixed(uL), ll - IntToFixed(uL), lDY, full, px - uL);
    v = v > t ? (uint8_t)(v - t) : 0;
  }
  if (two_right) {
    if (i >= n - 2) {
      const Fixed first = IntToFixed(uR) + kFixed1 - ur;
      const uint8_t ra = i == n - 2 ? partial_triangle_to_alpha(first, rDY)
                                    : (uint8_t)(full - partial_triangle_to_alpha(lr - ur - first, rDY));
      v = v > ra ? (uint8_t)(v - ra) : 0;
    }
  } else if (px >= uR && px < lR) {
    const uint8_t t = triangle_entry(false, ur - IntToFixed(uR), lr - IntToFixed(uR), rDY, full, px - uR);
    v = v > t ? (uint8_t)(v - t) : 0;
  }
  x = px;
  a = v;
}

SKC_HD void TrapSpan(const TrapRow& t, int k, int& x, int& len, uint8_t& a) {
  const Fixed joinLeft = FixedCeilToFixed(t.ll);
  const Fixed joinRite = FixedFloorToFixed(t.ur);
  if (joinLeft > joinRite) {
    AaaSpan(t.ul, t.ur, t.ll, t.lr, t.lDY, t.rDY, t.full, t.real, k, x, len, a);
    return;
  }
  if (t.ul < joinLeft) {
    const int n = FixedCeilToInt(joinLeft - t.ul);
    if (n == 1) {
      if (k == 0) {
        const uint8_t v = trapezoid_to_alpha(joinLeft - t.ul, joinLeft - t.ll);
        x = t.ul >> 16;
        len = 1;
        a = t.real ? v : partial_alpha_a(v, t.full);
        return;
      }
      k -= 1;
    } else if (n == 2) {
      if (k < 2) {
        const Fixed first = joinLeft - kFixed1 - t.ul;
        x = (t.ul >> 16) + k;
        len = 1;
        a = k == 0 ? partial_triangle_to_alpha(first, t.lDY)
                   : (uint8_t)(t.full - partial_triangle_to_alpha(t.ll - t.ul - first, t.lDY));
        return;
      }
      k -= 2;
    } else {
      const int c = AaaCount(t.ul, joinLeft);
      if (k < c) {
        AaaSpan(t.ul, joinLeft, t.ll, joinLeft, t.lDY, kMaxS32, t.full, t.real, k, x, len, a);
        return;
      }
      k -= c;
    }
  }
  if (joinLeft < joinRite) {
    if (k == 0) {
      x = FixedFloorToInt(joinLeft);
      len = FixedFloorToInt(joinRite - joinLeft);
      a = t.full;
      return;
    }
    k -= 1;
  }
  const int n = FixedCeilToInt(t.lr - joinRite);
  if (n == 1) {
    const uint8_t v = trapezoid_to_alpha(t.ur - joinRite, t.lr - joinRite);
    x = joinRite >> 16;
    len = 1;
    a = t.real ? v : partial_alpha_a(v, t.full);
  } else if (n == 2) {
    const Fixed first = joinRite + kFixed1 - t.ur;
    x = (joinRite >> 16) + k;
    len = 1;
    a = k == 0 ? (uint8_t)(t.full - partial_triangle_to_alpha(first, t.rDY))
               : partial_triangle_to_alpha(t.lr - t.ur - first, t.rDY);
  } else {
    AaaSpan(joinRite, t.ur, joinRite, t.lr, kMaxS32, t.rDY, t.full, t.real, k, x, len, a);
  }
}

// Per-pass sweep memory (capacity n edges; diff holds acc_width + 1).
struct SweepMem {
  Edge* W;            // edges in sorted order; pending edges are W[k..n)
  int32_t* act;       // active list (edge indices), list order
  int32_t* act2;      // next active list
  int32_t* xo;        // per list position: x before the step
  int32_t* xg;        //   x after GoY
  int32_t* xf;        //   x after the quad-piece update
  int32_t* dxo;       //   dx before the step
  int32_t* dyo;       //   dy before the step
  int32_t* dxf;       //   dx after the update
  int32_t* lowf;      //   lower_y after the update
  uint8_t* flags;     //   1 left, 2 right, 4 survives
  int32_t* ia;        // interval k: left position
  int32_t* ib;        //   right position
  int32_t* diff;      // row accumulator as a difference array
};
// Layout of the per-pass sweep memory; with base == nullptr only the size
// is computed, so SweepMemBytes and SweepMemAt can never disagree.
SKC_HD uint64_t SweepMemLayout(uint8_t* base, int n, int acc_width, SweepMem* m) {
  uint64_t o = 0;
  auto take = [&](uint64_t bytes) {
    uint8_t* p = base ? base + o : nullptr;
    o = (o + bytes + 15) & ~uint64_t(15);
    return p;
  };
  SweepMem t;
  t.W = (Edge*)take((uint64_t)n * sizeof(Edge));
  t.act = (int32_t*)take(4ull * n);
  t.act2 = (int32_t*)take(4ull * n);
  t.xo = (int32_t*)take(4ull * n);
  t.xg = (int32_t*)take(4ull * n);
  t.xf = (int32_t*)take(4ull * n);
  t.dxo = (int32_t*)take(4ull * n);
  t.dyo = (int32_t*)take(4ull * n);
  t.dxf = (int32_t*)take(4ull * n);
  t.lowf = (int32_t*)take(4ull * n);
  t.ia = (int32_t*)take(4ull * n);
  t.ib = (int32_t*)take(4ull * n);
  t.flags = (uint8_t*)take((uint64_t)n);
  t.diff = (int32_t*)take(4ull * ((uint64_t)acc_width + 1));
  if (m) *m = t;
  return o;
}
SKC_HD uint64_t SweepMemBytes(int n, int acc_width) {
  return SweepMemLayout(nullptr, n, acc_width, nullptr);
}
SKC_HD SweepMem SweepMemAt(uint8_t* base, int n, int acc_width) {
  SweepMem m;
  SweepMemLayout(base, n, acc_width, &m);
  return m;
}

template <typename Sink>
struct LaneSweep {
  Lanes L;
  SweepMem M;
  int n;
  uint32_t* err;      // self-check flag: an edge index outside [0, n)
  Sink* sink;
  int acc_left, acc_width;
  int acc_y;
  int touch_lo, touch_hi;
  float scan_top;

  // -- accumulator
  SKC_HD void flush_acc() {
    if (acc_y == kNaN32) return;
    if (touch_lo <= touch_hi) {
      sink->acc_row(L, acc_y, M.diff, acc_left, touch_lo, touch_hi);
      L.sync();
      for (int i = touch_lo + L.lane; i <= touch_hi; i += Lanes::n) M.diff[i] = 0;
      L.sync();
    }
    touch_lo = 0x7fffffff;
    touch_hi = -1;
  }
  SKC_HD void flush_if_need(int row) {
    if (acc_y == row) return;
    if (acc_y != kNaN32) flush_acc();
    acc_y = row;
  }

  // Lane-local output of one interval's trapezoid row.
  struct Out {
    LaneSweep* s;
    int y;
    bool count_only;    // count kept direct spans (and do the acc adds)
    bool do_acc;
    uint32_t kept;
    unsigned long long frags;
    uint2* write;       // write pass: next slot of this lane
    int lo, hi;         // accumulator range touched by this lane
    SKC_HD void real(int x, int len, uint8_t a) {
      if (!s->sink->keep(x, y, len, a)) return;
      kept++;
      frags += (unsigned)len;
      if (write) *write++ = s->sink->pack(x, len, a);
    }
    SKC_HD void acc(int x, int len, uint8_t a) {
      if (!do_acc) return;
      int o0 = x - s->acc_left, o1 = o0 + len;
      o0 = max_(o0, 0);
      o1 = min_(o1, s->acc_width);
      if (o0 >= o1 || a == 0) {
        if (o0 < o1) {
          lo = min_(lo, o0);
          hi = max_(hi, o1);
        }
        return;
      }
      AtomicAddI32(&s->M.diff[o0], (int32_t)a);
      AtomicAddI32(&s->M.diff[o1], -(int32_t)a);
      lo = min_(lo, o0);
      hi = max_(hi, o1);
    }
  };

  // Blit intervals [0, K) of a step (plus, when trailing_a >= 0, the
  // interval left open by the last edge, with its precomputed no_real).
  SKC_HDN void blit_intervals(int y, Fixed next_y, int K, int m, int k, uint8_t full,
                              Fixed left_clip, Fixed right_clip, int trailing_a, bool trailing_nr) {
    const int total = K + (trailing_a >= 0 ? 1 : 0);
    if (total == 0) return;
    if (y < scan_top) return;
    flush_if_need(y);
    sink->row_begin(L, y);
    uint32_t run = 0;  // kept direct spans so far in this step
    unsigned long long frags = 0;
    int lo = 0x7fffffff, hi = -1;
    for (int kb = 0; kb < total; kb += Lanes::n) {
      int ki = kb + L.lane;
      bool valid = ki < total;
      Fixed ul = 0, ur = 0, ll = 0, lr = 0, lDY = 0, rDY = 0;
      bool nr = false;
      if (valid) {
        if (ki < K) {
          int a = M.ia[ki], b = M.ib[ki];
          ul = max_(M.xo[a], left_clip);
          lDY = M.dyo[a];
          ur = min_(right_clip, M.xo[b]);
          ll = max_(left_clip, M.xf[a]);
          lr = min_(right_clip, M.xg[b]);
          rDY = M.dyo[b];
          int prev_right;
          if (ki == 0) {
            prev_right = FixedFloorToInt(left_clip);
          } else {
            int pb = M.ib[ki - 1];
            prev_right = FixedCeilToInt(max_(min_(right_clip, M.xo[pb]), M.xg[pb]));
          }
          bool tc = prev_right > FixedFloorToInt(ul) || prev_right > FixedFloorToInt(M.xf[a]);
          if (!tc) {
            // edges_too_close(right edge, its successor before the step)
            int32_t nxo, ndx;
            Fixed nup;
            if (b + 1 < m) {
              nxo = M.xo[b + 1];
              ndx = M.dxo[b + 1];
              nup = kMinS32;  // active: upper_y <= y < next_y
            } else if (k < n) {
              nxo = M.W[k].x;
              ndx = M.W[k].dx;
              nup = M.W[k].upper_y;
            } else {
              nxo = kMaxS32;
              ndx = 0;
              nup = kMaxS32;
            }
            tc = nup < next_y && wadd(M.xg[b], kFixed1) >= wsub(nxo, iabs_(ndx));
          }
          nr = tc;
        } else {
          int a = trailing_a;
          ul = max_(M.xo[a], left_clip);
          lDY = M.dyo[a];
          ur = right_clip;
          ll = max_(left_clip, M.xf[a]);
          lr = right_clip;
          rDY = 0;
          nr = trailing_nr;
        }
      }
      Out o;
      o.s = this;
      o.y = y;
      o.count_only = true;
      o.do_acc = true;
      o.kept = 0;
      o.frags = 0;
      o.write = nullptr;
      o.lo = 0x7fffffff;
      o.hi = -1;
      if (valid) TrapezoidRow(o, ul, ur, ll, lr, lDY, rDY, full, nr);
      lo = min_(lo, o.lo);
      hi = max_(hi, o.hi);
      const int32_t incl = LaneScanIncl(L, (int32_t)o.kept);
      const uint32_t chunk_total = (uint32_t)LaneBcast(L, incl, Lanes::n - 1);
      if (chunk_total) {
        const uint64_t at = sink->reserve(L, run, chunk_total);
        uint2* dst = sink->span_ptr(at + run + (uint32_t)(incl - (int32_t)o.kept));
        if (valid && o.kept && dst) {
          Out w = o;
          w.do_acc = false;
          w.kept = 0;
          w.frags = 0;
          w.write = dst;
          TrapezoidRow(w, ul, ur, ll, lr, lDY, rDY, full, nr);
        }
        L.sync();
      }
      run += chunk_total;
      frags += o.frags;
    }
    lo = LaneMin(L, lo);
    hi = LaneMax(L, hi);
    if (lo <= hi) {
      touch_lo = min_(touch_lo, lo);
      touch_hi = max_(touch_hi, hi);
    }
    sink->commit(L, run, frags);  // this lane's share
    L.sync();
  }

  // WalkEdges (sw_raster.cc:546-677)
  SKC_HDN void walk(bool even_odd, int start_y, int stop_y, Fixed left_clip, Fixed right_clip) {
    Edge* W = M.W;
    const int winding_mask = even_odd ? 1 : -1;
    Fixed y = max_(W[0].upper_y, IntToFixed(start_y));
    // initial activation: edges with upper_y <= y, in their sorted order
    int k = 0;
    Fixed nny = kMaxS32;
    {
      int32_t lmin = kMaxS32;
      for (int base = 0; base < n; base += Lanes::n) {
        int i = base + L.lane;
        bool act = i < n && W[i].upper_y <= y;
        unsigned mask = L.ballot(act);
        if (act) {
          Edge e = W[i];
          GoY(&e, y);
          W[i] = e;
          M.act[i] = i;
          if (e.lower_y > y) lmin = min_(lmin, e.lower_y);
        }
        k += Lanes::popc(mask);
        if (mask != (Lanes::n == 32 ? 0xffffffffu : 1u)) break;
      }
      lmin = LaneMin(L, lmin);
      nny = min_(nny, lmin);
      if (k < n && W[k].upper_y > y) nny = min_(nny, W[k].upper_y);
    }
    int m = k;
    L.sync();
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

      // ---- A: advance every active edge
      int32_t wcarry = 0;
      int nl = 0, nr = 0;
      for (int base = 0; base < m; base += Lanes::n) {
        int j = base + L.lane;
        bool valid = j < m;
        Edge e;
        int32_t wv = 0;
        if (valid) {
          int32_t idx = M.act[j];
          if ((unsigned)idx >= (unsigned)n) {  // self-check, never expected
            FlagError(err, 1);
            idx = 0;
          }
          e = W[idx];
          wv = e.winding;
        }
        int32_t incl = LaneScanIncl(L, wv) + wcarry;
        int32_t excl = incl - wv;
        bool in = (incl & winding_mask) != 0;
        bool pin = (excl & winding_mask) != 0;
        bool is_left = valid && in && !pin;
        bool is_right = valid && !in && pin;
        unsigned lm = L.ballot(is_left), rm = L.ballot(is_right);
        if (valid) {
          int32_t xo = e.x, dxo = e.dx, dyo = e.dy;
          GoYShift(&e, next_y, y_shift);
          int32_t xg = e.x;
          while (e.lower_y <= next_y) {
            if (e.curve_count > 0) {
              e.snapped_x = e.x;  // KeepContinuous (sw_edge.cc:294-297)
              e.snapped_y = e.y;
              if (!UpdateQuad(&e)) break;
            } else {
              break;
            }
          }
          bool surv = e.lower_y > next_y;
          int32_t widx = M.act[j];
          if ((unsigned)widx < (unsigned)n) W[widx] = e;
          M.xo[j] = xo;
          M.xg[j] = xg;
          M.xf[j] = e.x;
          M.dxo[j] = dxo;
          M.dyo[j] = dyo;
          M.dxf[j] = e.dx;
          M.lowf[j] = e.lower_y;
          M.flags[j] = (uint8_t)((is_left ? 1 : 0) | (is_right ? 2 : 0) | (surv ? 4 : 0));
          if (is_left) M.ia[nl + Lanes::popc(lm & L.lt_mask())] = j;
          if (is_right) M.ib[nr + Lanes::popc(rm & L.lt_mask())] = j;
        }
        nl += Lanes::popc(lm);
        nr += Lanes::popc(rm);
        wcarry = LaneBcast(L, incl, min_(Lanes::n, m - base) - 1);
      }
      const bool final_in = (wcarry & winding_mask) != 0;
      L.sync();

      // ---- B: coverage of the step's intervals, in list order
      blit_intervals(y >> 16, next_y, nr, m, k, full, left_clip, right_clip, -1, false);

      // ---- C: survivors in stable order of their new x; intersections
      int m2 = 0;
      bool cross = false;
      int32_t lmin = kMaxS32;
      for (int base = 0; base < m; base += Lanes::n) {
        int j = base + L.lane;
        bool valid = j < m;
        bool surv = valid && (M.flags[j] & 4);
        int rank = 0;
        int best = -1;
        int32_t bestx = 0;
        int32_t xj = valid ? M.xf[j] : 0;
        for (int i = 0; i < m; ++i) {
          if (!(M.flags[i] & 4)) continue;
          int32_t xi = M.xf[i];
          if (xi < xj || (xi == xj && i < j)) rank++;
          if (i < j && xi <= xj && (best < 0 || xi >= bestx)) {
            best = i;
            bestx = xi;
          }
        }
        if (surv) {
          M.act2[rank] = M.act[j];
          lmin = min_(lmin, M.lowf[j]);
          if (best >= 0 && wadd(M.xf[best], M.dxf[best]) > wadd(xj, M.dxf[j])) cross = true;
        }
        m2 += Lanes::popc(L.ballot(surv));
      }
      lmin = LaneMin(L, lmin);
      nny = min_(nny, lmin);
      if (L.ballot(cross)) nny = min_(nny, next_y + (kFixed1 >> kAccuracy));
      L.sync();

      // ---- trailing interval (right edge culled away), after the reorder
      if (final_in) {
        int a = M.ia[nr];
        // left edge's predecessor now: its new predecessor if it survived,
        // else the last processed survivor when it was removed
        int pred = -1;
        int32_t pred_x = left_clip;
        if (M.flags[a] & 4) {
          int32_t xa = M.xf[a];
          int best = -1;
          int32_t bx = 0;
          for (int i = 0; i < m; ++i) {
            if (!(M.flags[i] & 4) || i == a) continue;
            int32_t xi = M.xf[i];
            bool before = xi < xa || (xi == xa && i < a);
            if (before && (best < 0 || xi > bx || (xi == bx && i > best))) {
              best = i;
              bx = xi;
            }
          }
          pred = best;
          if (best >= 0) pred_x = bx;
        } else {
          int best = -1;
          int32_t bx = 0;
          for (int i = 0; i < a; ++i) {
            if (!(M.flags[i] & 4)) continue;
            int32_t xi = M.xf[i];
            if (best < 0 || xi >= bx) {
              best = i;
              bx = xi;
            }
          }
          pred = best;
          if (best >= 0) pred_x = bx;
        }
        (void)pred;
        bool tc = wadd(pred_x, kFixed1) >= wsub(M.xf[a], iabs_(M.dxf[a]));
        blit_intervals(y >> 16, next_y, 0, m, k, full, left_clip, right_clip, a, full == 0xFF && tc);
      }

      // swap lists
      {
        int32_t* t = M.act;
        M.act = M.act2;
        M.act2 = t;
      }
      m = m2;
      y = next_y;
      if (y >= IntToFixed(stop_y)) break;

      // ---- D: insert_new_edges (sw_raster.cc:207-247)
      if (k < n && W[k].upper_y <= y) {
        int c = 0;
        for (int base = k; base < n; base += Lanes::n) {
          int i = base + L.lane;
          unsigned mask = L.ballot(i < n && W[i].upper_y <= y);
          c += Lanes::popc(mask);
          if (mask != (Lanes::n == 32 ? 0xffffffffu : 1u)) break;
        }
        const int32_t x0 = W[k].x;
        // actives
        for (int base = 0; base < m; base += Lanes::n) {
          int i = base + L.lane;
          if (i < m) {
            int32_t ai = M.act[i];
            if ((unsigned)ai >= (unsigned)n) {
              FlagError(err, 1);
              ai = 0;
            }
            int32_t xa = W[ai].x;
            int before = 0;
            if (xa > x0) {
              before = 1;
              for (int t = 1; t < c; ++t) before += W[k + t].x <= xa ? 1 : 0;
            }
            M.act2[i + before] = M.act[i];
          }
        }
        // new edges
        for (int base = 0; base < c; base += Lanes::n) {
          int t = base + L.lane;
          if (t < c) {
            int32_t xt = W[k + t].x;
            int cnt = 0;
            for (int i = 0; i < m; ++i) {
              int32_t ai = M.act[i];
              int32_t xa = (unsigned)ai < (unsigned)n ? W[ai].x : 0;
              cnt += (xa <= x0 || (t >= 1 && xa < xt)) ? 1 : 0;
            }
            M.act2[t + cnt] = k + t;
            M.xo[t] = t + cnt;  // position of new edge t (scratch)
          }
        }
        L.sync();
        int32_t lmin2 = kMaxS32;
        bool cross2 = false;
        for (int base = 0; base < c; base += Lanes::n) {
          int t = base + L.lane;
          if (t < c) {
            const Edge& e = W[k + t];
            int pos = M.xo[t];
            if (pos > 0) {
              int32_t pi = M.act2[pos - 1];
              if ((unsigned)pi >= (unsigned)n) {
                FlagError(err, 1);
                pi = 0;
              }
              const Edge& p = W[pi];
              if (wadd(p.x, p.dx) > wadd(e.x, e.dx)) cross2 = true;
            }
            if (e.lower_y > y) lmin2 = min_(lmin2, e.lower_y);
          }
        }
        lmin2 = LaneMin(L, lmin2);
        nny = min_(nny, lmin2);
        if (L.ballot(cross2)) nny = min_(nny, y + (kFixed1 >> kAccuracy));
        int32_t* t = M.act;
        M.act = M.act2;
        M.act2 = t;
        m += c;
        k += c;
        L.sync();
      }
      if (k < n && W[k].upper_y > y) nny = min_(nny, W[k].upper_y);
    }
  }
};

}  // namespace skc
