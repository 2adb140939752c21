// Per-thread bodies of the raster kernels, host+device so the pipeline can
// also be executed on the CPU by tests (the GPU runs them through the
// __global__ wrappers in kernels.cu).
#pragma once
#include "kernels.cuh"
#include "stroke.cuh"
#include "regsweep.cuh"

namespace skc {

// ---------------------------------------------------------------------------
// geometry: Path -> QuadPath (-> stroke -> QuadPath) -> edges -> introsort
// ---------------------------------------------------------------------------
SKC_HDN void GeometryPass(const DevBatch& b, uint32_t p) {
  const PassDesc pd = b.passes[p];
  const DrawDesc dd = b.draws[pd.draw];
  PassGeom g;
  g.status = 0;
  g.n_edges = 0;
  g.start_y = g.stop_y = 0;
  g.left_bound = g.right_bound = 0;
  g.acc_left = g.acc_width = 0;
  g.scan_top = 0;
  g.row0 = g.row1 = 0;
  g.raw_spans = (pd.flags & kPassRawSpans) != 0 ? 1 : 0;
  for (int k = 0; k < 13; ++k) g.need[k] = 0;
  g.max_active = 0;

  SliceLayout L;
  L.compute(pd.cap, sizeof(Edge));
  uint8_t* base = b.scratch + pd.slice_off;
  PathView src;
  src.verbs = b.verbs + dd.v0;
  src.pts = b.pts + dd.p0;
  src.w = b.weights + dd.w0;
  src.nv = (int)dd.nv;
  src.np = (int)dd.np;
  src.nw = (int)dd.nw;

  DPath q1;
  q1.init(base + L.off[0], pd.cap[0], (P*)(base + L.off[1]), pd.cap[1], (float*)(base + L.off[2]),
          pd.cap[2]);
  QuadPath(src, &q1);
  g.need[0] = q1.nv;
  g.need[1] = q1.np;
  g.need[2] = q1.nw;
  if (q1.overflow()) {
    g.status = 1;
    b.geom[p] = g;
    return;
  }
  PathView quad = q1.view();
  DPath q2;
  if (pd.flags & kPassStroke) {
    DPath outer, inner;
    outer.init(base + L.off[3], pd.cap[3], (P*)(base + L.off[4]), pd.cap[4],
               (float*)(base + L.off[5]), pd.cap[5]);
    inner.init(base + L.off[6], pd.cap[6], (P*)(base + L.off[7]), pd.cap[7],
               (float*)(base + L.off[8]), pd.cap[8]);
    int imax[3];
    StrokePath(q1.view(), pd.stroke_width, pd.miter, (int)(pd.cap_join & 0xFF),
               (int)(pd.cap_join >> 8), &outer, &inner, imax);
    g.need[3] = outer.nv;
    g.need[4] = outer.np;
    g.need[5] = outer.nw;
    g.need[6] = imax[0];
    g.need[7] = imax[1];
    g.need[8] = imax[2];
    if (outer.overflow() || imax[0] > pd.cap[6] || imax[1] > pd.cap[7] || imax[2] > pd.cap[8]) {
      g.status = 1;
      b.geom[p] = g;
      return;
    }
    q2.init(base + L.off[9], pd.cap[9], (P*)(base + L.off[10]), pd.cap[10],
            (float*)(base + L.off[11]), pd.cap[11]);
    QuadPath(outer.view(), &q2);
    g.need[9] = q2.nv;
    g.need[10] = q2.np;
    g.need[11] = q2.nw;
    if (q2.overflow()) {
      g.status = 1;
      b.geom[p] = g;
      return;
    }
    quad = q2.view();
  }
  const Xform xf = PassXform(pd);
  RasterBounds rb = pd.clipped
                        ? ComputeBounds(quad, xf, pd.clip[0], pd.clip[1], pd.clip[2], pd.clip[3])
                        : ComputeBounds(quad, xf);
  if (rb.empty) {
    b.geom[p] = g;
    return;
  }
  Edge* edges = (Edge*)(base + L.off[12]);
  int n = BuildEdges(quad, xf, rb.st, rb.sb, edges, pd.cap[12]);
  g.need[12] = n;
  if (n > pd.cap[12]) {
    g.status = 1;
    b.geom[p] = g;
    return;
  }
  if (n == 0) {
    b.geom[p] = g;
    return;
  }
  int32_t* idx = (int32_t*)(base + L.off[14]);
  for (int i = 0; i < n; ++i) idx[i] = i;
  EdgeLess less;
  less.e = edges;
  introsort(idx, n, less);
  Edge* S = (Edge*)(base + L.off[13]);
  for (int i = 0; i < n; ++i) {
    S[i] = edges[idx[i]];
    S[i].prev = i == 0 ? n : i - 1;
    S[i].next = i + 1 == n ? n + 1 : i + 1;
  }
  // ProcessEdges sentinels (sw_raster.cc:706-729)
  Edge h;
  h.prev = -1;
  h.next = 0;
  h.upper_y = h.lower_y = kMinS32;
  h.x = kMinS32;
  h.dx = 0;
  h.dy = kMaxS32;
  h.upper_x = kMinS32;
  h.y = 0;
  h.curve_count = 0;
  h.curve_shift = 0;
  h.winding = 0;
  Edge tl = h;
  tl.prev = n - 1;
  tl.next = -1;
  tl.upper_y = tl.lower_y = kMaxS32;
  tl.x = kMaxS32;
  tl.upper_x = kMaxS32;
  S[n] = h;
  S[n + 1] = tl;
  // Bound of the sweep's active list: an edge joins it at upper_y and
  // leaves after its last piece, so the list never holds more edges than
  // the largest overlap of the [upper_y, last y) ranges.
  {
    int32_t* low = idx;  // free after the copy above
    for (int i = 0; i < n; ++i)
      low[i] = S[i].curve_count != 0 ? max_(S[i].lower_y, S[i].q_last_y) : S[i].lower_y;
    IntLess il;
    introsort(low, n, il);
    int cur = 0, best = 0;
    for (int i = 0, j = 0; i < n;) {
      if (j < n && low[j] <= S[i].upper_y) {
        --cur;
        ++j;
      } else {
        best = max_(best, ++cur);
        ++i;
      }
    }
    g.max_active = best;
  }

  const CanvasDesc cd = b.canvases[pd.canvas];
  g.n_edges = n;
  g.start_y = (int)rb.t;
  g.stop_y = (int)rb.sb;
  // static_cast<uint32_t>(float) << 16 with x86-64 conversion semantics
  g.left_bound = (Fixed)((uint32_t)(int64_t)rb.sl << 16);
  g.right_bound = (Fixed)((uint32_t)(int64_t)rb.sr << 16);
  g.acc_left = (int)rb.l;
  g.acc_width = (int)(rb.r - rb.l);
  g.scan_top = rb.st;
  // canvas rows; a ClipPath pass keeps all of its rows (the clip's span list
  // is empty or not over all rows, SWCanvas::State::HasClip)
  const bool all_rows = (pd.flags & kPassClipPath) != 0;
  int r0 = all_rows ? g.start_y : max_(g.start_y, 0), r1 = all_rows ? g.stop_y : min_(g.stop_y, (int)cd.h);
  if (r0 < r1) {
    g.row0 = r0;
    g.row1 = r1;
  }
  b.geom[p] = g;
}


// ---------------------------------------------------------------------------
// sweep: the span sink and the sweep passes
// ---------------------------------------------------------------------------
// SWSpanBrush::Brush clipping (sw_span_brush.cc:78-99); false = dropped
SKC_HD bool ClipSpan(int& x, int y, int& len, int W, int H) {
  if (y < 0 || y >= H) return false;
  if (x >= W || x + len < 0) return false;
  if (x < 0) {
    len += x;
    x = 0;
  }
  if (x + len >= W) len = W - x;
  return len > 0;
}

// keep() applies the clipping of SWSpanBrush::Brush and drops spans whose
// alpha & global alpha is 0 under src-over (they blend to nothing).  A raw
// sink (the passes of the path-clip stages) keeps every span of its rows as
// the raster made it, in the raw format of pack(); only sinks built with
// kRawCapable take that form (the generic sweep's), so the register sweeps
// carry no test for it.
template <bool kRawCapable>
struct SinkBase {
  int row0, row1, W, H;
  uint32_t ga;
  bool srcover;
  bool raw;
  SKC_HD bool keep(int& x, int y, int& len, uint8_t a) const {
    if (y < row0 || y >= row1) return false;
    if (kRawCapable && raw) return true;
    if (!ClipSpan(x, y, len, W, H)) return false;
    return !(srcover && (a & ga) == 0);
  }
  // A stored span: x | len << 16 and the alpha; raw: x (int32) and
  // len | alpha << 24.
  SKC_HD uint2 pack(int x, int len, uint32_t a) const {
    return (kRawCapable && raw) ? make_uint2((uint32_t)x, ((uint32_t)len & 0xFFFFFFu) | (a << 24))
                                : make_uint2((uint32_t)x | ((uint32_t)len << 16), a);
  }
};

SKC_HD unsigned long long LaneBcast64(const Lanes& L, unsigned long long v, int src) {
#ifdef SKC_WARP_LANES
  return __shfl_sync(0xffffffffu, v, src);
#else
  return v;
#endif
}

// Spans go to one device-wide pool handed out in chunks of `chunk` spans.
// A pass writes its rows one after another, each row contiguous -- a row
// that would run past the end of its chunk is moved to a fresh chunk -- and
// records (first span, count) per canvas row.  When the pool is exhausted
// the pass keeps taking chunks but writes nothing, so the allocator ends at
// the exact size the pass needs; the caller then sweeps again with a pool
// that large.  All members are warp-uniform; methods are called by the
// whole warp.
template <bool kRawCapable>
struct PoolSinkT : SinkBase<kRawCapable> {
  using SinkBase<kRawCapable>::keep;
  using SinkBase<kRawCapable>::pack;
  using SinkBase<kRawCapable>::row0;
  using SinkBase<kRawCapable>::row1;
  uint2* pool;
  uint64_t cap;                // pool capacity in spans
  unsigned long long* next;    // spans handed out so far
  uint32_t chunk;              // spans per chunk (holds any row of the pass)
  uint2* rows;                 // (first span, count) per row of [row0, row1)
  uint32_t* err;
  int cur_row;
  uint64_t row_start, cur, chunk_end;
  bool dead;
  uint64_t kept;
  unsigned long long frags;

  SKC_HD void finish_row(const Lanes& L) {
    if (!dead && cur > row_start && cur_row >= row0 && cur_row < row1 && L.leader())
      rows[cur_row - row0] = make_uint2((uint32_t)row_start, (uint32_t)(cur - row_start));
  }
  SKC_HD void row_begin(const Lanes& L, int y) {
    if (y == cur_row) return;
    finish_row(L);
    cur_row = y;
    row_start = cur;
  }
  // Room for `add` more spans after the `written` spans this step already
  // put at cur; returns cur (the row may have moved to a new chunk).
  SKC_HD uint64_t reserve(const Lanes& L, uint32_t written, uint32_t add) {
    if (SKC_LIKELY(cur + written + add <= chunk_end)) return cur;
    const uint64_t have = cur + written - row_start;
    if (have + add > chunk) {  // a row larger than a chunk (not expected)
      FlagError(err, 8);
      dead = true;
    }
    unsigned long long c = 0;
    if (L.leader()) {
#ifdef __CUDA_ARCH__
      c = atomicAdd(next, (unsigned long long)chunk);
#else
      c = *next;
      *next += chunk;
#endif
    }
    c = LaneBcast64(L, c, 0);
    if (c + chunk > cap) dead = true;
    if (!dead) {
      L.sync();
      for (uint64_t i = L.lane; i < have; i += Lanes::n) pool[c + i] = pool[row_start + i];
      L.sync();
    }
    cur = c + (cur - row_start);
    row_start = c;
    chunk_end = c + chunk;
    return cur;
  }
  SKC_HD uint2* span_ptr(uint64_t i) { return dead ? nullptr : pool + i; }
  // n: spans appended (warp-uniform); f: this lane's share of their
  // fragments (the shares are summed once, when the pass finishes)
  SKC_HD void commit(const Lanes&, uint32_t n, unsigned long long f) {
    cur += n;
    kept += n;
    frags += f;
  }
  // Sparse form of acc_row; returns false (nothing read, nothing written)
  // when the row has more than ev_cap nonzero entries.
  SKC_HD bool acc_row_sparse(const Lanes& L, int y, int32_t* diff, int left, int lo, int hi,
                             int32_t* ev, int ev_cap) {
    constexpr int V = 4;
    constexpr int kNone = 0x7fffffff;
    const bool vec = ((uintptr_t)diff & 15) == 0;
    int ne = 0;
    for (int base = vec ? (lo & ~(V - 1)) : lo; base < hi; base += Lanes::n * V) {
      const int i0 = base + L.lane * V;
      int32_t d[V];
      if (vec && i0 + V <= hi) {
        const int4 q = *(const int4*)(diff + i0);
        d[0] = q.x;
        d[1] = q.y;
        d[2] = q.z;
        d[3] = q.w;
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j) d[j] = i0 + j < hi ? diff[i0 + j] : 0;
      }
      int cnt = 0;
#pragma unroll
      for (int j = 0; j < V; ++j) cnt += d[j] != 0 ? 1 : 0;
      if (!L.ballot(cnt != 0)) continue;
      const int32_t incl = LaneScanIncl(L, cnt);
      const int total = LaneBcast(L, incl, Lanes::n - 1);
      if (SKC_COLD(ne + total > ev_cap)) return false;
      int at = ne + incl - cnt;
#pragma unroll
      for (int j = 0; j < V; ++j) {
        if (d[j] != 0) {
          ev[2 * at] = i0 + j;
          ev[2 * at + 1] = d[j];
          at++;
        }
      }
      ne += total;
    }
    L.sync();
    int open_start = -1;  // warp-uniform: the run still open after a step
    int32_t open_v = 0;
    int32_t carry = 0, prev_sat = 0;
    for (int eb = 0; eb < ne; eb += Lanes::n) {
      const int e = eb + L.lane;
      const bool valid = e < ne;
      int pos = kNone;
      int32_t v = 0;
      if (valid) {
        pos = ev[2 * e];
        v = ev[2 * e + 1];
        diff[pos] = 0;
      }
      const int32_t incl = LaneScanIncl(L, v) + carry;
      const int32_t sat = incl > 255 ? 255 : incl;
      int32_t before = LaneBcast(L, sat, L.lane > 0 ? L.lane - 1 : 0);
      if (L.lane == 0) before = prev_sat;
      const bool start = valid && sat != before;
      const unsigned starts = L.ballot(start);
      const unsigned later = starts & ~((2u << L.lane) - 1u);
      int next = (int)L.shfl((uint32_t)pos, later ? Lanes::ffs(later) - 1 : L.lane);
      if (!later) next = kNone;
      uint2 out[2];
      int cnt = 0;
      unsigned long long fr = 0;
      auto put = [&](int s0, int w, int32_t a) {
        int x = left + s0, len = w;
        if (keep(x, y, len, (uint8_t)a)) {
          out[cnt++] = pack(x, len, (uint32_t)a);
          fr += (unsigned)len;
        }
      };
      if (starts && open_start >= 0 && L.lane == Lanes::ffs(starts) - 1)
        put(open_start, pos - open_start, open_v);
      if (start && next != kNone && sat != 0) put(pos, next - pos, sat);
      if (starts) {
        const int src = 31 - clz_(starts);
        const int32_t lv = LaneBcast(L, sat, src);
        const int lp = LaneBcast(L, pos, src);
        open_start = lv != 0 ? lp : -1;
        open_v = lv;
      }
      const int32_t ci = LaneScanIncl(L, cnt);
      const uint32_t total = (uint32_t)LaneBcast(L, ci, Lanes::n - 1);
      if (total) {
        const uint64_t at = reserve(L, 0, total);
        uint2* dst = span_ptr(at + (uint32_t)(ci - cnt));
        if (dst) {
          for (int i = 0; i < cnt; ++i) dst[i] = out[i];
        }
        commit(L, total, fr);
      }
      carry = LaneBcast(L, incl, Lanes::n - 1);
      prev_sat = LaneBcast(L, sat, Lanes::n - 1);
    }
    if (open_start >= 0) {
      int x = left + open_start, len = hi - open_start;
      if (keep(x, y, len, (uint8_t)open_v)) {
        const uint64_t at = reserve(L, 0, 1);
        if (!dead && L.leader())
          pool[at] = pack(x, len, (uint32_t)open_v);
        commit(L, 1, L.leader() ? (unsigned)len : 0u);
      }
    }
    return true;
  }

  // The accumulated spans of a row follow its direct spans (the reference
  // flushes a row's accumulator only after leaving the row,
  // SpanBuilder::Flush, sw_raster.cc:103-136): the runs of equal nonzero
  // saturated prefix sums of diff[lo, hi), in increasing x.  Returns false
  // when the row lies outside the canvas (diff not read).
  //
  // Each lane takes V consecutive entries per chunk of Lanes::n * V; a run
  // starts at every entry whose saturated sum differs from its left
  // neighbour's and ends at the next such entry.  A lane closes the runs
  // that start at its entries (the last one ends at the next lane's first
  // start), the lane with the chunk's first start also closes the run left
  // open by earlier chunks, and the chunk's spans are written after one
  // prefix sum.  Every entry read is reset to zero.
  //
  // With an event scratch (ev, room for ev_cap (position, value) pairs) the
  // nonzero entries are first gathered in x order -- a difference array has
  // two per accumulated span, usually far fewer than the row is wide -- and
  // the runs are found over that list, 32 entries per step, with the same
  // rules; a row with more nonzero entries than ev_cap takes the dense path.
  SKC_HD bool acc_row(const Lanes& L, int y, int32_t* diff, int left, int lo, int hi,
                      int32_t* ev = nullptr, int ev_cap = 0) {
    if (y < row0 || y >= row1) return false;
    row_begin(L, y);
    if (ev && Lanes::n == 32 && acc_row_sparse(L, y, diff, left, lo, hi, ev, ev_cap)) return true;
    constexpr int V = Lanes::n == 32 ? 4 : 1;
    constexpr int kNone = 0x7fffffff;
    int open_start = -1;   // warp-uniform: the run still open after a chunk
    int32_t open_v = 0;
    int32_t carry = 0;     // prefix sum before this chunk
    int32_t prev_sat = 0;  // saturated value of the entry before this chunk
    // Entries outside [lo, hi] are zero, so the chunks can start at a
    // multiple of V (16-byte loads); a chunk of zeros changes no sum and
    // starts no run, and is skipped after one load.
    const bool vec = V == 4 && ((uintptr_t)diff & 15) == 0;
    for (int base = vec ? (lo & ~(V - 1)) : lo; base < hi; base += Lanes::n * V) {
      const int i0 = base + L.lane * V;
      int32_t sat[V];
      if (vec && i0 + V <= hi) {
        const int4 q = *(const int4*)(diff + i0);
        sat[0] = q.x;
        sat[1 % V] = q.y;
        sat[2 % V] = q.z;
        sat[3 % V] = q.w;
      } else {
#pragma unroll
        for (int j = 0; j < V; ++j) sat[j] = i0 + j < hi ? diff[i0 + j] : 0;
      }
      bool nz = false;
#pragma unroll
      for (int j = 0; j < V; ++j) nz |= sat[j] != 0;
      if (!L.ballot(nz)) continue;
      if (nz) {
#pragma unroll
        for (int j = 0; j < V; ++j)
          if (i0 + j < hi) diff[i0 + j] = 0;
      }
      int32_t run = 0;
#pragma unroll
      for (int j = 0; j < V; ++j) {
        run += sat[j];
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
      const unsigned has = L.ballot(bits != 0);
      const int first_pos = bits ? i0 + Lanes::ffs(bits) - 1 : kNone;
      const unsigned later = has & ~((2u << L.lane) - 1u);
      int next_first = (int)L.shfl((uint32_t)first_pos, later ? Lanes::ffs(later) - 1 : L.lane);
      if (!later) next_first = kNone;
      // this lane's spans, in x order
      uint2 out[V + 1];
      int cnt = 0;
      unsigned long long fr = 0;
      auto put = [&](int s0, int w, int32_t a) {
        int x = left + s0, len = w;
        if (keep(x, y, len, (uint8_t)a)) {
          out[cnt++] = pack(x, len, (uint32_t)a);
          fr += (unsigned)len;
        }
      };
      if (has && open_start >= 0 && L.lane == Lanes::ffs(has) - 1)
        put(open_start, first_pos - open_start, open_v);
#pragma unroll
      for (int j = 0; j < V; ++j) {
        if (!(bits & (1u << j))) continue;
        const unsigned rest = bits & ~((2u << j) - 1u);
        const int end = rest ? i0 + Lanes::ffs(rest) - 1 : next_first;
        if (end != kNone && sat[j] != 0) put(i0 + j, end - (i0 + j), sat[j]);
      }
      // the run left open: the chunk's last start, if any
      if (has) {
        const int src = 31 - clz_(has);
        const int lb = 31 - clz_(bits ? bits : 1u);
        const int32_t lv = sat[lb];
        const int lpos = i0 + lb;
        const int32_t v = LaneBcast(L, lv, Lanes::n == 32 ? src : 0);
        const int pos = LaneBcast(L, lpos, Lanes::n == 32 ? src : 0);
        open_start = v != 0 ? pos : -1;
        open_v = v;
      }
      const int32_t ci = LaneScanIncl(L, cnt);
      const uint32_t total = (uint32_t)LaneBcast(L, ci, Lanes::n - 1);
      if (total) {
        const uint64_t at = reserve(L, 0, total);
        uint2* dst = span_ptr(at + (uint32_t)(ci - cnt));
        if (dst) {
          for (int i = 0; i < cnt; ++i) dst[i] = out[i];
        }
        commit(L, total, fr);
      }
      carry += LaneBcast(L, incl, Lanes::n - 1);
      prev_sat = LaneBcast(L, sat[V - 1], Lanes::n - 1);
    }
    if (open_start >= 0) {
      int x = left + open_start, len = hi - open_start;
      if (keep(x, y, len, (uint8_t)open_v)) {
        const uint64_t at = reserve(L, 0, 1);
        if (!dead && L.leader()) pool[at] = pack(x, len, (uint32_t)open_v);
        commit(L, 1, L.leader() ? (unsigned)len : 0u);
      }
    }
    return true;
  }
};

using PoolSink = PoolSinkT<true>;       // the generic sweep's: every pass form
using PoolSinkReg = PoolSinkT<false>;   // the register sweeps': never raw

template <typename Sink>
SKC_HD void InitPoolSink(const DevBatch& b, uint32_t p, const PassGeom& g, Sink* s) {
  const PassDesc pd = b.passes[p];
  const PassSweep sw = b.sweep[p];
  const CanvasDesc cd = b.canvases[pd.canvas];
  s->row0 = g.row0;
  s->row1 = g.row1;
  s->W = (int)cd.w;
  s->H = (int)cd.h;
  s->ga = pd.ga;
  s->srcover = (pd.flags & kPassSrcOver) != 0;
  s->raw = (pd.flags & kPassRawSpans) != 0;
  s->pool = b.spans;
  s->cap = b.span_cap;
  s->next = b.span_next;
  s->chunk = sw.chunk;
  s->rows = b.rowspan + sw.rbase;
  s->err = b.err;
  s->cur_row = kNaN32;
  s->row_start = s->cur = s->chunk_end = 0;
  s->dead = false;
  s->kept = 0;
  s->frags = 0;
}

template <typename Sink>
SKC_HD void FinishPass(const DevBatch& b, uint32_t p, Sink* s, const Lanes& L) {
  s->finish_row(L);
  const unsigned long long frags = LaneSum64(L, s->frags);
  L.sync();
  if (L.leader()) {
    b.pass_spans[p] = (uint32_t)s->kept;
    if (b.pass_frags) b.pass_frags[p] = frags;
  }
}

SKC_HD void EmptyPass(const DevBatch& b, uint32_t p, const Lanes& L) {
  if (L.leader()) {
    b.pass_spans[p] = 0;
    if (b.pass_frags) b.pass_frags[p] = 0;
  }
}

// The generic sweep of pass p (LaneSweep, state in the pass's sweep memory).
template <typename Sink>
SKC_HDN void RunSweep(const DevBatch& b, uint32_t p, const PassGeom& g, Sink* sink,
                      const Lanes& lanes) {
  const PassDesc pd = b.passes[p];
  const PassSweep sw = b.sweep[p];
  SliceLayout L;
  L.compute(pd.cap, sizeof(Edge));
  const Edge* S = (const Edge*)(b.scratch + pd.slice_off + L.off[13]);
  int n = g.n_edges;
  SweepMem M = SweepMemAt(b.sweepmem + sw.work_off, n, g.acc_width);
  for (int i = lanes.lane; i < n; i += Lanes::n) M.W[i] = S[i];
  for (int i = lanes.lane; i <= g.acc_width; i += Lanes::n) M.diff[i] = 0;
  lanes.sync();
  LaneSweep<Sink> s;
  s.L = lanes;
  s.M = M;
  s.n = n;
  s.err = b.err;
  s.sink = sink;
  s.acc_left = g.acc_left;
  s.acc_width = g.acc_width;
  s.acc_y = kNaN32;
  s.touch_lo = 0x7fffffff;
  s.touch_hi = -1;
  s.scan_top = g.scan_top;
  s.walk((pd.flags & kPassEvenOdd) != 0, g.start_y, g.stop_y, g.left_bound, g.right_bound);
  s.flush_acc();
}

// Sweep of pass p through the generic sweep.  Row entries a register attempt
// may have written are cleared first.  kRaw: the pass may be a path clip's
// (raw spans); batches without path clips take the form without that test.
template <bool kRaw = true>
SKC_HDN void SweepPass(const DevBatch& b, uint32_t p, const Lanes& lanes) {
  const PassGeom g = b.geom[p];
  const int nrows = g.row1 - g.row0;
  if (g.n_edges <= 0 || nrows <= 0) {
    EmptyPass(b, p, lanes);
    return;
  }
  uint2* rows = b.rowspan + b.sweep[p].rbase;
  for (int r = lanes.lane; r < nrows; r += Lanes::n) rows[r] = make_uint2(0, 0);
  lanes.sync();
  PoolSinkT<kRaw> sink;
  InitPoolSink(b, p, g, &sink);
  RunSweep(b, p, g, &sink, lanes);
  FinishPass(b, p, &sink, lanes);
}

template <int M>
SKC_HD uint64_t RegSmemBytes(int32_t diff_cap) {
  return sizeof(RegSharedT<M>) + 4ull * (uint64_t)diff_cap;
}

// The register sweep of pass p (RegWalk); returns 0 when its active list
// outgrows the registers.  The accumulator sits in shared memory when it fits.
template <int M, typename Sink>
SKC_HD int RunRegSweep(const DevBatch& b, uint32_t p, const PassGeom& g, Sink* sink,
                       const Lanes& lanes, RegSharedT<M>* sh, int32_t* sdiff, int32_t sdiff_cap) {
  const PassDesc pd = b.passes[p];
  const PassSweep sw = b.sweep[p];
  SliceLayout L;
  L.compute(pd.cap, sizeof(Edge));
  const Edge* S = (const Edge*)(b.scratch + pd.slice_off + L.off[13]);
  const int n = g.n_edges;
  SweepMem Mm = SweepMemAt(b.sweepmem + sw.work_off, n, g.acc_width);
  for (int i = lanes.lane; i < n; i += Lanes::n) Mm.W[i] = S[i];
  int32_t* diff = g.acc_width + 1 <= sdiff_cap ? sdiff : Mm.diff;
  for (int i = lanes.lane; i <= g.acc_width; i += Lanes::n) diff[i] = 0;
  lanes.sync();
  AccState as;
  as.diff = diff;
  as.left = g.acc_left;
  as.width = g.acc_width;
  as.y = kNaN32;
  as.lo = 0x7fffffff;
  as.hi = -1;
  as.ev = sh->u.ev;
  as.ev_cap = RegSharedT<M>::kFlushEvents;
  if (!RegWalk(lanes, *sh, Mm.W, n, sink, as, g.scan_top, (pd.flags & kPassEvenOdd) != 0,
               g.start_y, g.stop_y, g.left_bound, g.right_bound))
    return 0;
  AccFlush(lanes, as, sink);
  return 1;
}

// Which sweep form takes pass p: the register form for up to 32, 64 or 128
// active edges, or the generic form, by the geometry's bound of the active
// list (PassGeom::max_active); pass_class != 0 forces the generic form.
// The forms' kernels take disjoint passes and depend on nothing the others
// write, so their launches may overlap.
enum : int { kSweepReg64 = 0, kSweepReg128 = 2, kSweepGeneric = 1, kSweepReg32 = 3 };
// The 32-edge form runs last (lightest form) and takes only short passes,
// so that no long sweep starts at the end of the sweep launches.
constexpr int kReg32MaxRows = 1100;
SKC_HD int SweepForm(const PassGeom& g, uint8_t pass_class) {
  if (pass_class != 0) return pass_class;
  if (g.raw_spans) return kSweepGeneric;  // the path-clip stages' passes (rare)
  const int ma = g.max_active;
  return (ma <= 32 && g.row1 - g.row0 <= kReg32MaxRows) ? kSweepReg32
         : ma <= 64                                     ? kSweepReg64
         : ma <= kRegMaxM                               ? kSweepReg128
                                                        : kSweepGeneric;
}

// Sweep of pass p through the register form of size M.  Returns false when
// its active list outgrows M after all: the caller then sweeps the pass with
// the generic form (SweepPass, which clears the rows the attempt wrote).
// The generic form is not inlined here, so the register kernels stay small.
template <int M>
SKC_HD bool SweepPassReg(const DevBatch& b, uint32_t p, const Lanes& lanes, RegSharedT<M>* sh,
                         int32_t* sdiff, int32_t sdiff_cap) {
  const PassGeom g = b.geom[p];
  if (g.n_edges <= 0 || g.row1 <= g.row0) {
    EmptyPass(b, p, lanes);
    return true;
  }
  // rows the sweep leaves without spans read as empty
  uint2* rows = b.rowspan + b.sweep[p].rbase;
  for (int r = lanes.lane; r < g.row1 - g.row0; r += Lanes::n) rows[r] = make_uint2(0, 0);
  lanes.sync();
  PoolSinkReg sink;
  InitPoolSink(b, p, g, &sink);
  if (!RunRegSweep<M>(b, p, g, &sink, lanes, sh, sdiff, sdiff_cap)) {
    lanes.sync();
    return false;
  }
  FinishPass(b, p, &sink, lanes);
  return true;
}



// ---------------------------------------------------------------------------
// StackBlur lines
// ---------------------------------------------------------------------------
SKC_HD int32_t StackBlurShr(int32_t r) {
  uint32_t d = (uint32_t)(r + 1) * (uint32_t)(r + 1);
  return (31 - clz_(d)) + 9;
}
SKC_HD uint64_t StackBlurMul(int32_t r) {
  uint64_t d = (uint64_t)(r + 1) * (uint64_t)(r + 1);
  return ((1ull << StackBlurShr(r)) + d - 1) / d;
}

// Blur one line of n pixels (stride in pixels) from src into dst. v_bug
// reproduces the vertical pass's out_sum initialisation (slots 0 and 3 from
// slot 1, sw_stack_blur.cc:175-179).
SKC_HDN void BlurLine(const uint8_t* src, uint8_t* dst, int n, size_t stride, int r, bool v_bug) {
  const int rp1 = r + 1;
  const int nm1 = n - 1;
  const uint64_t sum_factor = (uint64_t)(rp1 * (rp1 + 1) / 2);
  const uint64_t mul = StackBlurMul(r);
  const int shr = StackBlurShr(r);
  auto px = [&](int i, int c) -> uint64_t { return src[(size_t)i * stride * 4 + c]; };
  uint64_t sum[4], in_sum[4], out_sum[4];
  for (int c = 0; c < 4; ++c) {
    uint64_t p0 = px(0, c);
    sum[c] = p0 * sum_factor;
    out_sum[c] = p0 * rp1;
    in_sum[c] = 0;
  }
  if (v_bug) {
    out_sum[0] = px(0, 1) * rp1;
    out_sum[3] = px(0, 1) * rp1;
  }
  for (int i = 1; i <= r; ++i) {
    int k = min_(i, nm1);
    for (int c = 0; c < 4; ++c) {
      uint64_t v = px(k, c);
      sum[c] += v * (uint64_t)(rp1 - i);
      in_sum[c] += v;
    }
  }
  for (int i = 0; i < n; ++i) {
    uint8_t* o = dst + (size_t)i * stride * 4;
    int kout = max_(i - r, 0), kin = min_(i + rp1, nm1), kmid = min_(i + 1, nm1);
    for (int c = 0; c < 4; ++c) {
      o[c] = (uint8_t)((sum[c] * mul) >> shr);
      sum[c] -= out_sum[c];
      out_sum[c] -= px(kout, c);
      in_sum[c] += px(kin, c);
      sum[c] += in_sum[c];
      uint64_t vm = px(kmid, c);
      out_sum[c] += vm;
      in_sum[c] -= vm;
    }
  }
}


// Scalar composite of one row task (CPU execution of the pipeline; the GPU
// runs the warp-parallel form in kernels.cu with identical per-pixel order).
SKC_HDN void CompositeRowScalar(const DevBatch& b, const RowTask& rt, uint32_t* row) {
  const CanvasDesc cd = b.canvases[rt.canvas];
  const int y = (int)rt.y, x0 = (int)rt.x0, x1 = (int)rt.x1;
  uint32_t* gpx = (uint32_t*)(b.pixels + cd.px_off) + (size_t)y * cd.w + x0;
  for (int i = 0; i < x1 - x0; ++i) row[i] = cd.has_clear ? cd.clear_pm : RGBAtoARGB(gpx[i]);
  const uint32_t band = cd.band0 + ((uint32_t)y >> b.band_shift);
  for (uint32_t e = b.band_off[band]; e < b.band_off[band + 1]; ++e) {
    const PassComp pc = b.comp[b.bins[e]];
    if (y < pc.row0 || y >= pc.row1) continue;
    const uint2 rs = b.rowspan[pc.rbase + (y - pc.row0)];
    const Brush br = b.brushes[pc.brush];
    for (uint32_t s = rs.x; s < rs.x + rs.y; ++s) {
      uint2 sp = b.spans[s];
      int sx = (int)(sp.x & 0xFFFF), slen = (int)(sp.x >> 16);
      int xs = max_(sx, x0), xe = min_(sx + slen, x1);
      uint32_t alpha = sp.y & br.global_alpha;
      for (int x = xs; x < xe; ++x) {
        uint32_t c = BrushColor(br, x, y, b.stop_colors, b.stop_offsets, b.pixels, b.roundtrip,
                                b.conicals);
        if (alpha != 255) c = AlphaMulQ(c, alpha);
        if (br.cf_type) c = FilterColor(br, c, b.srgb_tables, b.cf_matrices);
        row[x - x0] = BlendPixel(row[x - x0], c, br.blend);
      }
    }
  }
  for (int i = 0; i < x1 - x0; ++i) gpx[i] = ARGBtoRGBA(row[i]);
}

}  // namespace skc
