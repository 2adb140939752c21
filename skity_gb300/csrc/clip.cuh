// Path clips: the span algebra of SWCanvas::State (src/render/sw/
// sw_canvas.cc:42-265) on one canvas row at a time, restated for one GPU
// thread per row.  The reference runs it over whole span lists, but every
// operation it uses pairs spans of the same row only, and keeps the lists in
// row order, so a row's result depends on that row's inputs alone (one
// exception, noted at ClipMergeRow).
//
// Inputs are rows of spans in the raw format (SinkBase::pack with raw set):
// x as an int32, len | cover << 24.  Outputs go to an emit(x, len, cover)
// callback, in the order the reference appends them.
#pragma once
#include "passes.cuh"

namespace skc {

struct RowSpans {  // the raw spans of one row
  const uint2* s;
  uint32_t n;
};
struct SpanV {
  int32_t x, len, cover;
};
SKC_HD SpanV RawSpanAt(const RowSpans& r, uint32_t i) {
  const uint2 v = r.s[i];
  return SpanV{(int32_t)v.x, (int32_t)(v.y & 0xFFFFFFu), (int32_t)(v.y >> 24)};
}

// FindSpan (sw_canvas.cc:218-262): the pieces of s under each span of the
// clip row, in clip order, covers min'd (with the reference's + 1 when the
// clip span starts inside s).
template <typename Emit>
SKC_HD void ClipFindSubSpans(const SpanV& s, const RowSpans& clip, Emit& emit) {
  for (uint32_t i = 0; i < clip.n; ++i) {
    const SpanV c = RawSpanAt(clip, i);
    const int32_t cover = min_(c.cover, s.cover);
    if (c.x < s.x) {
      if (c.x + c.len < s.x) continue;
      emit(s.x, min_(c.x + c.len, s.x + s.len) - s.x, cover);
    } else if (c.x == s.x) {
      emit(s.x, min_(s.len, c.len), cover);
    } else {
      if (s.x + s.len < c.x) continue;
      emit(c.x, min_(s.x + s.len - c.x + 1, c.len), cover);
    }
  }
}

struct SpanXLess {  // std::sort by x over span indices
  const RowSpans* r;
  SKC_HD bool operator()(int32_t a, int32_t b) const {
    return (int32_t)r->s[a].x < (int32_t)r->s[b].x;
  }
};

// spans_subtraction (sw_canvas.cc:59-133) on one row: every span of a minus
// the spans of b (ordered by x the way std::sort orders them; `order` holds
// room for b.n indices).  False when b has more than `cap` spans.
template <typename Emit>
SKC_HD bool ClipSubtractRow(const RowSpans& a, const RowSpans& b, int32_t* order, uint32_t cap,
                            Emit& emit) {
  if (b.n > cap) return false;
  for (uint32_t i = 0; i < b.n; ++i) order[i] = (int32_t)i;
  if (b.n > 1) introsort(order, (int)b.n, SpanXLess{&b});
  for (uint32_t i = 0; i < a.n; ++i) {
    const SpanV sp = RawSpanAt(a, i);
    if (b.n == 0) {
      emit(sp.x, sp.len, sp.cover);
      continue;
    }
    int32_t x = sp.x, len = sp.len;
    for (uint32_t j = 0; j < b.n; ++j) {
      const SpanV m = RawSpanAt(b, (uint32_t)order[j]);
      if (m.x + m.len < x || m.x > x + len) continue;
      if (m.x < x) {
        if (m.x + m.len > x + len) {  // all of it is subtracted
          len = 0;
          break;
        }
        const int32_t end = x + len, piece = m.x + m.len - x;
        if (piece == 0) continue;
        emit(x, piece, sp.cover);  // the reference emits the overlapped part here
        x += piece;
        len = end - x;
      } else if (m.x + m.len < x + len) {
        const int32_t end = x + len;
        emit(x, m.x - x, sp.cover);
        x = m.x + m.len;
        len = end - x;
      } else {
        emit(x, m.x - x, sp.cover);
        len = 0;
      }
      if (len <= 0) break;
    }
    if (len > 0) emit(x, len, sp.cover);
  }
  return true;
}

// The spans of a then b in one index space, for the merge.
struct MergeLess {
  const RowSpans* a;
  const RowSpans* b;
  SKC_HD uint2 at(int32_t i) const { return i < (int32_t)a->n ? a->s[i] : b->s[i - (int32_t)a->n]; }
  SKC_HD bool operator()(int32_t i, int32_t j) const {
    const uint2 p = at(i), q = at(j);
    if ((int32_t)p.x != (int32_t)q.x) return (int32_t)p.x < (int32_t)q.x;
    return (p.y >> 24) > (q.y >> 24);
  }
};

// PerformMerge (sw_canvas.cc:195-216) on one row: a's spans then b's,
// ordered by (x, cover descending) with std::sort's algorithm.  The
// reference sorts the whole concatenated list at once; the order it gives
// equal keys (same x and cover, different lengths) can differ from this
// per-row sort -- the one place the row-by-row form is not exact.
template <typename Emit>
SKC_HD bool ClipMergeRow(const RowSpans& a, const RowSpans& b, int32_t* order, uint32_t cap,
                         Emit& emit) {
  const uint32_t n = a.n + b.n;
  if (n > cap) return false;
  for (uint32_t i = 0; i < n; ++i) order[i] = (int32_t)i;
  MergeLess less{&a, &b};
  if (n > 1) introsort(order, (int)n, less);
  for (uint32_t i = 0; i < n; ++i) {
    const uint2 v = less.at(order[i]);
    emit((int32_t)v.x, (int32_t)(v.y & 0xFFFFFFu), (int32_t)(v.y >> 24));
  }
  return true;
}

// One row of a clip state (OnClipPath, sw_canvas.cc:317-336): the parent's
// row (when the parent has a clip) combined with the clip path's raster row
// by RecursiveClip (:177-193).  op_parent / op: Canvas::ClipOp.
template <typename Emit>
SKC_HD bool ClipStateRow(bool parent_has, uint32_t op_parent, const RowSpans& parent,
                         const RowSpans& raster, uint32_t op, int32_t* order, uint32_t cap,
                         Emit& emit) {
  if (!parent_has) {
    for (uint32_t i = 0; i < raster.n; ++i) {
      const SpanV s = RawSpanAt(raster, i);
      emit(s.x, s.len, s.cover);
    }
    return true;
  }
  if (op_parent == op) {
    if (op == 1) {  // PerformClip with an intersect state: FindSpan per span
      for (uint32_t i = 0; i < raster.n; ++i) ClipFindSubSpans(RawSpanAt(raster, i), parent, emit);
      return true;
    }
    return ClipMergeRow(raster, parent, order, cap, emit);
  }
  return op_parent == 0 ? ClipSubtractRow(raster, parent, order, cap, emit)
                        : ClipSubtractRow(parent, raster, order, cap, emit);
}

// One row of a draw under a clip state (DoBrush, sw_canvas.cc:338-353,
// PerformClip :157-175): the draw's raster row clipped by the state's row.
template <typename Emit>
SKC_HD bool ClipDrawRow(bool has, uint32_t op, const RowSpans& state, const RowSpans& draw,
                        int32_t* order, uint32_t cap, Emit& emit) {
  if (!has) {
    for (uint32_t i = 0; i < draw.n; ++i) {
      const SpanV s = RawSpanAt(draw, i);
      emit(s.x, s.len, s.cover);
    }
    return true;
  }
  if (op == 0) return ClipSubtractRow(draw, state, order, cap, emit);
  for (uint32_t i = 0; i < draw.n; ++i) ClipFindSubSpans(RawSpanAt(draw, i), state, emit);
  return true;
}

// The raw rows the stages read: row y of pass p, of clip state k (1-based).
// A row placed past the end of the pool (a render whose pool ran out, which
// the host reruns with a larger pool) reads as empty.
SKC_HD RowSpans PoolRow(const DevBatch& b, uint2 rs) {
  if ((uint64_t)rs.x + rs.y > b.span_cap) return RowSpans{nullptr, 0};
  return RowSpans{b.spans + rs.x, rs.y};
}
SKC_HD RowSpans PassRow(const DevBatch& b, uint32_t p, int32_t y) {
  const PassGeom& g = b.geom[p];
  if (g.n_edges <= 0 || y < g.row0 || y >= g.row1) return RowSpans{nullptr, 0};
  return PoolRow(b, b.rowspan[b.sweep[p].rbase + (uint32_t)(y - g.row0)]);
}
SKC_HD RowSpans StateRow(const DevBatch& b, uint32_t k, int32_t y) {
  if (k == 0) return RowSpans{nullptr, 0};
  const ClipStateDesc& st = b.clip_states[k - 1];
  if (y < st.y0 || y >= st.y1) return RowSpans{nullptr, 0};
  return PoolRow(b, b.clip_rows[st.rbase + (uint32_t)(y - st.y0)]);
}

constexpr uint32_t kClipRowCap = 256;  // spans of one row a sort takes

// Counts, then writes a row's output into the span pool (one exact-size
// allocation per row; past the pool's end nothing is written and the
// counter keeps growing, so the host can grow the pool and rerun).
struct RowOut {
  uint2* pool;
  uint64_t cap;
  bool write;
  bool raw;         // the raw format (clip states) or the compositor's (draws, brush-clipped)
  int W, H, y;      // draws: the brush's clipping (SWSpanBrush::Brush, sw_span_brush.cc:66-104)
  bool srcover;
  uint32_t ga;
  uint64_t at;
  uint32_t n;
  SKC_HD void operator()(int32_t x, int32_t len, int32_t cover) {
    if (!raw) {
      int cx = x, clen = len;
      if (!ClipSpan(cx, y, clen, W, H)) return;
      if (srcover && (((uint32_t)cover & ga) == 0)) return;
      x = cx;
      len = clen;
    }
    if (write && at + n < cap)
      pool[at + n] = raw ? make_uint2((uint32_t)x, ((uint32_t)len & 0xFFFFFFu) | ((uint32_t)cover << 24))
                         : make_uint2((uint32_t)x | ((uint32_t)len << 16), (uint32_t)cover);
    ++n;
  }
};

}  // namespace skc

namespace skc {

SKC_HD unsigned long long ReserveSpans(unsigned long long* next, uint32_t n) {
#ifdef __CUDA_ARCH__
  return atomicAdd(next, (unsigned long long)n);
#else
  const unsigned long long at = *next;
  *next += n;
  return at;
#endif
}
SKC_HD void FlagOr(uint32_t* word, uint32_t bits) {
#ifdef __CUDA_ARCH__
  atomicOr(word, bits);
#else
  *word |= bits;
#endif
}

// Row y of clip state k (1-based): OnClipPath on the parent state's row.
// Every row writes the state's op (the same value); a row with spans marks
// the state as holding a clip.
SKC_HD void ClipStateStage(const DevBatch& b, uint32_t k, int32_t y, int32_t* order) {
  const ClipStateDesc& st = b.clip_states[k - 1];
  const bool parent_has = st.parent != 0 && b.clip_flags[2 * (st.parent - 1)] != 0;
  const uint32_t op_parent = st.parent != 0 ? b.clip_flags[2 * (st.parent - 1) + 1] : 0u;
  const RowSpans parent = StateRow(b, st.parent, y);
  const RowSpans raster = PassRow(b, st.pass, y);
  RowOut out{b.spans, b.span_cap, false, true, 0, 0, y, false, 255u, 0, 0};
  if (!ClipStateRow(parent_has, op_parent, parent, raster, st.op, order, kClipRowCap, out)) {
    FlagError(b.err, 32);
    return;
  }
  const uint32_t n = out.n;
  out.n = 0;
  out.at = n ? ReserveSpans(b.span_next, n) : 0;
  out.write = true;
  if (n) ClipStateRow(parent_has, op_parent, parent, raster, st.op, order, kClipRowCap, out);
  b.clip_rows[st.rbase + (uint32_t)(y - st.y0)] = make_uint2((uint32_t)out.at, n);
  if (y == st.y0) b.clip_flags[2 * (k - 1) + 1] = !parent_has ? st.op : (op_parent != st.op ? 1u : op_parent);
  if (n) FlagOr(&b.clip_flags[2 * (k - 1)], 1u);
}

// Item i of the draws under a path clip: row y of pass p, its raw spans
// clipped by the state's row and the brush, rewritten in the compositor's
// format over the pass's row entry.
SKC_HD void ClipApplyStage(const DevBatch& b, uint32_t i, int32_t* order) {
  const uint2 item = b.clip_items[i];
  const uint32_t p = item.x;
  const int32_t y = (int32_t)item.y;
  const PassDesc& pd = b.passes[p];
  const uint32_t k = pd.path_clip;
  const bool has = b.clip_flags[2 * (k - 1)] != 0;
  const uint32_t op = b.clip_flags[2 * (k - 1) + 1];
  const RowSpans state = StateRow(b, k, y);
  const RowSpans draw = PassRow(b, p, y);
  const CanvasDesc& cd = b.canvases[pd.canvas];
  RowOut out{b.spans, b.span_cap, false, false, (int)cd.w, (int)cd.h, y,
             (pd.flags & kPassSrcOver) != 0, pd.ga, 0, 0};
  if (!ClipDrawRow(has, op, state, draw, order, kClipRowCap, out)) {
    FlagError(b.err, 32);
    return;
  }
  const uint32_t n = out.n;
  out.n = 0;
  out.at = n ? ReserveSpans(b.span_next, n) : 0;
  out.write = true;
  if (n) ClipDrawRow(has, op, state, draw, order, kClipRowCap, out);
  const PassGeom& g = b.geom[p];
  b.rowspan[b.sweep[p].rbase + (uint32_t)(y - g.row0)] = make_uint2((uint32_t)out.at, n);
}

}  // namespace skc
