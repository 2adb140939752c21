// Device planning of a render: everything the sweeps and the compositor need
// after the geometry stage, computed on the GB300 from the passes' geometry.
//
//   k_plan_sizes    1 thread / pass : sweep-memory bytes and row count
//   k_scan2         1 block         : exclusive prefix sums (u64) of both
//   k_plan_place    1 thread / pass : PassSweep, PassComp, sweep form, band
//                                     range
//   k_sort_*        sweep order     : passes by expected sweep length, longest
//                                     first (stable bucket sort)
//   k_bin_count     1 warp / segment: passes meeting a band (warp ballots)
//   k_scan2         1 block         : segment offsets
//   k_bin_fill      1 warp / segment: the bins, draw order kept by ballot ranks
//   k_sort_*        tile order      : compositor tiles by work, most first
//   k_plan_stats    1 thread / pass : span / fragment / edge totals
//
// A segment is one band of a canvas together with a run of at most
// kSegPasses of that canvas's passes; each band's bin is the concatenation
// of its segments' passes, so the bins come out in pass (= draw) order.
//
// The reference has no counterpart: its software canvas blends each draw's
// spans as soon as they are made (sw_span_brush.cc:66-106), so nothing needs
// binning there.  Which passes meet which band, and the order of a band's
// passes, are what the host planner (BuildBins, batch.h) computes; the
// orders of the sweeps and of the compositor's tiles only balance the load.
#include <cuda_runtime.h>

#include "kernels.cuh"
#include "sweep.cuh"

namespace skc {

namespace {

constexpr int kPlanThreads = 256;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kBinWarps = 4;

__device__ __forceinline__ unsigned long long Align256U(unsigned long long v) {
  return (v + 255ull) & ~255ull;
}

// Sweep bytes and rows of pass p (zero for a pass with nothing to sweep or
// whose geometry overflowed).
__device__ __forceinline__ void PassNeeds(const PassGeom& g, unsigned long long* bytes,
                                          unsigned long long* rows) {
  const int nr = g.row1 - g.row0;
  const bool has = g.status == 0 && g.n_edges > 0 && nr > 0;
  *bytes = has ? Align256U(SweepMemBytes(g.n_edges, g.acc_width > 0 ? g.acc_width : 0)) : 0ull;
  *rows = has ? (unsigned long long)nr : 0ull;
}

// Sort key of a work estimate: 0 for no work, else 8 buckets per octave
// (1 + 8 floor(log2 c) + the next three bits of c), at most kSortBuckets - 1:
// the orders below are by work to within about 9%, ties in index order.
constexpr uint32_t kSortBuckets = 512;
__device__ __forceinline__ uint32_t WorkBucket(unsigned long long c) {
  if (!c) return 0u;
  const uint32_t e = 63u - (uint32_t)__clzll(c);
  const uint32_t sub = e >= 3 ? (uint32_t)(c >> (e - 3)) & 7u : (uint32_t)(c << (3 - e)) & 7u;
  const uint32_t k = 1u + 8u * e + sub;
  return k < kSortBuckets ? k : kSortBuckets - 1u;
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_sizes(DevBatch b, DevPlan q) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= b.n_passes) return;
  const PassGeom g = b.geom[p];
  if (g.status != 0) {
    atomicOr(&q.st->flags, kPlanGeomOverflow);
    atomicAdd(&q.st->geom_overflows, 1u);
  }
  unsigned long long bytes, rows;
  PassNeeds(g, &bytes, &rows);
  q.a[p] = bytes;
  q.r[p] = rows;
}

// Exclusive prefix sums, in place, of a[0, n) and (if c) c[0, n); the totals
// go to *ta and *tc.  One block walks the arrays in tiles of
// kScanThreads * kScanItems elements, carrying the running totals.
__global__ void __launch_bounds__(kScanThreads)
    k_scan2(unsigned long long* a, unsigned long long* c, uint32_t n, unsigned long long* ta,
            unsigned long long* tc) {
  __shared__ unsigned long long wa[32], wc[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  unsigned long long carry_a = 0, carry_c = 0;
  for (uint32_t base = 0; base < n; base += kScanThreads * kScanItems) {
    unsigned long long va[kScanItems], vc[kScanItems], sa = 0, sc = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      const uint32_t i = base + (uint32_t)t * kScanItems + j;
      va[j] = i < n ? a[i] : 0ull;
      vc[j] = (c && i < n) ? c[i] : 0ull;
      sa += va[j];
      sc += vc[j];
    }
    unsigned long long ia = sa, ic = sc;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long xa = __shfl_up_sync(0xffffffffu, ia, o);
      const unsigned long long xc = __shfl_up_sync(0xffffffffu, ic, o);
      if (lane >= o) {
        ia += xa;
        ic += xc;
      }
    }
    if (lane == 31) {
      wa[w] = ia;
      wc[w] = ic;
    }
    __syncthreads();
    if (w == 0) {
      unsigned long long xa = wa[lane], xc = wc[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long ya = __shfl_up_sync(0xffffffffu, xa, o);
        const unsigned long long yc = __shfl_up_sync(0xffffffffu, xc, o);
        if (lane >= o) {
          xa += ya;
          xc += yc;
        }
      }
      wa[lane] = xa;
      wc[lane] = xc;
    }
    __syncthreads();
    unsigned long long pa = carry_a + (w ? wa[w - 1] : 0ull) + ia - sa;
    unsigned long long pc = carry_c + (w ? wc[w - 1] : 0ull) + ic - sc;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
      const uint32_t i = base + (uint32_t)t * kScanItems + j;
      if (i < n) {
        a[i] = pa;
        if (c) c[i] = pc;
      }
      pa += va[j];
      pc += vc[j];
    }
    carry_a += wa[31];
    carry_c += wc[31];
    __syncthreads();
  }
  if (t == 0) {
    *ta = carry_a;
    if (tc) *tc = carry_c;
  }
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_place(DevBatch b, DevPlan q) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < b.n_passes) {
    const PassGeom g = b.geom[p];
    const PassDesc& pd = b.passes[p];
    const uint32_t canvas = pd.canvas, brush = pd.brush;
    const CanvasDesc& cd = b.canvases[canvas];
    unsigned long long bytes, rows;
    PassNeeds(g, &bytes, &rows);
    const unsigned long long off = q.a[p], rb = q.r[p];
    bool has = bytes != 0;
    if (has) {
      uint32_t short_of = 0;
      if (off + bytes > q.sweep_cap) short_of |= kPlanSweepMem;
      if (rb + rows > q.rows_cap) short_of |= kPlanRows;
      if (short_of) {
        atomicOr(&q.st->flags, short_of);
        has = false;
      }
    }
    PassSweep sw;
    sw.work_off = off;
    sw.bytes = has ? bytes : 0ull;
    sw.rbase = (uint32_t)rb;
    sw.chunk = SpanChunk(cd.w, g.n_edges);
    ((PassSweep*)b.sweep)[p] = sw;
    PassComp pc;
    pc.row0 = has ? g.row0 : 0;
    pc.row1 = has ? g.row1 : 0;
    pc.rbase = (uint32_t)rb;
    pc.brush = brush;
    ((PassComp*)b.comp)[p] = pc;
    b.pass_class[p] = has ? (uint8_t)0 : kSweepSkip;
    const uint32_t s = (uint32_t)b.band_shift;
    q.pband[p] = has ? make_uint2(cd.band0 + ((uint32_t)g.row0 >> s),
                                  cd.band0 + ((uint32_t)(g.row1 - 1) >> s))
                     : make_uint2(1u, 0u);
  }
}

__global__ void __launch_bounds__(32 * kBinWarps) k_bin_count(DevPlan q) {
  const uint32_t seg = blockIdx.x * kBinWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (seg >= q.n_segs) return;
  const BandSeg sg = q.segs[seg];
  uint32_t cnt = 0;
  for (uint32_t pb = sg.p0; pb < sg.p1; pb += 32) {
    const uint32_t p = pb + lane;
    bool t = false;
    if (p < sg.p1) {
      const uint2 r = q.pband[p];
      t = r.x <= sg.band && sg.band <= r.y;
    }
    cnt += __popc(__ballot_sync(0xffffffffu, t));
  }
  if (lane == 0) q.seg_cnt[seg] = cnt;
}

__global__ void __launch_bounds__(32 * kBinWarps) k_bin_fill(DevPlan q) {
  const uint32_t seg = blockIdx.x * kBinWarps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (seg >= q.n_segs) return;
  const BandSeg sg = q.segs[seg];
  const unsigned long long off = q.seg_cnt[seg];
  const unsigned long long total = q.st->bins_need;
  if (lane == 0) {
    if (sg.first) q.band_off[sg.band] = (uint32_t)(off < q.bins_cap ? off : q.bins_cap);
    if (seg + 1 == q.n_segs) q.band_off[q.n_bands] = (uint32_t)(total < q.bins_cap ? total : q.bins_cap);
    if (seg + 1 == q.n_segs && total > q.bins_cap) atomicOr(&q.st->flags, kPlanBins);
  }
  unsigned long long at = off;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t pb = sg.p0; pb < sg.p1; pb += 32) {
    const uint32_t p = pb + lane;
    bool t = false;
    if (p < sg.p1) {
      const uint2 r = q.pband[p];
      t = r.x <= sg.band && sg.band <= r.y;
    }
    const uint32_t m = __ballot_sync(0xffffffffu, t);
    const unsigned long long pos = at + __popc(m & lt);
    if (t && pos < q.bins_cap) q.bins[pos] = p;
    at += __popc(m);
  }
}

// ---- stable descending bucket sort (sweep order and tile order) ----------
// Items are sorted by their key, heaviest first, items of equal key in index
// order: a counting sort over blocks of kSortItems items -- per-block key
// histograms, one prefix sum over (key descending, block), then each block
// places its items, warp by warp, ranking equal keys inside a warp with
// __match_any_sync.
constexpr int kSortThreads = 256;
constexpr int kSortItems = 2048;

// Key of item i: kind 0 the sweep of pass i (rows x (1 + active-list bound)),
// kind 1 compositor tile i (passes in its band's bin + 1) x its width; the
// temp canvases' tiles (i >= n_main) sort after every main tile.
__device__ __forceinline__ uint32_t SortKey(const DevBatch& b, const DevPlan& q, int kind,
                                            uint32_t i) {
  if (kind == 0) {
    const PassGeom g = b.geom[i];
    const unsigned long long rows = b.sweep[i].bytes ? (unsigned long long)(g.row1 - g.row0) : 0ull;
    return WorkBucket(rows * (unsigned long long)(1 + (g.max_active > 0 ? g.max_active : 0)));
  }
  const RowTask t = q.tasks_in[i];
  const CanvasDesc& cd = b.canvases[t.canvas];
  const uint32_t band = cd.band0 + (t.y >> b.band_shift);
  const unsigned long long n = q.band_off[band + 1] - q.band_off[band];
  const uint32_t k = WorkBucket((n + 1ull) * (unsigned long long)(t.x1 - t.x0));
  return i < q.n_main ? kSortBuckets + k : k;
}

// hist[(nb - 1 - key) * nblocks + block] = items of the block with that key
__global__ void __launch_bounds__(kSortThreads)
    k_sort_hist(DevBatch b, DevPlan q, int kind, uint32_t n, uint32_t nb) {
  __shared__ uint32_t h[2 * kSortBuckets];
  for (uint32_t k = threadIdx.x; k < nb; k += kSortThreads) h[k] = 0;
  __syncthreads();
  const uint32_t i0 = blockIdx.x * kSortItems;
  for (uint32_t j = threadIdx.x; j < kSortItems; j += kSortThreads) {
    const uint32_t i = i0 + j;
    if (i >= n) break;
    const uint32_t key = SortKey(b, q, kind, i);
    q.sort_keys[i] = (uint16_t)key;
    atomicAdd(&h[key], 1u);
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < nb; k += kSortThreads)
    q.sort_hist[(unsigned long long)(nb - 1 - k) * gridDim.x + blockIdx.x] = h[k];
}

__global__ void __launch_bounds__(kSortThreads)
    k_sort_place(DevPlan q, int kind, uint32_t n, uint32_t nb) {
  __shared__ uint32_t cur[2 * kSortBuckets];
  for (uint32_t k = threadIdx.x; k < nb; k += kSortThreads)
    cur[k] = (uint32_t)q.sort_hist[(unsigned long long)(nb - 1 - k) * gridDim.x + blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t i0 = blockIdx.x * kSortItems;
  for (uint32_t base = 0; base < (uint32_t)kSortItems; base += kSortThreads) {
    const uint32_t i = i0 + base + threadIdx.x;
    const bool valid = i < n;
    const uint32_t key = valid ? q.sort_keys[i] : 0xFFFFFFFFu;
    // warps of the round in order, so equal keys keep their index order
    for (int ww = 0; ww < kSortThreads / 32; ++ww) {
      if (w == ww) {
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (valid) {
          const uint32_t rank = __popc(peers & lt);
          const uint32_t pos = cur[key] + rank;
          if (kind == 0) q.sweep_order[pos] = i;
          else q.tasks_out[pos] = q.tasks_in[i];
          __syncwarp(peers);
          if ((peers >> lane) == 1u) cur[key] += __popc(peers);  // the group's last lane
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ unsigned long long WarpSum64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_stats(DevBatch b, DevPlan q) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long spans = 0, edges = 0, f[4] = {0, 0, 0, 0};
  if (p < b.n_passes) {
    const PassGeom g = b.geom[p];
    if (g.status == 0 && g.n_edges > 0) edges = (unsigned long long)g.n_edges;
    if (b.sweep[p].bytes) {
      spans = b.pass_spans[p];
      // sweep and two-point conical gradients count with the radial ones
      const uint32_t kind = b.brushes[b.passes[p].brush].kind;
      f[kind >= 4 ? 2 : kind] = b.pass_frags[p];
    }
  }
  spans = WarpSum64(spans);
  edges = WarpSum64(edges);
#pragma unroll
  for (int k = 0; k < 4; ++k) f[k] = WarpSum64(f[k]);
  if ((threadIdx.x & 31) == 0) {
    if (spans) atomicAdd(&q.st->spans, spans);
    if (edges) atomicAdd(&q.st->edges, edges);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (f[k]) atomicAdd(&q.st->frags_by_brush[k], f[k]);
  }
}

inline unsigned Blocks(uint64_t n, int per) { return (unsigned)((n + per - 1) / per); }

int LaunchSort(const DevBatch& b, const DevPlan& q, int kind, uint32_t n, uint32_t nb,
               cudaStream_t s) {
  const unsigned blocks = Blocks(n, kSortItems);
  k_sort_hist<<<blocks, kSortThreads, 0, s>>>(b, q, kind, n, nb);
  k_scan2<<<1, kScanThreads, 0, s>>>(q.sort_hist, nullptr, blocks * nb,
                                      kind == 0 ? &q.st->sort_total[0] : &q.st->sort_total[1],
                                      nullptr);
  k_sort_place<<<blocks, kSortThreads, 0, s>>>(q, kind, n, nb);
  return 3;
}

}  // namespace

int LaunchPlan(const DevBatch& b, const DevPlan& q, cudaStream_t s) {
  const uint32_t np = b.n_passes;
  int n = 0;
  if (np) {
    k_plan_sizes<<<Blocks(np, kPlanThreads), kPlanThreads, 0, s>>>(b, q);
    k_scan2<<<1, kScanThreads, 0, s>>>(q.a, q.r, np, &q.st->sweep_need, &q.st->rows_need);
    k_plan_place<<<Blocks(np, kPlanThreads), kPlanThreads, 0, s>>>(b, q);
    n += 3 + LaunchSort(b, q, 0, np, kSortBuckets, s);
  }
  if (q.n_segs) {
    k_bin_count<<<Blocks(q.n_segs, kBinWarps), 32 * kBinWarps, 0, s>>>(q);
    k_scan2<<<1, kScanThreads, 0, s>>>(q.seg_cnt, nullptr, q.n_segs, &q.st->bins_need, nullptr);
    k_bin_fill<<<Blocks(q.n_segs, kBinWarps), 32 * kBinWarps, 0, s>>>(q);
    n += 3;
  }
  const uint32_t nt = q.n_main + q.n_temp;
  if (nt) n += LaunchSort(b, q, 1, nt, 2 * kSortBuckets, s);
  return n;
}

int LaunchPlanStats(const DevBatch& b, const DevPlan& q, cudaStream_t s) {
  if (!b.n_passes) return 0;
  k_plan_stats<<<Blocks(b.n_passes, kPlanThreads), kPlanThreads, 0, s>>>(b, q);
  return 1;
}

}  // namespace skc
