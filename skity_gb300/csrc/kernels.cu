// GB300 kernels of the raster pipeline.
//
//   k_geometry   1 thread / pass : Path -> QuadPath (-> stroke -> QuadPath)
//                                  (1 to 32 passes a warp by the batch's size)
//                                  -> fixed-point edges -> introsort
//   k_sweep_*    1 warp / pass   : analytic-AA sweep (register form, generic
//                                  form for very long active lists) writing
//                                  each row's spans contiguously into the
//                                  span pool
//   k_composite  1 warp / row tile: replays the spans of the row band's
//                                  passes in draw order into a shared-memory
//                                  tile, then writes the tile back
//   k_blur_h/_v  1 thread / row / column of each blur temp canvas: StackBlur
//
// Geometry and sweeps are inherently sequential per path (the reference's
// scanline sweep carries state across rows), so the parallelism there is
// across paths; compositing is parallel across rows and, inside a row,
// across pixels with a fixed lane per pixel column (no cross-lane hazards).
#include <cuda_runtime.h>

#include <algorithm>


#include "passes.cuh"
#include "clip.cuh"

namespace skc {

// Geometry: lanes [0, lanes) of each warp take a pass each, the others idle.
// A pass's chain is long and branchy (curve subdivision, the stroker, edge
// set-up, the sort), so the lanes of a warp diverge on almost every verb:
// packing 32 passes a warp costs the least issue when there are passes
// enough to fill the GPU many times over, while a batch of few passes
// finishes sooner with fewer per warp (its time is its longest chains').
// Measured on the GB300: 32 a warp for the 256-canvas batch (135,670
// passes: 6.1 ms against 26.0 at 1), 8 for the 20,000-path scene (36.0 ms
// against 42.8 at 32), 1 for the 305-path tiger picture (7.8 ms against 10.2).
__global__ void __launch_bounds__(128) k_geometry(DevBatch b, uint32_t lanes) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = t & 31;
  if (lane >= lanes) return;
  const uint32_t i = (t >> 5) * lanes + lane;
  if (i >= b.n_list) return;
  GeometryPass(b, b.pass_list ? b.pass_list[i] : i);
}

// Passes per warp: n / (16 warps per SM over the SMs), a power of two in [1, 32].
static uint32_t GeometryLanes(uint32_t n) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
    cudaGetLastError();
    sms = 152;
  }
  const uint32_t per = n / (16u * (uint32_t)sms);
  uint32_t lanes = 1;
  while (lanes < 32 && lanes * 2 <= per) lanes *= 2;
  return lanes;
}

int LaunchGeometry(const DevBatch& b, cudaStream_t stream) {
  if (b.n_list == 0) return 0;
  const uint32_t lanes = GeometryLanes(b.n_list);
  const uint32_t warps = (b.n_list + lanes - 1) / lanes;
  k_geometry<<<(warps + 3) / 4, 128, 0, stream>>>(b, lanes);
  return 1;
}

// Sweeps: one warp per pass, passes taken in the batch's sweep order
// (longest expected sweeps first, so the long ones do not form the tail).
// Four forms, each launched over every pass and taking the ones SweepForm
// gives it: register forms for up to 32, 64 and 128 active edges (2 warps
// per block, each with its RegSharedT block and accumulator in shared
// memory), then the generic sweep (4 warps per block, state in global
// memory) for longer lists.
constexpr int kSweepWarps = 4;
constexpr int kRegWarpsMax = 4;  // warps per CTA of the register sweeps: DevBatch::reg_warps

__device__ __forceinline__ uint32_t DynamicSmemBytes() {
  uint32_t v;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(v));
  return v;
}

__device__ __forceinline__ uint32_t SweepPassAt(const DevBatch& b, uint32_t i) {
  return b.sweep_order ? b.sweep_order[i] : i;
}

// Lets the next overlapped launch start once every CTA of this one runs.
__device__ __forceinline__ void AllowNextLaunch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// End of a sweep kernel that may have overlapped the one before it: the
// CTA that finishes last waits for that kernel to complete, so this kernel
// completes only after every earlier sweep kernel has, and the work queued
// after the sweeps sees all of them done.  (In a launch that overlapped
// nothing the wait returns at once.)
__device__ __forceinline__ void FinishOverlapped(unsigned int* done) {
  if (!done) return;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(done, 1u) == gridDim.x - 1) asm volatile("griddepcontrol.wait;" ::: "memory");
  }
}

template <int M, int kForm>
__global__ void __launch_bounds__(32 * kRegWarpsMax) k_sweep_reg(DevBatch b) {
  extern __shared__ __align__(16) uint8_t reg_smem[];
  AllowNextLaunch();
  const int w = threadIdx.x >> 5;
  const uint32_t nw = blockDim.x >> 5;
  const uint32_t i = blockIdx.x * nw + w;
  if (i < b.n_passes) {
    const uint32_t p = SweepPassAt(b, i);
    if (SweepForm(b.geom[p], b.pass_class[p]) == kForm) {
      if (DynamicSmemBytes() < nw * RegSmemBytes<M>(b.reg_diff_cap)) {  // self-check
        FlagError(b.err, 16);
      } else {
        Lanes L;
        L.lane = threadIdx.x & 31;
        uint8_t* mine = reg_smem + (size_t)w * RegSmemBytes<M>(b.reg_diff_cap);
        if (!SweepPassReg<M>(b, p, L, (RegSharedT<M>*)mine,
                             (int32_t*)(mine + sizeof(RegSharedT<M>)), b.reg_diff_cap) &&
            L.leader()) {
          // each pass is taken by one form, so the list holds at most n_passes
          const uint32_t at = b.sweep_retry ? atomicAdd(b.sweep_retry, 1u) : b.n_passes;
          if (at < b.n_passes) {
            b.sweep_retry[1 + at] = p;
          } else {
            FlagError(b.err, 32);  // no list: the pass stays unswept, the render fails
          }
        }
      }
    }
  }
  FinishOverlapped(b.sweep_done ? b.sweep_done + (kForm & 3) : nullptr);
}

// The passes the register forms gave up on, swept with the generic form after
// every register form has finished (a plain launch after them).
__global__ void __launch_bounds__(32 * kSweepWarps) k_sweep_retry(DevBatch b) {
  if (!b.sweep_retry) return;
  const uint32_t n = min(b.sweep_retry[0], b.n_passes);
  const uint32_t nw = gridDim.x * kSweepWarps;
  Lanes L;
  L.lane = threadIdx.x & 31;
  for (uint32_t i = blockIdx.x * kSweepWarps + (threadIdx.x >> 5); i < n; i += nw)
    SweepPass(b, b.sweep_retry[1 + i], L);
}

template <bool kRaw>
__global__ void __launch_bounds__(32 * kSweepWarps) k_sweep(DevBatch b) {
  AllowNextLaunch();
  const uint32_t i = blockIdx.x * kSweepWarps + (threadIdx.x >> 5);
  if (i < b.n_passes) {
    const uint32_t p = SweepPassAt(b, i);
    Lanes L;
    L.lane = threadIdx.x & 31;
    if (SweepForm(b.geom[p], b.pass_class[p]) == kSweepGeneric) SweepPass<kRaw>(b, p, L);
  }
  FinishOverlapped(b.sweep_done ? b.sweep_done + kSweepGeneric : nullptr);
}

// Launch with programmatic stream serialization: the kernel may start as
// soon as every CTA of the kernel before it has started (and signalled, at
// its beginning), so it fills the SMs that kernel's tail leaves idle.  The
// sweep forms take disjoint passes and read nothing the others write.
template <typename... Args>
static void LaunchOverlapped(void (*kernel)(Args...), dim3 grid, dim3 block, size_t smem,
                             cudaStream_t stream, bool overlap, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = overlap ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int M, int kForm>
static void LaunchRegForm(const DevBatch& b, cudaStream_t stream, bool overlap) {
  const uint32_t nw = b.reg_warps == 1 || b.reg_warps == 4 ? b.reg_warps : 2;
  const size_t smem = nw * RegSmemBytes<M>(b.reg_diff_cap);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_sweep_reg<M, kForm>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
  LaunchOverlapped(k_sweep_reg<M, kForm>, dim3((b.n_passes + nw - 1) / nw), dim3(32 * nw), smem,
                   stream, overlap, b);
}

// With b.sweep_done (four zeroed counters) the later forms overlap the
// earlier ones' tails; without, they run one after the other.
int LaunchSweep(const DevBatch& b, cudaStream_t stream) {
  if (b.n_passes == 0) return 0;
  // heaviest form first: the longest sweeps start at once, and each later
  // (lighter) form fills the SMs the earlier ones' tails leave idle
  const bool overlap = b.sweep_done != nullptr;
  // path-clip passes (raw spans) come only with clip states
  LaunchOverlapped(b.n_clip_states ? k_sweep<true> : k_sweep<false>,
                   dim3((b.n_passes + kSweepWarps - 1) / kSweepWarps),
                   dim3(32 * kSweepWarps), 0, stream, false, b);
  LaunchRegForm<kRegMaxM, kSweepReg128>(b, stream, overlap);
  LaunchRegForm<64, kSweepReg64>(b, stream, overlap);
  LaunchRegForm<32, kSweepReg32>(b, stream, overlap);
  k_sweep_retry<<<64, 32 * kSweepWarps, 0, stream>>>(b);
  return 5;
}

// ---------------------------------------------------------------------------
// composite: one warp per row tile (x0, x1) of a canvas row, the tile held in
// shared memory.  The passes come from the row band's bin (draw order); each
// pass row's spans are loaded 32 at a time, the ones meeting the tile are
// applied in emission order, in batches of disjoint spans (every pixel's
// blends stay in the reference's order).
// ---------------------------------------------------------------------------
constexpr int kCompWarps = 4;
// CTAs per SM the compositor's register budget leaves room for (its stalls
// are mostly dependent integer chains: more resident warps hide them)
constexpr int kCompMinBlocks = 6;
// spans up to this many tile pixels are shaded by one lane
constexpr int kShortSpan = 4;

// gradient stops a warp stages in shared memory (longer gradients are read
// from global memory)
constexpr int kStagedStops = 16;
// shared memory of one compositor warp: its tile row, then the staged stops
__host__ __device__ constexpr size_t CompWarpSmem(uint32_t chunk) {
  return (size_t)chunk * 4 + kStagedStops * (16 + 4);
}

template <bool kAll>
__device__ __forceinline__ void CompositeTile(const DevBatch& b, const RowTask& rt, uint32_t* row,
                                              float4* stage_colors, float* stage_offsets,
                                              int lane);

// counter == null: warp w of block k takes tile 4k + w; otherwise every warp
// takes tiles from the counter until none is left (persistent grid).
// kAll: the general form (every brush kind, colour filter and blend mode),
// launched for batches with a general canvas; the common form has no calls
// and keeps its loops in registers.
template <bool kAll>
__global__ void __launch_bounds__(32 * kCompWarps, kCompMinBlocks)
    k_composite(DevBatch b, const RowTask* __restrict__ tasks, uint32_t n_tasks, uint32_t chunk,
                unsigned int* counter) {
  extern __shared__ __align__(16) uint8_t reg_smem[];
  // a device plan that fell short: the host grows its buffers and renders
  // again, so nothing is composited from it
  if (b.plan && b.plan->flags) return;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint8_t* mine = reg_smem + (size_t)wib * CompWarpSmem(chunk);
  uint32_t* row = (uint32_t*)mine;
  float4* stage_colors = (float4*)(mine + (size_t)chunk * 4);
  float* stage_offsets = (float*)(stage_colors + kStagedStops);
  if (!counter) {
    const uint32_t task = blockIdx.x * kCompWarps + wib;
    if (task < n_tasks) CompositeTile<kAll>(b, tasks[task], row, stage_colors, stage_offsets, lane);
    return;
  }
  for (;;) {
    uint32_t task = 0;
    if (lane == 0) task = atomicAdd(counter, 1u);
    task = __shfl_sync(0xffffffffu, task, 0);
    if (task >= n_tasks) return;
    CompositeTile<kAll>(b, tasks[task], row, stage_colors, stage_offsets, lane);
    __syncwarp();
  }
}

// The spans [s0, s1) of one pass row applied to the row tile.  kAll: every
// brush kind, colour filter and blend mode; otherwise the common ones only
// (solid, linear, radial and image brushes; clear, src, dst, src-over).
template <bool kAll>
__device__ __forceinline__ void CompositeSpans(const DevBatch& b, const Brush& br,
                                               const float4* stop_colors,
                                               const float* stop_offsets, uint32_t s0,
                                               uint32_t s1, int x0, int x1, int y, uint32_t* row,
                                               int lane) {
  const uint2* sp = b.spans;
  for (uint32_t sb = s0; sb < s1; sb += 32) {
    int xs = 0, xe = 0;
    uint32_t alpha = 0;
    bool pending = false;
    if (sb + lane < s1) {
      const uint2 mine = sp[sb + lane];
      const int sx = (int)(mine.x & 0xFFFF), slen = (int)(mine.x >> 16);
      xs = max(sx, x0);
      xe = min(sx + slen, x1);
      alpha = mine.y & br.global_alpha;
      pending = xs < xe;
    }
    // Spans are applied in batches: the longest run of pending spans
    // (in emission order) in which each starts at or after the end of
    // the one before.  Those are disjoint, so inside a batch the order
    // does not matter: short spans are shaded by their own lane, long
    // ones by the whole warp (pixel column mod 32 per lane).
    uint32_t pmask = __ballot_sync(0xffffffffu, pending);
    while (pmask) {
      const uint32_t below = pmask & ((1u << lane) - 1u);
      const int prev = below ? 31 - __clz(below) : lane;
      const int prev_xe = __shfl_sync(0xffffffffu, xe, prev);
      const bool clash = pending && below && prev_xe > xs;
      const uint32_t cmask = __ballot_sync(0xffffffffu, clash);
      const uint32_t batch = cmask ? pmask & ((1u << (__ffs(cmask) - 1)) - 1u) : pmask;
      const bool mine_now = (batch >> lane) & 1u;
      const bool is_short = xe - xs <= kShortSpan;
      if (mine_now && is_short) {
        for (int x = xs; x < xe; ++x) {
          uint32_t c = kAll ? BrushColor(br, x, y, stop_colors, stop_offsets, b.pixels,
                                         b.roundtrip, b.conicals)
                            : BrushColorCommon(br, x, y, stop_colors, stop_offsets, b.pixels,
                                               b.roundtrip);
          if (alpha != 255) c = AlphaMulQ(c, alpha);
          if (kAll && br.cf_type) c = FilterColor(br, c, b.srgb_tables, b.cf_matrices);
          uint32_t& d = row[x - x0];
          d = kAll ? BlendPixel(d, c, br.blend) : BlendPixelCommon(d, c, br.blend);
        }
      }
      uint32_t lmask = __ballot_sync(0xffffffffu, mine_now && !is_short);
      while (lmask) {
        const int j = __ffs(lmask) - 1;
        lmask &= lmask - 1;
        const int qs = __shfl_sync(0xffffffffu, xs, j);
        const int qe = __shfl_sync(0xffffffffu, xe, j);
        const uint32_t qa = __shfl_sync(0xffffffffu, alpha, j);
        for (int x = qs + ((lane - qs) & 31); x < qe; x += 32) {
          uint32_t c = kAll ? BrushColor(br, x, y, stop_colors, stop_offsets, b.pixels,
                                         b.roundtrip, b.conicals)
                            : BrushColorCommon(br, x, y, stop_colors, stop_offsets, b.pixels,
                                               b.roundtrip);
          if (qa != 255) c = AlphaMulQ(c, qa);
          if (kAll && br.cf_type) c = FilterColor(br, c, b.srgb_tables, b.cf_matrices);
          uint32_t& d = row[x - x0];
          d = kAll ? BlendPixel(d, c, br.blend) : BlendPixelCommon(d, c, br.blend);
        }
      }
      __syncwarp();
      if (mine_now) pending = false;
      pmask &= ~batch;
    }
  }
}

template <bool kAll>
__device__ __forceinline__ void CompositeTile(const DevBatch& b, const RowTask& rt, uint32_t* row,
                                              float4* stage_colors, float* stage_offsets,
                                              int lane) {
  const CanvasDesc cd = b.canvases[rt.canvas];
  const int y = (int)rt.y;
  const int x0 = (int)rt.x0, x1 = (int)rt.x1;
  const int n = x1 - x0;
  uint32_t* gpx = (uint32_t*)(b.pixels + cd.px_off) + (size_t)y * cd.w + x0;
  for (int i = lane; i < n; i += 32) {
    row[i] = cd.has_clear ? cd.clear_pm : RGBAtoARGB(gpx[i]);
  }
  __syncwarp();
  const uint32_t band = cd.band0 + ((uint32_t)y >> b.band_shift);
  const uint32_t e0 = b.band_off[band], e1 = b.band_off[band + 1];
  // 32 bin entries at a time: each lane looks up its pass's row entry, so
  // the row-table loads of 32 passes are in flight together and passes
  // with no spans on this row cost no serial step
  for (uint32_t eb = e0; eb < e1; eb += 32) {
    const uint32_t e = eb + lane;
    uint2 rs = make_uint2(0, 0);
    uint32_t brush = 0;
    if (e < e1) {
      const PassComp pc = b.comp[b.bins[e]];
      if (y >= pc.row0 && y < pc.row1) {
        rs = b.rowspan[pc.rbase + (y - pc.row0)];
        brush = pc.brush;
      }
    }
    uint32_t mask = __ballot_sync(0xffffffffu, rs.y != 0);
    while (mask) {
      const int bit = __ffs(mask) - 1;
      mask &= mask - 1;
      const uint32_t s0 = __shfl_sync(0xffffffffu, rs.x, bit);
      const uint32_t s1 = s0 + __shfl_sync(0xffffffffu, rs.y, bit);
      const uint32_t qbrush = __shfl_sync(0xffffffffu, brush, bit);
      Brush br = b.brushes[qbrush];
      const float4* stop_colors = b.stop_colors;
      const float* stop_offsets = b.stop_offsets;
      if ((br.kind == 1 || br.kind == 2) && br.stop_count <= (uint32_t)kStagedStops) {
        // the gradient's stops, read for every pixel, staged in shared memory
        __syncwarp();
        if (lane < (int)br.stop_count) {
          stage_colors[lane] = b.stop_colors[br.stop0 + lane];
          stage_offsets[lane] = b.stop_offsets[br.stop0 + lane];
        }
        __syncwarp();
        stop_colors = stage_colors;
        stop_offsets = stage_offsets;
        br.stop0 = 0;
      }
      CompositeSpans<kAll>(b, br, stop_colors, stop_offsets, s0, s1, x0, x1, y, row, lane);
    }
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) gpx[i] = ARGBtoRGBA(row[i]);
}

int LaunchComposite(const DevBatch& b, const RowTask* tasks, uint32_t n_tasks, uint32_t chunk,
                    uint32_t ctas_per_sm, uint32_t num_sms, unsigned int* counter,
                    cudaStream_t stream) {
  if (n_tasks == 0) return 0;
  size_t smem = (size_t)kCompWarps * CompWarpSmem(chunk);
  auto kernel = b.any_general ? k_composite<true> : k_composite<false>;
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  uint32_t grid = (n_tasks + kCompWarps - 1) / kCompWarps;
  if (ctas_per_sm > 0 && counter) {
    grid = std::min<uint32_t>(grid, ctas_per_sm * std::max<uint32_t>(num_sms, 1));
  } else {
    counter = nullptr;
  }
  kernel<<<grid, 32 * kCompWarps, smem, stream>>>(b, tasks, n_tasks, chunk, counter);
  return 1;
}

// ---------------------------------------------------------------------------
// Path clips (clip.cuh): each clip state's span rows, one launch per state
// in order (a state reads its parent's rows and whether the parent's list
// is empty, known only once the parent's launch is complete), then the rows
// of the draws under a clip, one thread per (pass, row).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_clip_state(DevBatch b, uint32_t k, int32_t y0, int32_t y1) {
  const int32_t y = y0 + (int32_t)(blockIdx.x * blockDim.x + threadIdx.x);
  if (y >= y1) return;
  int32_t order[kClipRowCap];
  ClipStateStage(b, k, y, order);
}

__global__ void __launch_bounds__(128) k_clip_apply(DevBatch b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n_clip_items) return;
  int32_t order[kClipRowCap];
  ClipApplyStage(b, i, order);
}

int LaunchPathClips(const DevBatch& b, const ClipStateDesc* states, uint32_t n_states,
                    cudaStream_t stream) {
  int launches = 0;
  for (uint32_t k = 1; k <= n_states; ++k) {
    const ClipStateDesc& st = states[k - 1];
    if (st.y1 <= st.y0) continue;
    const uint32_t rows = (uint32_t)(st.y1 - st.y0);
    k_clip_state<<<(rows + 127) / 128, 128, 0, stream>>>(b, k, st.y0, st.y1);
    launches++;
  }
  if (b.n_clip_items) {
    k_clip_apply<<<(b.n_clip_items + 127) / 128, 128, 0, stream>>>(b);
    launches++;
  }
  return launches;
}

// ---------------------------------------------------------------------------
// StackBlur (src/render/sw/sw_stack_blur.cc:18-284) on blur temp canvases.
// The reference's ring buffer only ever holds input pixels at clamped
// indices, so each step reads them directly: the value leaving the left half
// is pixel(max(i - r, 0)), the one entering is pixel(min(i + r + 1, n - 1)),
// the one crossing the centre is pixel(min(i + 1, n - 1)).  Horizontal pass:
// canvas -> blur scratch; vertical pass: blur scratch -> canvas.
// ---------------------------------------------------------------------------
// Staged StackBlur: a block copies a run of whole rows (horizontal pass) or
// a 32-column strip of every row (vertical pass) of one temp canvas into
// shared memory with coalesced 4-byte loads -- the rows are contiguous in
// memory, and 32 lanes cover 128 contiguous bytes of a strip row -- blurs
// each line there with one thread per line (BlurLine, the same arithmetic
// as the direct kernels above), and writes the result back coalesced.
// Lines are stored an odd number of words apart, so the threads, each
// walking its own line, hit distinct banks.  Temp canvases whose lines do
// not fit the shared-memory budget take the direct kernels (they return at
// once for the staged ones, and the staged ones for them).
constexpr int kBlurThreads = 64;
constexpr uint32_t kBlurSmemWords = 12 * 1024;  // 48 KiB: input and output lines

__host__ __device__ inline uint32_t OddStride(uint32_t n) { return n | 1u; }
// Rows per block of the staged horizontal pass (0: the row does not fit).
__host__ __device__ inline uint32_t BlurRowsPerBlock(uint32_t w) {
  const uint32_t r = kBlurSmemWords / (2 * OddStride(w));
  return r < (uint32_t)kBlurThreads ? r : (uint32_t)kBlurThreads;
}
// The staged vertical pass takes canvases whose 32-column strip fits.
__host__ __device__ inline bool BlurStripFits(uint32_t h) {
  return 2ull * OddStride(32) * h <= kBlurSmemWords;
}

__global__ void k_blur_h(DevBatch b, const uint32_t* temps, uint32_t n_temp, uint32_t max_h) {
  uint32_t t = blockIdx.y;
  uint32_t yrow = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_temp) return;
  const CanvasDesc cd = b.canvases[temps[t]];
  // staged, or a layer's temp canvas (no blur)
  if (yrow >= cd.h || BlurRowsPerBlock(cd.w) != 0 || cd.blur_style == 0) return;
  const uint8_t* src = b.pixels + cd.px_off + (size_t)yrow * cd.w * 4;
  uint8_t* dst = b.pixels + cd.blur_off + (size_t)yrow * cd.w * 4;
  int r = min(cd.blur_radius, 254);
  if (r <= 1) {
    for (uint32_t i = 0; i < cd.w * 4; ++i) dst[i] = src[i];
    return;
  }
  BlurLine(src, dst, (int)cd.w, 1, r, false);
}

__global__ void k_blur_v(DevBatch b, const uint32_t* temps, uint32_t n_temp, uint32_t max_w) {
  uint32_t t = blockIdx.y;
  uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_temp) return;
  const CanvasDesc cd = b.canvases[temps[t]];
  if (x >= cd.w || BlurStripFits(cd.h) || cd.blur_style == 0) return;  // staged, or a layer
  int r = min(cd.blur_radius, 254);
  const uint8_t* src = b.pixels + cd.blur_off + (size_t)x * 4;
  uint8_t* dst = b.pixels + cd.out_off + (size_t)x * 4;
  if (r <= 1) {
    for (uint32_t yy = 0; yy < cd.h; ++yy)
      for (int c = 0; c < 4; ++c) dst[(size_t)yy * cd.w * 4 + c] = src[(size_t)yy * cd.w * 4 + c];
    return;
  }
  BlurLine(src, dst, (int)cd.h, cd.w, r, true);
}

// MaskFilterOnFilter's styles (mask_filter.cc:61-100) for the temp canvases
// that are not kNormal: the blurred image (out_off) against the unblurred
// one (px_off), per pixel, in place in out_off.  One thread per pixel; the
// grid's y is the temp canvas.
__global__ void k_blur_style(DevBatch b, const uint32_t* temps, uint32_t n_temp) {
  const uint32_t t = blockIdx.y;
  if (t >= n_temp) return;
  const CanvasDesc cd = b.canvases[temps[t]];
  if (cd.blur_style <= 1) return;
  const uint64_t n = (uint64_t)cd.w * cd.h;
  const uint32_t* raw = (const uint32_t*)(b.pixels + cd.px_off);
  uint32_t* out = (uint32_t*)(b.pixels + cd.out_off);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = ARGBtoRGBA(BlurStylePixel(cd.blur_style, RGBAtoARGB(raw[i]), RGBAtoARGB(out[i])));
}

__global__ void __launch_bounds__(kBlurThreads)
    k_blur_h_staged(DevBatch b, const uint32_t* temps, uint32_t n_temp) {
  extern __shared__ uint32_t bsm[];
  const uint32_t t = blockIdx.y;
  if (t >= n_temp) return;
  const CanvasDesc cd = b.canvases[temps[t]];
  const uint32_t rows = BlurRowsPerBlock(cd.w);
  if (rows == 0 || cd.blur_style == 0) return;  // direct pass, or a layer (no blur)
  const uint32_t y0 = blockIdx.x * rows;
  if (y0 >= cd.h) return;
  const uint32_t nr = min(rows, cd.h - y0);
  const uint32_t ws = OddStride(cd.w);
  uint32_t* in = bsm;
  uint32_t* out = bsm + rows * ws;
  const uint32_t* src = (const uint32_t*)(b.pixels + cd.px_off) + (size_t)y0 * cd.w;
  uint32_t* dst = (uint32_t*)(b.pixels + cd.blur_off) + (size_t)y0 * cd.w;
  const uint32_t n = nr * cd.w;
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) in[(i / cd.w) * ws + i % cd.w] = src[i];
  __syncthreads();
  const int r = min(cd.blur_radius, 254);
  if (threadIdx.x < nr) {
    const uint32_t* li = in + threadIdx.x * ws;
    uint32_t* lo = out + threadIdx.x * ws;
    if (r <= 1) {
      for (uint32_t x = 0; x < cd.w; ++x) lo[x] = li[x];
    } else {
      BlurLine((const uint8_t*)li, (uint8_t*)lo, (int)cd.w, 1, r, false);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = out[(i / cd.w) * ws + i % cd.w];
}

__global__ void __launch_bounds__(32)
    k_blur_v_staged(DevBatch b, const uint32_t* temps, uint32_t n_temp) {
  extern __shared__ uint32_t bsm[];
  const uint32_t t = blockIdx.y;
  if (t >= n_temp) return;
  const CanvasDesc cd = b.canvases[temps[t]];
  if (!BlurStripFits(cd.h) || cd.blur_style == 0) return;  // direct pass, or a layer
  const uint32_t x0 = blockIdx.x * 32;
  if (x0 >= cd.w) return;
  const uint32_t nc = min(32u, cd.w - x0);
  const uint32_t ws = OddStride(32);
  uint32_t* in = bsm;
  uint32_t* out = bsm + cd.h * ws;
  const uint32_t* src = (const uint32_t*)(b.pixels + cd.blur_off) + x0;
  uint32_t* dst = (uint32_t*)(b.pixels + cd.out_off) + x0;
  const uint32_t lane = threadIdx.x;
  for (uint32_t y = 0; y < cd.h; ++y)
    if (lane < nc) in[y * ws + lane] = src[(size_t)y * cd.w + lane];
  __syncwarp();
  const int r = min(cd.blur_radius, 254);
  if (lane < nc) {
    if (r <= 1) {
      for (uint32_t y = 0; y < cd.h; ++y) out[y * ws + lane] = in[y * ws + lane];
    } else {
      BlurLine((const uint8_t*)(in + lane), (uint8_t*)(out + lane), (int)cd.h, ws, r, true);
    }
  }
  __syncwarp();
  for (uint32_t y = 0; y < cd.h; ++y)
    if (lane < nc) dst[(size_t)y * cd.w + lane] = out[y * ws + lane];
}

int LaunchBlur(const DevBatch& b, const uint32_t* temps, uint32_t n_temp, uint32_t max_h,
               uint32_t max_w, uint32_t max_style, cudaStream_t stream) {
  // no blurred temp canvases (the temps are layers): nothing to blur
  if (n_temp == 0 || max_w == 0 || max_h == 0) return 0;
  // staged passes (their blocks for canvases that do not fit return at once)
  const uint32_t min_rows = std::max<uint32_t>(BlurRowsPerBlock(max_w), 1);
  dim3 gsh((max_h + min_rows - 1) / min_rows, n_temp);
  const uint32_t smem_h = std::min<uint32_t>(2u * kBlurThreads * OddStride(max_w), kBlurSmemWords);
  k_blur_h_staged<<<gsh, kBlurThreads, smem_h * 4, stream>>>(b, temps, n_temp);
  // direct passes for the canvases the staged ones do not take
  int n = 1;
  if (BlurRowsPerBlock(max_w) == 0) {
    dim3 gh((max_h + 63) / 64, n_temp);
    k_blur_h<<<gh, 64, 0, stream>>>(b, temps, n_temp, max_h);
    n++;
  }
  dim3 gsv((max_w + 31) / 32, n_temp);
  const uint32_t smem_v = (uint32_t)std::min<uint64_t>(2ull * OddStride(32) * max_h, kBlurSmemWords);
  k_blur_v_staged<<<gsv, 32, smem_v * 4, stream>>>(b, temps, n_temp);
  n++;
  if (!BlurStripFits(max_h)) {
    dim3 gv((max_w + 63) / 64, n_temp);
    k_blur_v<<<gv, 64, 0, stream>>>(b, temps, n_temp, max_w);
    n++;
  }
  if (max_style <= 1) return n;  // kNormal blurs in place: nothing to combine
  const uint64_t px = (uint64_t)max_w * max_h;
  dim3 gs((unsigned)std::min<uint64_t>((px + 255) / 256, 1024), n_temp);
  k_blur_style<<<gs, 256, 0, stream>>>(b, temps, n_temp);
  return n + 1;
}

}  // namespace skc
