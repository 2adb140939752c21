// GB300 kernels of the raster pipeline.
//
//   k_geometry   1 thread / pass : Path -> QuadPath (-> stroke -> QuadPath)
//                                  -> fixed-point edges -> introsort
//   k_sweep_*    1 warp / pass   : analytic-AA sweep (register form, generic
//                                  form for very long active lists) writing
//                                  each row's spans contiguously into the
//                                  span pool
//   k_composite  1 warp / row     : replays every pass's spans of the row in
//                                  draw order into a shared-memory row, then
//                                  writes the row back (16-byte stores)
//   k_blur_h/_v  1 thread / row / column of each blur temp canvas: StackBlur
//
// Geometry and sweeps are inherently sequential per path (the reference's
// scanline sweep carries state across rows), so the parallelism there is
// across paths; compositing is parallel across rows and, inside a row,
// across pixels with a fixed lane per pixel column (no cross-lane hazards).
#include <cuda_runtime.h>


#include "passes.cuh"

namespace skc {

__global__ void __launch_bounds__(128) k_geometry(DevBatch b) {
  uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_list) return;
  GeometryPass(b, b.pass_list ? b.pass_list[t] : t);
}

int LaunchGeometry(const DevBatch& b, cudaStream_t stream) {
  if (b.n_list == 0) return 0;
  k_geometry<<<(b.n_list + 127) / 128, 128, 0, stream>>>(b);
  return 1;
}

// Sweeps: one warp per pass.  The register sweep takes every pass whose
// active list fits kRegMaxM edges (2 warps per block, each with its
// RegShared block and accumulator in shared memory); the generic sweep
// (4 warps per block, state in global memory) takes the passes the count
// kernel marked, after the register kernels.
constexpr int kSweepWarps = 4;
constexpr int kRegWarps = 2;

__device__ __forceinline__ uint32_t DynamicSmemBytes() {
  uint32_t v;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(v));
  return v;
}

__global__ void __launch_bounds__(32 * kRegWarps) k_sweep_reg(DevBatch b) {
  extern __shared__ __align__(16) uint8_t reg_smem[];
  const int w = threadIdx.x >> 5;
  const uint32_t p = blockIdx.x * kRegWarps + w;
  if (p >= b.n_passes) return;
  if (DynamicSmemBytes() < kRegWarps * RegSmemBytes(b.reg_diff_cap)) {  // self-check
    FlagError(b.err, 16);
    return;
  }
  Lanes L;
  L.lane = threadIdx.x & 31;
  uint8_t* mine = reg_smem + (size_t)w * RegSmemBytes(b.reg_diff_cap);
  SweepPassReg(b, p, L, (RegShared*)mine, (int32_t*)(mine + sizeof(RegShared)), b.reg_diff_cap);
}

__global__ void __launch_bounds__(32 * kSweepWarps) k_sweep(DevBatch b) {
  uint32_t p = blockIdx.x * kSweepWarps + (threadIdx.x >> 5);
  Lanes L;
  L.lane = threadIdx.x & 31;
  if (p < b.n_passes && b.pass_class[p] == 1) SweepPass(b, p, L);
}

int LaunchSweep(const DevBatch& b, cudaStream_t stream) {
  if (b.n_passes == 0) return 0;
  const size_t smem = kRegWarps * RegSmemBytes(b.reg_diff_cap);
  k_sweep_reg<<<(b.n_passes + kRegWarps - 1) / kRegWarps, 32 * kRegWarps, smem, stream>>>(b);
  k_sweep<<<(b.n_passes + kSweepWarps - 1) / kSweepWarps, 32 * kSweepWarps, 0, stream>>>(b);
  return 2;
}

// ---------------------------------------------------------------------------
// composite: one warp per row task, the row held in shared memory
// ---------------------------------------------------------------------------
constexpr int kCompWarps = 4;

__global__ void __launch_bounds__(32 * kCompWarps)
    k_composite(DevBatch b, const RowTask* __restrict__ tasks, uint32_t n_tasks, uint32_t chunk) {
  extern __shared__ __align__(16) uint8_t reg_smem[];
  uint32_t* smem = (uint32_t*)reg_smem;
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  uint32_t task = blockIdx.x * kCompWarps + wib;
  if (task >= n_tasks) return;
  const RowTask rt = tasks[task];
  const CanvasDesc cd = b.canvases[rt.canvas];
  uint32_t* row = smem + wib * chunk;
  const int y = (int)rt.y;
  const int x0 = (int)rt.x0, x1 = (int)rt.x1;
  const int n = x1 - x0;
  uint32_t* gpx = (uint32_t*)(b.pixels + cd.px_off) + (size_t)y * cd.w + x0;
  for (int i = lane; i < n; i += 32) {
    row[i] = cd.has_clear ? cd.clear_pm : RGBAtoARGB(gpx[i]);
  }
  __syncwarp();
  for (uint32_t pb = cd.pass0; pb < cd.pass1; pb += 32) {
    uint32_t p = pb + lane;
    bool hit = false;
    PassComp pc;
    pc.row0 = pc.row1 = 0;
    pc.rbase = pc.brush = 0;
    if (p < cd.pass1) {
      pc = b.comp[p];
      hit = y >= pc.row0 && y < pc.row1;
    }
    uint32_t mask = __ballot_sync(0xffffffffu, hit);
    while (mask) {
      int bit = __ffs(mask) - 1;
      mask &= mask - 1;
      const int32_t qrow0 = __shfl_sync(0xffffffffu, pc.row0, bit);
      const uint32_t qrbase = __shfl_sync(0xffffffffu, pc.rbase, bit);
      const uint32_t qbrush = __shfl_sync(0xffffffffu, pc.brush, bit);
      const uint2 rs = b.rowspan[qrbase + (y - qrow0)];
      const uint32_t s0 = rs.x, s1 = rs.x + rs.y;
      if (s0 == s1) continue;
      const Brush br = b.brushes[qbrush];
      const uint2* sp = b.spans;
      for (uint32_t sb = s0; sb < s1; sb += 32) {
        uint2 mine = make_uint2(0, 0);
        if (sb + lane < s1) mine = sp[sb + lane];
        const int cnt = (int)min(32u, s1 - sb);
        for (int j = 0; j < cnt; ++j) {
          const uint32_t xs_len = __shfl_sync(0xffffffffu, mine.x, j);
          const uint32_t cover = __shfl_sync(0xffffffffu, mine.y, j);
          const int sx = (int)(xs_len & 0xFFFF);
          const int slen = (int)(xs_len >> 16);
          const int xs = max(sx, x0), xe = min(sx + slen, x1);
          if (xs >= xe) continue;
          const uint32_t alpha = cover & br.global_alpha;
          // each lane owns the pixels whose column is lane mod 32
          for (int x = xs + ((lane - xs) & 31); x < xe; x += 32) {
            uint32_t c = BrushColor(br, x, y, b.stop_colors, b.stop_offsets, b.pixels, b.roundtrip);
            if (alpha != 255) c = AlphaMulQ(c, alpha);
            uint32_t& d = row[x - x0];
            d = BlendPixel(d, c, br.blend);
          }
        }
      }
    }
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) gpx[i] = ARGBtoRGBA(row[i]);
}

int LaunchComposite(const DevBatch& b, const RowTask* tasks, uint32_t n_tasks, uint32_t chunk,
                    cudaStream_t stream) {
  if (n_tasks == 0) return 0;
  size_t smem = (size_t)kCompWarps * chunk * sizeof(uint32_t);
  if (smem > 48 * 1024) {
    cudaFuncSetAttribute(k_composite, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  k_composite<<<(n_tasks + kCompWarps - 1) / kCompWarps, 32 * kCompWarps, smem, stream>>>(
      b, tasks, n_tasks, chunk);
  return 1;
}

// ---------------------------------------------------------------------------
// StackBlur (src/render/sw/sw_stack_blur.cc:18-284) on blur temp canvases.
// The reference's ring buffer only ever holds input pixels at clamped
// indices, so each step reads them directly: the value leaving the left half
// is pixel(max(i - r, 0)), the one entering is pixel(min(i + r + 1, n - 1)),
// the one crossing the centre is pixel(min(i + 1, n - 1)).  Horizontal pass:
// canvas -> blur scratch; vertical pass: blur scratch -> canvas.
// ---------------------------------------------------------------------------
__global__ void k_blur_h(DevBatch b, const uint32_t* temps, uint32_t n_temp, uint32_t max_h) {
  uint32_t t = blockIdx.y;
  uint32_t yrow = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_temp) return;
  const CanvasDesc cd = b.canvases[temps[t]];
  if (yrow >= cd.h) return;
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
  if (x >= cd.w) return;
  int r = min(cd.blur_radius, 254);
  const uint8_t* src = b.pixels + cd.blur_off + (size_t)x * 4;
  uint8_t* dst = b.pixels + cd.px_off + (size_t)x * 4;
  if (r <= 1) {
    for (uint32_t yy = 0; yy < cd.h; ++yy)
      for (int c = 0; c < 4; ++c) dst[(size_t)yy * cd.w * 4 + c] = src[(size_t)yy * cd.w * 4 + c];
    return;
  }
  BlurLine(src, dst, (int)cd.h, cd.w, r, true);
}

int LaunchBlur(const DevBatch& b, const uint32_t* temps, uint32_t n_temp, uint32_t max_h,
               uint32_t max_w, cudaStream_t stream) {
  if (n_temp == 0) return 0;
  dim3 gh((max_h + 63) / 64, n_temp);
  k_blur_h<<<gh, 64, 0, stream>>>(b, temps, n_temp, max_h);
  dim3 gv((max_w + 63) / 64, n_temp);
  k_blur_v<<<gv, 64, 0, stream>>>(b, temps, n_temp, max_w);
  return 2;
}

}  // namespace skc
