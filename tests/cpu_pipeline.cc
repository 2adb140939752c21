// Test-only: runs the CUDA kernels' per-thread bodies (skity_gb300/csrc/
// passes.cuh) sequentially on the CPU, with the same host-side batch
// building (batch.h) and the same buffer planning as the GPU pipeline.
//
// This is NOT a fallback of the library (the library has none): it lets the
// CPU test suite check the device code paths -- geometry, introsort, sweep,
// span layout, compositing, blur -- against the oracle before any GPU run.
#include <cstdint>
#include <cstring>
#include <vector>

#include "../skity_gb300/csrc/batch.h"
#include "../skity_gb300/csrc/passes.cuh"
#include "../skity_gb300/csrc/clip.cuh"

using namespace skc;

// mode 0: register sweep with the generic sweep for passes it gives up on
// (the GPU pipeline's choice); mode 1: generic sweep for every pass; mode 2:
// every pass through the 32-edge register form, so that the passes with more
// active edges take the give-up path (swept again after the register forms).
extern "C" int skc_cpu_render_mode(const uint8_t* stream, size_t len, uint8_t* out_rgba,
                                   uint64_t stats[6], int mode, uint64_t pool_hint) {
  StreamView sv;
  if (!ParseStream(stream, len, &sv)) return -2;
  HostBatch hb;
  int rc = AddStreamCanvas(hb, sv);
  if (rc) return rc;
  const uint32_t np = (uint32_t)hb.passes.size();
  if (hb.verbs.empty()) hb.verbs.push_back(0);
  if (hb.pts.empty()) hb.pts.push_back(mkP(0, 0));
  if (hb.weights.empty()) hb.weights.push_back(0);
  if (hb.stop_colors.empty()) {
    hb.stop_colors.push_back(make_float4(0, 0, 0, 0));
    hb.stop_offsets.push_back(0);
  }
  std::vector<uint8_t> pixels(hb.pixel_bytes + 16, 0);
  for (const HostBatch::ImageUpload& u : hb.image_uploads)  // the draws' images
    std::memcpy(pixels.data() + u.off, u.bytes.data(), u.bytes.size());
  std::vector<uint8_t> rtab(256);
  for (int v = 0; v < 256; ++v) rtab[v] = ChannelToByte(v / 255.f);

  DevBatch b{};
  b.verbs = hb.verbs.data();
  b.pts = hb.pts.data();
  b.weights = hb.weights.data();
  b.draws = hb.draws.data();
  b.n_passes = np;
  b.canvases = hb.canvases.data();
  std::vector<PassGeom> geom(np);
  std::vector<uint8_t> scratch;
  uint64_t retries = 0;
  for (int attempt = 0; attempt < 8; ++attempt) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < np; ++i) {
      SliceLayout L;
      L.compute(hb.passes[i].cap, sizeof(Edge));
      hb.passes[i].slice_off = total;
      total += L.bytes;
    }
    scratch.assign(total + 16, 0);
    b.passes = hb.passes.data();
    b.scratch = scratch.data();
    b.geom = geom.data();
    for (uint32_t p = 0; p < np; ++p) GeometryPass(b, p);
    uint32_t grown = 0;
    for (uint32_t p = 0; p < np; ++p) {
      if (geom[p].status) {
        GrowCaps(hb.passes[p], geom[p]);
        grown++;
      }
    }
    retries += grown;
    if (!grown) break;
    if (attempt == 7) return -7;
  }
  std::vector<PassSweep> sw;
  SweepPlan pl = PlanSweep(hb, geom, sw);
  // exact size: an overrun of the planned layout is caught by the sanitizer
  // build of this harness and shows up as a mismatch otherwise
  std::vector<uint8_t> sweepmem(pl.sweep_bytes, 0);
  std::vector<uint2> rowspan(pl.rows + 1);
  std::vector<uint32_t> pass_spans(np + 1, 0);
  std::vector<PassComp> comp;
  PlanComp(hb, geom, sw, comp);
  std::vector<uint32_t> band_off, bins;
  b.band_shift = 4;
  BuildBins(hb, comp, AssignBands(hb, b.band_shift), b.band_shift, band_off, bins);
  b.sweep = sw.data();
  b.sweepmem = sweepmem.data();
  uint32_t err = 0;
  b.err = &err;
  b.rowspan = rowspan.data();
  b.pass_spans = pass_spans.data();
  b.comp = comp.data();
  b.band_off = band_off.data();
  b.bins = bins.data();
  Lanes lanes;
  std::vector<uint8_t> pclass(np + 1);
  b.pass_class = pclass.data();
  b.reg_diff_cap = RegDiffCap(pl);
  std::vector<int32_t> regmem32((RegSmemBytes<32>(b.reg_diff_cap) + 3) / 4);
  auto* sh32 = (RegSharedT<32>*)regmem32.data();
  int32_t* sdiff32 = (int32_t*)((uint8_t*)regmem32.data() + sizeof(RegSharedT<32>));
  std::vector<int32_t> regmem64((RegSmemBytes<64>(b.reg_diff_cap) + 3) / 4);
  auto* sh64 = (RegSharedT<64>*)regmem64.data();
  int32_t* sdiff64 = (int32_t*)((uint8_t*)regmem64.data() + sizeof(RegSharedT<64>));
  std::vector<int32_t> regmem((RegSmemBytes<kRegMaxM>(b.reg_diff_cap) + 3) / 4);
  auto* sh = (RegSharedT<kRegMaxM>*)regmem.data();
  int32_t* sdiff = (int32_t*)((uint8_t*)regmem.data() + sizeof(RegSharedT<kRegMaxM>));
  std::vector<uint32_t> order;
  SweepOrder(geom, order);
  b.sweep_order = order.data();
  // path clips (the device's k_clip_state / k_clip_apply, in launch order)
  std::vector<uint2> clip_items;
  const uint64_t clip_state_rows = PlanPathClips(hb, geom, clip_items);
  std::vector<uint32_t> clip_flags(2 * hb.clip_states.size() + 2, 0);
  std::vector<uint2> clip_rows(clip_state_rows + 1);
  b.clip_states = hb.clip_states.data();
  b.n_clip_states = (uint32_t)hb.clip_states.size();
  b.clip_flags = clip_flags.data();
  b.clip_rows = clip_rows.data();
  b.clip_items = clip_items.data();
  b.n_clip_items = (uint32_t)clip_items.size();
  std::vector<int32_t> clip_order(kClipRowCap);
  // span pool: start small so that the regrowth path runs too
  std::vector<uint2> pool(pool_hint ? pool_hint : 1024);
  unsigned long long next = 0;
  uint64_t generic = 0, spans = 0;
  // the path-clip stages read rows the sweep wrote: a row past the end of a
  // short pool reads as empty, so a chain of clip states can show more need
  // on each try (the pool doubles until it holds everything)
  const int attempts = 3 + (int)hb.clip_states.size();
  for (int attempt = 0; attempt < attempts; ++attempt) {
    std::fill(rowspan.begin(), rowspan.end(), make_uint2(0, 0));
    std::fill(pclass.begin(), pclass.end(), (uint8_t)(mode == 1 ? 1 : 0));
    if (mode == 2)  // every pass of plain spans through the 32-edge form
      for (uint32_t p = 0; p < np; ++p)
        if (!geom[p].raw_spans) pclass[p] = (uint8_t)kSweepReg32;
    std::vector<uint32_t> retry;
    next = 0;
    b.spans = pool.data();
    b.span_cap = pool.size();
    b.span_next = &next;
    generic = 0;
    // the sweep launches of the device pipeline (heaviest form first), each
    // in the sweep order
    for (uint32_t i = 0; i < np; ++i) {
      const uint32_t p = order[i];
      if (SweepForm(geom[p], pclass[p]) == kSweepGeneric) {
        SweepPass(b, p, lanes);
        generic++;
      }
    }
    for (uint32_t i = 0; i < np; ++i) {
      const uint32_t p = order[i];
      if (SweepForm(geom[p], pclass[p]) == kSweepReg128)
        if (!SweepPassReg<kRegMaxM>(b, p, lanes, sh, sdiff, b.reg_diff_cap)) retry.push_back(p);
    }
    for (uint32_t i = 0; i < np; ++i) {
      const uint32_t p = order[i];
      if (SweepForm(geom[p], pclass[p]) == kSweepReg64)
        if (!SweepPassReg<64>(b, p, lanes, sh64, sdiff64, b.reg_diff_cap)) retry.push_back(p);
    }
    for (uint32_t i = 0; i < np; ++i) {
      const uint32_t p = order[i];
      if (SweepForm(geom[p], pclass[p]) == kSweepReg32)
        if (!SweepPassReg<32>(b, p, lanes, sh32, sdiff32, b.reg_diff_cap)) retry.push_back(p);
    }
    // the passes the register forms gave up on, after them (k_sweep_retry)
    for (uint32_t p : retry) SweepPass(b, p, lanes);
    generic += retry.size();
    std::fill(clip_flags.begin(), clip_flags.end(), 0u);
    for (uint32_t k = 1; k <= b.n_clip_states; ++k) {
      const ClipStateDesc& st = hb.clip_states[k - 1];
      for (int32_t y = st.y0; y < st.y1; ++y) ClipStateStage(b, k, y, clip_order.data());
    }
    for (uint32_t i = 0; i < b.n_clip_items; ++i) ClipApplyStage(b, i, clip_order.data());
    if (next <= pool.size()) break;
    if (attempt == attempts - 1) return -7;
    pool.assign(hb.clip_states.empty() ? next : 2 * next, make_uint2(0, 0));
  }
  for (uint32_t p = 0; p < np; ++p) spans += pass_spans[p];
  b.brushes = hb.brushes.data();
  b.conicals = hb.conicals.data();
  std::vector<uint8_t> srgb(512);
  SRGBTables(srgb.data());
  b.srgb_tables = srgb.data();
  if (hb.cf_matrices.empty()) hb.cf_matrices.push_back(0);
  b.cf_matrices = hb.cf_matrices.data();
  b.stop_colors = hb.stop_colors.data();
  b.stop_offsets = hb.stop_offsets.data();
  b.pixels = pixels.data();
  b.roundtrip = rtab.data();
  std::vector<uint32_t> row(65536);
  std::vector<RowTask> tasks;
  BuildRowTasks(hb, hb.temp_canvases, 65535, tasks);
  for (const RowTask& t : tasks) CompositeRowScalar(b, t, row.data());
  for (uint32_t c : hb.temp_canvases) {
    const CanvasDesc& cd = hb.canvases[c];
    if (cd.blur_style == 0) continue;  // a layer: no blur
    int r = std::min(cd.blur_radius, 254);
    for (uint32_t y = 0; y < cd.h; ++y) {
      const uint8_t* src = pixels.data() + cd.px_off + (size_t)y * cd.w * 4;
      uint8_t* dst = pixels.data() + cd.blur_off + (size_t)y * cd.w * 4;
      if (r <= 1) std::memcpy(dst, src, (size_t)cd.w * 4);
      else BlurLine(src, dst, (int)cd.w, 1, r, false);
    }
    for (uint32_t x = 0; x < cd.w; ++x) {
      const uint8_t* src = pixels.data() + cd.blur_off + (size_t)x * 4;
      uint8_t* dst = pixels.data() + cd.out_off + (size_t)x * 4;
      if (r <= 1) {
        for (uint32_t y = 0; y < cd.h; ++y) std::memcpy(dst + (size_t)y * cd.w * 4, src + (size_t)y * cd.w * 4, 4);
      } else {
        BlurLine(src, dst, (int)cd.h, cd.w, r, true);
      }
    }
    if (cd.blur_style > 1) {  // k_blur_style
      const uint32_t* raw = (const uint32_t*)(pixels.data() + cd.px_off);
      uint32_t* outp = (uint32_t*)(pixels.data() + cd.out_off);
      for (uint64_t i = 0; i < (uint64_t)cd.w * cd.h; ++i)
        outp[i] = ARGBtoRGBA(BlurStylePixel(cd.blur_style, RGBAtoARGB(raw[i]), RGBAtoARGB(outp[i])));
    }
  }
  BuildRowTasks(hb, hb.main_canvases, 65535, tasks);
  for (const RowTask& t : tasks) CompositeRowScalar(b, t, row.data());
  if (err) return -6;
  const CanvasDesc& cd = hb.canvases[hb.main_canvases[0]];
  std::memcpy(out_rgba, pixels.data() + cd.px_off, (size_t)cd.w * cd.h * 4);
  if (stats) {
    stats[0] = np;
    stats[1] = pl.edges;
    stats[2] = spans;
    stats[3] = retries;
    stats[4] = hb.temp_canvases.size();
    stats[5] = generic;
  }
  return 0;
}

extern "C" int skc_cpu_render(const uint8_t* stream, size_t len, uint8_t* out_rgba,
                              uint64_t stats[6]) {
  return skc_cpu_render_mode(stream, len, out_rgba, stats, 0, 0);
}

// The device introsort on an arbitrary key array, for the permutation test
// against std::sort.
struct KeyLess {
  const int32_t* k;
  bool operator()(int32_t a, int32_t b) const { return k[a] < k[b]; }
};
extern "C" void skc_cpu_introsort(const int32_t* keys, int32_t* idx, int n) {
  for (int i = 0; i < n; ++i) idx[i] = i;
  KeyLess less{keys};
  introsort(idx, n, less);
}

// std::sort with the same "less" on the same initial order: the permutation
// the reference's SortEdges produces (sw_raster.cc:679-704).
#include <algorithm>
extern "C" void skc_std_sort(const int32_t* keys, int32_t* idx, int n) {
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx, idx + n, [&](int32_t a, int32_t b) { return keys[a] < keys[b]; });
}

// FixedDiv (three 32-bit divisions) against the 64-bit quotient on n
// numerator / denominator pairs; returns the number of mismatches.
extern "C" int64_t skc_cpu_fixed_div_check(const int32_t* numer, const int32_t* denom, int64_t n) {
  int64_t bad = 0;
  for (int64_t i = 0; i < n; ++i)
    if (denom[i] != 0 && FixedDiv(numer[i], denom[i]) != FixedDivWide(numer[i], denom[i])) ++bad;
  return bad;
}

// The threaded stream build (BuildStreams) against the one-thread loop on
// the same streams: 0 when every array and counter of the two batches is
// byte-identical, else the number of the first one that differs; negative:
// the status of a failing build.
template <typename T>
static bool SameBytes(const std::vector<T>& a, const std::vector<T>& b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}
extern "C" int skc_build_streams_compare(uint32_t count, const uint8_t* const* streams,
                                         const size_t* bytes, unsigned threads) {
  HostBatch one, many;
  int32_t rc1 = BuildStreams(one, count, streams, bytes, 1);
  int32_t rc2 = BuildStreams(many, count, streams, bytes, threads);
  if (rc1 != rc2) return 100;
  if (rc1) return rc1;
  if (!SameBytes(one.verbs, many.verbs)) return 1;
  if (!SameBytes(one.pts, many.pts)) return 2;
  if (!SameBytes(one.weights, many.weights)) return 3;
  if (!SameBytes(one.draws, many.draws)) return 4;
  if (!SameBytes(one.passes, many.passes)) return 5;
  if (!SameBytes(one.brushes, many.brushes)) return 6;
  if (!SameBytes(one.conicals, many.conicals)) return 7;
  if (!SameBytes(one.cf_matrices, many.cf_matrices)) return 8;
  if (!SameBytes(one.clip_states, many.clip_states)) return 9;
  if (!SameBytes(one.canvases, many.canvases)) return 10;
  if (!SameBytes(one.stop_colors, many.stop_colors)) return 11;
  if (!SameBytes(one.stop_offsets, many.stop_offsets)) return 12;
  if (!SameBytes(one.main_canvases, many.main_canvases)) return 13;
  if (!SameBytes(one.temp_canvases, many.temp_canvases)) return 14;
  if (one.pixel_bytes != many.pixel_bytes || one.draw_count != many.draw_count) return 15;
  if (one.max_temp_w != many.max_temp_w || one.max_temp_h != many.max_temp_h ||
      one.max_temp_style != many.max_temp_style)
    return 16;
  if (one.image_uploads.size() != many.image_uploads.size()) return 17;
  for (size_t i = 0; i < one.image_uploads.size(); ++i)
    if (one.image_uploads[i].off != many.image_uploads[i].off ||
        !SameBytes(one.image_uploads[i].bytes, many.image_uploads[i].bytes))
      return 18;
  return 0;
}

// The canvas matrix the C ABI canvas keeps (skity_cuda_canvas_translate /
// scale / rotate / skew / concat / set_matrix: the current matrix times the
// call's, skc::MatMul) for a sequence of calls: op 0 translate (2 args),
// 1 scale (2), 2 rotate (3), 3 skew (2), 4 concat (9), 5 set matrix (9);
// out: Matrix::Get9.
extern "C" void skc_canvas_matrix(const int* ops, int n, const float* args, float out[9]) {
  Mat4 m;
  m.identity();
  for (int i = 0; i < n; ++i) {
    switch (ops[i]) {
      case 0: m = MatMul(m, MatTranslate(args[0], args[1])); args += 2; break;
      case 1: m = MatMul(m, MatScale(args[0], args[1])); args += 2; break;
      case 2: m = MatMul(m, MatRotateDeg(args[0], args[1], args[2])); args += 3; break;
      case 3: m = MatMul(m, MatSkew(args[0], args[1])); args += 2; break;
      case 4: m = MatMul(m, MatFrom9(args)); args += 9; break;
      case 5: m = MatFrom9(args); args += 9; break;
    }
  }
  const float v[9] = {m.e[0][0], m.e[1][0], m.e[3][0], m.e[0][1], m.e[1][1],
                      m.e[3][1], m.e[0][3], m.e[1][3], m.e[3][3]};
  std::memcpy(out, v, sizeof v);
}
