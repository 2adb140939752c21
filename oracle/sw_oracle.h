/* C interface of the CPU oracle (oracle/sw_oracle.cc). Test infrastructure
 * only: used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
 * leg as the checker and the timed CPU restatement, never by the library. */
#ifndef SKITY_ORACLE_SW_ORACLE_H
#define SKITY_ORACLE_SW_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct sko_stats {
  uint64_t fragments;  /* sum of clipped span lengths blended */
  uint64_t spans;      /* spans emitted by the rasteriser */
  uint64_t edges;      /* fixed-point edges built */
  uint64_t tie_groups; /* adjacent edges equal in (upper_y, x, dx) */
  double seconds;      /* wall time of the replay (clear + draws) */
  uint64_t draws;
} sko_stats;

/* Replays draws [first, first+count) of a scene stream onto a fresh canvas
 * (cleared as the stream says) and writes premultiplied RGBA8 rows to
 * out_rgba (width*height*4 bytes). Returns 0, or -2 for a malformed stream. */
int sko_render(const uint8_t* scene, size_t len, uint32_t first, uint32_t count,
               uint8_t* out_rgba, sko_stats* stats);
/* Same replay on `threads` host threads, each blending its own band of rows
 * (identical output). */
int sko_render_mt(const uint8_t* scene, size_t len, uint32_t first, uint32_t count,
                  uint8_t* out_rgba, uint32_t threads, sko_stats* stats);
/* Cubic::ToQuads quad count for one cubic (x0,y0,...,x3,y3). */
int sko_cubic_quad_count(const float pts[8]);
/* SWQuadEdge::SetQuad on a monotone quad: out = {1<<shift? no: shift,
 * winding, first_y, last_y}; returns 0 if the quad makes no edge. */
int sko_quad_edge(const float pts[6], int32_t out[4]);
/* The path one draw's fill rasterises (QuadPath of the draw's path):
 * counts = {verbs, points}; at most vcap verbs and pcap points are written. */
int sko_fill_quads(const uint8_t* scene, size_t len, uint32_t draw, uint8_t* verbs,
                   uint32_t vcap, float* pts, uint32_t pcap, uint32_t counts[2]);
/* FP64 exact-area coverage (oracle/exact_area.cc) of a QuadPath: width*height
 * coverages in [0, 1]; quads flattened within tol pixels. */
int ska_exact_coverage(const uint8_t* verbs, uint32_t nv, const float* pts, uint32_t np,
                       int even_odd, int width, int height, double tol, double* cov);
/* Spans (x, y, len, cover) of one draw's fill, in emission order; returns
 * the span count (may exceed cap; only cap are written). */
int sko_path_spans(const uint8_t* scene, size_t len, uint32_t draw, int32_t* out,
                   uint32_t cap);

#ifdef __cplusplus
}
#endif
#endif
