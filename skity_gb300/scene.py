"""Draw streams ("scenes") and the seeded synthetic scene generator.

A scene is one canvas's worth of work in the form the C-ABI consumes: an
optional ``Canvas::Clear`` colour followed by ``Canvas::DrawPath`` calls in
order.  It is stored as flat little-endian arrays (plain pointers + sizes at
the C boundary, see ``include/skity_cuda.h``):

* ``verbs``   u8, skity ``Path::Verb`` values (kMove=0, kLine=1, kQuad=2,
  kConic=3, kCubic=4, kClose=5; include/skity/graphic/path.hpp:45-60);
* ``points``  f32 (x, y) pairs, one per verb point as ``Path::points_`` holds
  them (include/skity/graphic/path.hpp:590);
* ``weights`` f32 conic weights (``Path::conic_weights_``);
* per draw: verb/point/weight offsets and one 80-byte paint record mirroring
  ``skity::Paint`` (include/skity/graphic/paint.hpp:46-285);
* gradient records (``Shader::MakeLinear`` / ``MakeRadial``,
  src/effect/gradient_shader.cc:96-158) and their colour stops;
* optionally (header flag 1), per draw the canvas clip bounds in device
  space, float (left, top, right, bottom): ``Canvas::ClipRect`` with
  ``kIntersect`` under a translation, which the software canvas applies as
  the global clip bounds that bound the scan (src/render/canvas.cc:463-476,
  src/render/sw/sw_canvas.cc:279-295); without the section every draw has
  the canvas's initial bounds ``kMaxCullRect`` (+-1e9,
  include/skity/render/canvas.hpp:26);
* optionally (header flag 2), per draw the paint's colour filter
  (``ColorFilters::Blend / Matrix / LinearToSRGBGamma / SRGBToLinearGamma /
  Compose``, include/skity/effect/color_filter.hpp), 96 bytes each;
* optionally (header flag 4), the canvas's path clips (``Canvas::ClipPath``,
  ``ClipRRect``, ``ClipRect`` with ``kDifference``; the software canvas keeps
  them as span lists, src/render/sw/sw_canvas.cc:157-336): a table of clip
  states -- each one ClipPath call on top of its parent state, with the
  path, the op, the translation and the global clip bounds in effect -- and
  per draw the clip state it is drawn under (0: none).

The binary file layout (``Scene.to_bytes``) is read by the CPU oracle, by the
reference-driver recipe and by the C-ABI batch entry point.

Random numbers: SplitMix64-seeded xoshiro256**, one independent stream per
path (seed, path index), vectorised over paths with numpy uint64 arithmetic,
so a scene is bit-identical on every machine and numpy version.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

# Path::Verb
MOVE, LINE, QUAD, CONIC, CUBIC, CLOSE = 0, 1, 2, 3, 4, 5
VERB_POINTS = {MOVE: 1, LINE: 1, QUAD: 2, CONIC: 2, CUBIC: 3, CLOSE: 0}
# Paint::Style / Cap / Join, BlendMode, Path::PathFillType, TileMode
FILL, STROKE, STROKE_AND_FILL, STROKE_THEN_FILL = 0, 1, 2, 3
BUTT, ROUND, SQUARE = 0, 1, 2
MITER_JOIN, ROUND_JOIN, BEVEL_JOIN = 0, 1, 2
BLEND_CLEAR, BLEND_SRC, BLEND_DST, BLEND_SRC_OVER = 0, 1, 2, 3
WINDING, EVEN_ODD = 0, 1
TILE_CLAMP, TILE_REPEAT, TILE_MIRROR, TILE_DECAL = 0, 1, 2, 3
GRAD_LINEAR, GRAD_RADIAL, GRAD_SWEEP, GRAD_CONICAL = 1, 2, 3, 4
BLUR_NONE, BLUR_NORMAL = 0, 1

MAGIC = b"SKSC"
VERSION = 1
FLAG_CLIPS = 1    # header flags: the per-draw clip section is present
FLAG_FILTERS = 2  # the per-draw colour-filter section is present
FLAG_PATH_CLIPS = 4  # the clip-state table and per-draw clip states are present
FLAG_IMAGES = 8  # the image table, its pixels and the per-draw image shaders are present
FLAG_LAYERS = 16  # the layer table (Canvas::SaveLayer ... Restore) is present
FLAG_MATRICES = 32  # the per-draw canvas matrix section is present
FLAG_CLIP_MATRICES = 64  # the per-clip-state canvas matrix section is present
IDENTITY6 = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)  # (sx, kx, tx, ky, sy, ty)
# layer record: Canvas::SaveLayer(bounds, paint) under the canvas translation
# and global clip bounds in effect before the call; draws [start, restore)
# are drawn into the layer, which is composited onto the canvas (DrawImage of
# the layer with the layer paint's alpha and blend mode) just before draw
# `restore` (LAYER_OPEN: not restored, never composited).  Layers do not nest.
LAYER_OPEN = 0xFFFFFFFF
LAYER_DTYPE = np.dtype([("bounds", "<f4", 4), ("translate", "<f4", 2), ("clip", "<f4", 4),
                        ("start", "<u4"), ("restore", "<u4"), ("alpha", "<f4"),
                        ("blend", "<u4"), ("pad", "<u4", 2)])
assert LAYER_DTYPE.itemsize == 64
CLIP_DIFFERENCE, CLIP_INTERSECT = 0, 1  # Canvas::ClipOp
# clip state record: parent state (1-based, 0: none), ClipOp, the path's
# fill type, its verb / point / weight counts, the canvas translation and
# the global clip bounds (l, t, r, b) in effect at the ClipPath call
CLIP_STATE_DTYPE = np.dtype([("parent", "<u4"), ("op", "<u4"), ("fill_type", "<u4"),
                             ("nv", "<u4"), ("np", "<u4"), ("nw", "<u4"),
                             ("translate", "<f4", 2), ("bounds", "<f4", 4)])
assert CLIP_STATE_DTYPE.itemsize == 48
NO_CLIP = (-1e9, -1e9, 1e9, 1e9)  # kMaxCullRect

# paint record: 20 x 4 bytes: the Paint fields the raster path reads, the
# path's fill type, and the canvas translation in effect for the draw
# (Canvas::Translate; the rest of the canvas matrix is identity)
PAINT_DTYPE = np.dtype([
    ("style", "<u4"), ("cap", "<u4"), ("join", "<u4"), ("blend", "<u4"),
    ("fill_type", "<u4"), ("gradient", "<i4"), ("blur_style", "<u4"),
    ("blur_radius", "<f4"), ("fill_color", "<f4", 4), ("stroke_color", "<f4", 4),
    ("stroke_width", "<f4"), ("miter", "<f4"), ("translate", "<f4", 2)])
assert PAINT_DTYPE.itemsize == 80
# gradient record: 12 x 4 bytes (matches skity_cuda_gradient)
# colour-filter record: type (0 none, 1 + ColorFilterType: 1 blend, 2 matrix,
# 3 linear->sRGB gamma, 4 sRGB->linear gamma, 5 compose), blend mode, the
# blend colour (ARGB u32), the 4x5 row-major matrix
FILTER_NONE, FILTER_BLEND, FILTER_MATRIX, FILTER_LINEAR_TO_SRGB, FILTER_SRGB_TO_LINEAR, \
    FILTER_COMPOSE = 0, 1, 2, 3, 4, 5
FILTER_DTYPE = np.dtype([("type", "<u4"), ("mode", "<u4"), ("color", "<u4"), ("pad", "<u4"),
                         ("matrix", "<f4", 20)])
assert FILTER_DTYPE.itemsize == 96

# image record: size, AlphaType (2 premultiplied, 3 unpremultiplied) and the
# byte offset of its RGBA8 rows (width * 4 bytes each) in the pixel blob
ALPHA_PREMUL, ALPHA_UNPREMUL = 2, 3
IMAGE_DTYPE = np.dtype([("width", "<u4"), ("height", "<u4"), ("alpha_type", "<u4"),
                        ("pad", "<u4"), ("offset", "<u8")])
assert IMAGE_DTYPE.itemsize == 24
# per-draw image shader (Shader::MakeShader(image, sampling, tile_x, tile_y,
# local)): the image (1-based, 0: none), FilterMode (0 nearest, 1 linear, 2
# cubic, which the software backend samples bilinearly), the tile modes, the
# local matrix in MapPoint form (sx, kx, tx, ky, sy, ty; scale and translate
# only); rect = 1: the draw is DrawImageRect(image, src, dst) (its path is
# the dst rectangle)
FILTER_NEAREST, FILTER_LINEAR, FILTER_CUBIC = 0, 1, 2
IMAGE_SHADER_DTYPE = np.dtype([("image", "<u4"), ("filter", "<u4"), ("tile_x", "<u4"),
                               ("tile_y", "<u4"), ("local", "<f4", 6), ("rect", "<u4"),
                               ("pad", "<u4"), ("src", "<f4", 4), ("dst", "<f4", 4)])
assert IMAGE_SHADER_DTYPE.itemsize == 80

GRADIENT_DTYPE = np.dtype([
    ("type", "<u4"), ("tile_mode", "<u4"), ("stop_count", "<u4"),
    ("stop_start", "<u4"), ("has_offsets", "<u4"), ("reserved", "<u4"),
    ("p0", "<f4", 2), ("p1", "<f4", 2), ("radius", "<f4", 2)])
assert GRADIENT_DTYPE.itemsize == 48


def default_paint() -> np.ndarray:
    """A ``skity::Paint()`` as constructed (paint.hpp:274-285): fill style,
    butt cap, miter join, width 1, miter limit 4, opaque black, src-over."""
    p = np.zeros((), PAINT_DTYPE)
    p["blend"] = BLEND_SRC_OVER
    p["gradient"] = -1
    p["fill_color"] = (0.0, 0.0, 0.0, 1.0)
    p["stroke_color"] = (0.0, 0.0, 0.0, 1.0)
    p["stroke_width"] = 1.0
    p["miter"] = 4.0
    return p


@dataclass
class Scene:
    width: int
    height: int
    clear: tuple | None = (1.0, 1.0, 1.0, 1.0)
    verbs: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint8))
    points: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float32))
    weights: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    verb_off: np.ndarray = field(default_factory=lambda: np.zeros(1, np.uint32))
    point_off: np.ndarray = field(default_factory=lambda: np.zeros(1, np.uint32))
    weight_off: np.ndarray = field(default_factory=lambda: np.zeros(1, np.uint32))
    paints: np.ndarray = field(default_factory=lambda: np.zeros(0, PAINT_DTYPE))
    gradients: np.ndarray = field(default_factory=lambda: np.zeros(0, GRADIENT_DTYPE))
    stop_colors: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.float32))
    stop_offsets: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    clips: np.ndarray | None = None  # (n_draws, 4) float32 LTRB, or None: no clip
    filters: np.ndarray | None = None  # (n_draws,) FILTER_DTYPE, or None: no colour filters
    # path clips: (states CLIP_STATE_DTYPE, verbs u8, points (n, 2) f32, weights f32,
    # per-draw state u32), or None
    path_clips: tuple | None = None
    # images: (IMAGE_DTYPE records, pixel blob u8, per-draw IMAGE_SHADER_DTYPE), or None
    images: tuple | None = None
    layers: np.ndarray | None = None  # LAYER_DTYPE records, or None
    # (n_draws, 6) float32 canvas matrices (sx, kx, tx, ky, sy, ty: the
    # Matrix::Get9 order without the perspective row), or None: each draw's
    # matrix is its paint's translation
    matrices: np.ndarray | None = None
    # (n_clip_states, 6) float32 canvas matrices of the ClipPath calls (the
    # states' translations are then zero), or None: each state's matrix is
    # its translation
    clip_matrices: np.ndarray | None = None

    @property
    def n_draws(self) -> int:
        return len(self.paints)

    def to_bytes(self) -> bytes:
        nd = self.n_draws
        flags = (FLAG_CLIPS if self.clips is not None else 0) | \
            (FLAG_FILTERS if self.filters is not None else 0) | \
            (FLAG_PATH_CLIPS if self.path_clips is not None else 0) | \
            (FLAG_IMAGES if self.images is not None else 0) | \
            (FLAG_LAYERS if self.layers is not None else 0) | \
            (FLAG_MATRICES if self.matrices is not None else 0) | \
            (FLAG_CLIP_MATRICES if self.clip_matrices is not None else 0)
        out = [MAGIC, struct.pack("<7I", VERSION, self.width, self.height,
                                  1 if self.clear is not None else 0, flags, 0, 0)]
        out.append(np.asarray(self.clear if self.clear is not None else (0, 0, 0, 0),
                              np.float32).tobytes())
        out.append(struct.pack("<6I", nd, len(self.verbs), len(self.points),
                               len(self.weights), len(self.gradients), len(self.stop_offsets)))
        for a in (self.verb_off, self.point_off, self.weight_off):
            assert len(a) == nd + 1
            out.append(np.ascontiguousarray(a, np.uint32).tobytes())
        vb = np.ascontiguousarray(self.verbs, np.uint8).tobytes()
        out.append(vb + b"\0" * ((-len(vb)) % 4))
        out.append(np.ascontiguousarray(self.points, np.float32).tobytes())
        out.append(np.ascontiguousarray(self.weights, np.float32).tobytes())
        out.append(np.ascontiguousarray(self.paints, PAINT_DTYPE).tobytes())
        out.append(np.ascontiguousarray(self.gradients, GRADIENT_DTYPE).tobytes())
        out.append(np.ascontiguousarray(self.stop_colors, np.float32).tobytes())
        out.append(np.ascontiguousarray(self.stop_offsets, np.float32).tobytes())
        if self.clips is not None:
            c = np.ascontiguousarray(self.clips, np.float32).reshape(-1, 4)
            assert len(c) == nd
            out.append(c.tobytes())
        if self.filters is not None:
            f = np.ascontiguousarray(self.filters, FILTER_DTYPE)
            assert len(f) == nd
            out.append(f.tobytes())
        if self.path_clips is not None:
            states, cverbs, cpts, cwts, per_draw = self.path_clips
            states = np.ascontiguousarray(states, CLIP_STATE_DTYPE)
            out.append(struct.pack("<I", len(states)))
            out.append(states.tobytes())
            vb = np.ascontiguousarray(cverbs, np.uint8).tobytes()
            out.append(vb + b"\0" * ((-len(vb)) % 4))
            out.append(np.ascontiguousarray(cpts, np.float32).tobytes())
            out.append(np.ascontiguousarray(cwts, np.float32).tobytes())
            pd = np.ascontiguousarray(per_draw, np.uint32)
            assert len(pd) == nd
            out.append(pd.tobytes())
        if self.images is not None:
            recs, blob, shaders = self.images
            recs = np.ascontiguousarray(recs, IMAGE_DTYPE)
            blob = np.ascontiguousarray(blob, np.uint8).tobytes()
            out.append(struct.pack("<I", len(recs)))
            out.append(recs.tobytes())
            out.append(struct.pack("<Q", len(blob)))
            out.append(blob + b"\0" * ((-len(blob)) % 4))
            sh = np.ascontiguousarray(shaders, IMAGE_SHADER_DTYPE)
            assert len(sh) == nd
            out.append(sh.tobytes())
        if self.layers is not None:
            lay = np.ascontiguousarray(self.layers, LAYER_DTYPE)
            out.append(struct.pack("<I", len(lay)))
            out.append(lay.tobytes())
        if self.matrices is not None:
            m = np.ascontiguousarray(self.matrices, np.float32).reshape(-1, 6)
            assert len(m) == nd
            out.append(m.tobytes())
        if self.clip_matrices is not None:
            assert self.path_clips is not None
            m = np.ascontiguousarray(self.clip_matrices, np.float32).reshape(-1, 6)
            assert len(m) == len(self.path_clips[0])
            out.append(m.tobytes())
        return b"".join(out)

    @staticmethod
    def from_bytes(buf: bytes) -> "Scene":
        if buf[:4] != MAGIC:
            raise ValueError("not a scene stream")
        ver, w, h, has_clear, flags, _, _ = struct.unpack_from("<7I", buf, 4)
        if ver != VERSION:
            raise ValueError(f"scene version {ver}")
        o = 32
        clear = tuple(np.frombuffer(buf, np.float32, 4, o).tolist()); o += 16
        nd, nv, npt, nw, ng, ns = struct.unpack_from("<6I", buf, o); o += 24

        def take(dt, n, shape=None):
            nonlocal o
            a = np.frombuffer(buf, dt, n, o).copy()
            o += a.nbytes
            return a.reshape(shape) if shape else a
        vo = take(np.uint32, nd + 1); po = take(np.uint32, nd + 1); wo = take(np.uint32, nd + 1)
        verbs = take(np.uint8, nv); o += (-nv) % 4
        pts = take(np.float32, 2 * npt, (npt, 2))
        wts = take(np.float32, nw)
        paints = take(PAINT_DTYPE, nd)
        grads = take(GRADIENT_DTYPE, ng)
        sc = take(np.float32, 4 * ns, (ns, 4))
        so = take(np.float32, ns)
        clips = take(np.float32, 4 * nd, (nd, 4)) if flags & FLAG_CLIPS else None
        filters = take(FILTER_DTYPE, nd) if flags & FLAG_FILTERS else None
        path_clips = None
        if flags & FLAG_PATH_CLIPS:
            (n_states,) = struct.unpack_from("<I", buf, o); o += 4
            states = take(CLIP_STATE_DTYPE, n_states)
            tv, tp, tw = (int(states["nv"].sum()), int(states["np"].sum()),
                          int(states["nw"].sum()))
            cverbs = take(np.uint8, tv); o += (-tv) % 4
            cpts = take(np.float32, 2 * tp, (tp, 2))
            cwts = take(np.float32, tw)
            per_draw = take(np.uint32, nd)
            path_clips = (states, cverbs, cpts, cwts, per_draw)
        images = None
        if flags & FLAG_IMAGES:
            (n_images,) = struct.unpack_from("<I", buf, o); o += 4
            recs = take(IMAGE_DTYPE, n_images)
            (nb,) = struct.unpack_from("<Q", buf, o); o += 8
            blob = take(np.uint8, nb); o += (-nb) % 4
            images = (recs, blob, take(IMAGE_SHADER_DTYPE, nd))
        layers = None
        if flags & FLAG_LAYERS:
            (n_layers,) = struct.unpack_from("<I", buf, o); o += 4
            layers = take(LAYER_DTYPE, n_layers)
        matrices = take(np.float32, 6 * nd, (nd, 6)) if flags & FLAG_MATRICES else None
        clip_matrices = None
        if flags & FLAG_CLIP_MATRICES:
            n = len(path_clips[0]) if path_clips is not None else 0
            clip_matrices = take(np.float32, 6 * n, (n, 6))
        return Scene(w, h, clear if has_clear else None, verbs, pts, wts, vo, po, wo,
                     paints, grads, sc, so, clips, filters, path_clips, images, layers,
                     matrices, clip_matrices)

    def subset(self, first: int, count: int) -> "Scene":
        """Draws [first, first+count) of this scene, same canvas and clear."""
        last = min(self.n_draws, first + count)
        v0, v1 = int(self.verb_off[first]), int(self.verb_off[last])
        p0, p1 = int(self.point_off[first]), int(self.point_off[last])
        w0, w1 = int(self.weight_off[first]), int(self.weight_off[last])
        paints = self.paints[first:last].copy()
        used = sorted({int(g) for g in paints["gradient"] if g >= 0})
        remap = {g: i for i, g in enumerate(used)}
        grads = self.gradients[used].copy() if used else np.zeros(0, GRADIENT_DTYPE)
        sc, so, start = [], [], 0
        for i, g in enumerate(used):
            s0, n = int(self.gradients[g]["stop_start"]), int(self.gradients[g]["stop_count"])
            sc.append(self.stop_colors[s0:s0 + n]); so.append(self.stop_offsets[s0:s0 + n])
            grads[i]["stop_start"] = start; start += n
        for p in paints:
            if p["gradient"] >= 0:
                p["gradient"] = remap[int(p["gradient"])]
        return Scene(self.width, self.height, self.clear,
                     self.verbs[v0:v1].copy(), self.points[p0:p1].copy(),
                     self.weights[w0:w1].copy(),
                     (self.verb_off[first:last + 1] - v0).astype(np.uint32),
                     (self.point_off[first:last + 1] - p0).astype(np.uint32),
                     (self.weight_off[first:last + 1] - w0).astype(np.uint32),
                     paints, grads,
                     np.concatenate(sc) if sc else np.zeros((0, 4), np.float32),
                     np.concatenate(so) if so else np.zeros(0, np.float32),
                     None if self.clips is None else self.clips[first:last].copy(),
                     None if self.filters is None else self.filters[first:last].copy(),
                     None if self.path_clips is None else
                     self.path_clips[:4] + (self.path_clips[4][first:last].copy(),),
                     None if self.images is None else
                     self.images[:2] + (self.images[2][first:last].copy(),),
                     self._subset_layers(first, last),
                     None if self.matrices is None else self.matrices[first:last].copy(),
                     None if self.clip_matrices is None else self.clip_matrices.copy())

    def _subset_layers(self, first: int, last: int):
        """The layers of draws [first, last): those restored before `first`
        are gone; one restored past `last` is not restored in the subset."""
        if self.layers is None:
            return None
        out = []
        for rec in self.layers:
            start, restore = int(rec["start"]), int(rec["restore"])
            if restore != LAYER_OPEN and restore < first:
                continue
            if start > last:
                continue
            r = rec.copy()
            r["start"] = max(start, first) - first
            r["restore"] = (restore - first) if restore != LAYER_OPEN and restore <= last \
                else LAYER_OPEN
            out.append(r)
        return np.array(out, LAYER_DTYPE) if out else None


def map_clip(clip, rect, tx=0.0, ty=0.0):
    """Canvas::ClipRect(rect, kIntersect) under Translate(tx, ty): the
    global clip bounds after the call (Canvas::CalculateGlobalClipBounds,
    src/render/canvas.cc:463-476): the rect mapped by the translation
    (Matrix::MapRect, src/geometry/matrix.cc:306-337 -- corners x + tx,
    then min/max) intersected with `clip` (Rect::Intersect,
    src/geometry/rect.cc:160-172), or the empty rect (0, 0, 0, 0)."""
    f = np.float32
    xs = (f(rect[0]) + f(tx), f(rect[2]) + f(tx))
    ys = (f(rect[1]) + f(ty), f(rect[3]) + f(ty))
    ml, mr, mt, mb = min(xs), max(xs), min(ys), max(ys)
    l, r = max(f(clip[0]), ml), min(f(clip[2]), mr)
    t, b = max(f(clip[1]), mt), min(f(clip[3]), mb)
    if not (l < r and t < b):
        return (0.0, 0.0, 0.0, 0.0)
    return (float(l), float(t), float(r), float(b))


def map_clip_matrix(clip, rect, m):
    """Canvas::ClipRect / ClipPath(kIntersect) under the canvas matrix `m`
    (sx, kx, tx, ky, sy, ty): the global clip bounds after the call -- the
    rect's corners mapped as Matrix::MapRect maps them ((sx x + kx y) + tx,
    in float32), their min and max, intersected with `clip`, or the empty
    rect (0, 0, 0, 0)."""
    f = np.float32
    sx, kx, tx, ky, sy, ty = (f(v) for v in m)
    xs, ys = [], []
    for x, y in ((rect[0], rect[1]), (rect[2], rect[1]), (rect[2], rect[3]),
                 (rect[0], rect[3])):
        x, y = f(x), f(y)
        xs.append(f(f(sx * x) + f(kx * y)) + tx)
        ys.append(f(f(ky * x) + f(sy * y)) + ty)
    ml, mr, mt, mb = xs[0], xs[0], ys[0], ys[0]
    for i in range(1, 4):
        ml, mr = min(xs[i], ml), max(xs[i], mr)
        mt, mb = min(ys[i], mt), max(ys[i], mb)
    l, r = max(f(clip[0]), ml), min(f(clip[2]), mr)
    t, b = max(f(clip[1]), mt), min(f(clip[3]), mb)
    if not (l < r and t < b):
        return (0.0, 0.0, 0.0, 0.0)
    return (float(l), float(t), float(r), float(b))


RECT_VERBS = [MOVE, LINE, LINE, LINE, CLOSE]


def rect_points(rect):
    """Path::AddRect(rect) (src/graphic/path.cc:815-835): clockwise from the
    top-left corner."""
    l, t, r, b = rect
    return [(l, t), (r, t), (r, b), (l, b)]


class SceneBuilder:
    """Appends Canvas::DrawPath calls to a Scene, the way skity::Path builds
    its verb/point arrays (src/graphic/path.cc:494-569, 837-860)."""

    def __init__(self, width: int, height: int, clear=(1.0, 1.0, 1.0, 1.0)):
        self.width, self.height, self.clear = width, height, clear
        self._verbs, self._pts, self._wts = [], [], []
        self._vo, self._po, self._wo = [0], [0], [0]
        self._paints, self._grads, self._sc, self._so = [], [], [], []
        self._clips, self._filters = [], []
        self._nv = self._np = self._nw = 0
        # path clips: state records and their paths; the current state and
        # the save stack of it (Canvas::Save / Restore)
        self._cstates, self._cverbs, self._cpts, self._cwts = [], [], [], []
        self._cmatrices = []
        self._cstate, self._csaved, self._draw_cstate = 0, [], []
        self._images, self._blobs, self._nblob, self._shaders = [], [], 0, []
        self._layers = []
        self._matrices = []

    def add_gradient(self, kind, p0, p1, radius, colors, offsets=None,
                     tile_mode=TILE_CLAMP) -> int:
        g = np.zeros((), GRADIENT_DTYPE)
        g["type"], g["tile_mode"] = kind, tile_mode
        colors = np.asarray(colors, np.float32).reshape(-1, 4)
        g["stop_count"] = len(colors)
        g["stop_start"] = sum(len(c) for c in self._sc)
        g["has_offsets"] = 1 if offsets is not None else 0
        g["p0"], g["p1"], g["radius"] = p0, p1, radius
        self._grads.append(g)
        self._sc.append(colors)
        self._so.append(np.asarray(offsets if offsets is not None
                                   else np.zeros(len(colors)), np.float32))
        return len(self._grads) - 1

    def add_image(self, pixels, alpha_type=ALPHA_PREMUL) -> int:
        """An image of (height, width, 4) RGBA8 pixels; returns its 1-based
        index for image_shader()."""
        px = np.ascontiguousarray(pixels, np.uint8)
        assert px.ndim == 3 and px.shape[2] == 4
        r = np.zeros((), IMAGE_DTYPE)
        r["width"], r["height"], r["alpha_type"], r["offset"] = \
            px.shape[1], px.shape[0], alpha_type, self._nblob
        self._images.append(r)
        self._blobs.append(px.reshape(-1))
        self._nblob += px.size
        return len(self._images)

    def draw_image_rect(self, image, src, dst, paint, filter=FILTER_NEAREST, clip=None,
                        color_filter=None):
        """Canvas::DrawImageRect(image, src, dst, sampling, &paint)
        (sw_canvas.cc:641-677): a fill of the dst rectangle with a decal image
        shader whose local matrix maps src onto dst.  An empty src or dst
        draws nothing."""
        f32 = np.float32
        sl, st, sr, sb = (f32(v) for v in src)
        dl, dt, dr, db = (f32(v) for v in dst)
        sw, sh, dw, dh = sr - sl, sb - st, dr - dl, db - dt
        if sw == 0 or sh == 0 or dw == 0 or dh == 0:
            return
        sx, sy = dw / sw, dh / sh
        # Translate(dst.L, dst.T) * Scale(sx, sy) * Translate(-src.L, -src.T)
        local = (sx, 0.0, sx * -sl + dl, 0.0, sy, sy * -st + dt)
        rec = image_shader(image, filter, TILE_DECAL, TILE_DECAL, local)
        rec["rect"], rec["src"], rec["dst"] = 1, (sl, st, sr, sb), (dl, dt, dr, db)
        p = paint.copy()
        p["style"], p["gradient"] = FILL, -1
        self.draw_path([MOVE, LINE, LINE, LINE, CLOSE],
                       [(dl, dt), (dr, dt), (dr, db), (dl, db)], p, clip=clip,
                       color_filter=color_filter, image_shader=rec)

    def draw_path(self, verbs, points, paint, weights=(), clip=None, color_filter=None,
                  image_shader=None, matrix=None):
        """`clip`: device-space clip bounds (l, t, r, b) in effect for the
        draw (see map_clip); None: the canvas's initial bounds.
        `color_filter`: a FILTER_DTYPE record, or None.
        `image_shader`: an IMAGE_SHADER_DTYPE record (image_shader()), or None.
        `matrix`: the canvas matrix of the draw (sx, kx, tx, ky, sy, ty), in
        place of the paint's translation (which must then be zero); None: the
        translation."""
        if matrix is not None:
            assert tuple(paint["translate"]) == (0.0, 0.0)
        self._matrices.append(None if matrix is None else tuple(float(np.float32(v)) for v in matrix))
        verbs = np.asarray(verbs, np.uint8)
        points = np.asarray(points, np.float32).reshape(-1, 2)
        self._verbs.append(verbs); self._pts.append(points)
        self._wts.append(np.asarray(weights, np.float32))
        self._nv += len(verbs); self._np += len(points); self._nw += len(weights)
        self._vo.append(self._nv); self._po.append(self._np); self._wo.append(self._nw)
        self._paints.append(paint)
        self._clips.append(NO_CLIP if clip is None else tuple(clip))
        self._filters.append(np.zeros((), FILTER_DTYPE) if color_filter is None else color_filter)
        self._draw_cstate.append(self._cstate)
        self._shaders.append(np.zeros((), IMAGE_SHADER_DTYPE) if image_shader is None
                             else image_shader)

    def save(self):
        """Canvas::Save for the path-clip state."""
        self._csaved.append(self._cstate)

    def restore(self):
        if self._csaved:
            self._cstate = self._csaved.pop()

    def clip_path(self, verbs, points, op, fill_type=WINDING, weights=(), translate=(0.0, 0.0),
                  bounds=NO_CLIP, matrix=None):
        """Canvas::ClipPath(path, op) on the current state, with the canvas
        translation (or the whole canvas matrix `matrix`, sx, kx, tx, ky, sy,
        ty, with `translate` zero) and the global clip bounds in effect at the
        call."""
        if matrix is not None:
            assert tuple(translate) == (0.0, 0.0)
        self._cmatrices.append(None if matrix is None
                               else tuple(float(np.float32(v)) for v in matrix))
        st = np.zeros((), CLIP_STATE_DTYPE)
        verbs = np.asarray(verbs, np.uint8)
        points = np.asarray(points, np.float32).reshape(-1, 2)
        weights = np.asarray(weights, np.float32)
        st["parent"], st["op"], st["fill_type"] = self._cstate, op, fill_type
        st["nv"], st["np"], st["nw"] = len(verbs), len(points), len(weights)
        st["translate"], st["bounds"] = translate, bounds
        self._cstates.append(st)
        self._cverbs.append(verbs)
        self._cpts.append(points)
        self._cwts.append(weights)
        self._cstate = len(self._cstates)
        return self._cstate

    def save_layer(self, bounds, alpha=1.0, blend=BLEND_SRC_OVER, translate=(0.0, 0.0),
                   clip=NO_CLIP):
        """Canvas::SaveLayer(bounds, paint) under the canvas translation and
        global clip bounds `clip` in effect before the call.  Returns the clip
        bounds of the draws inside the layer (Canvas::SaveLayer narrows them
        by the bounds, src/render/canvas.cc:255-276), or None when the
        reference saves no layer (empty bounds, or bounds outside the clip:
        a Save with an empty clip instead)."""
        f = np.float32
        b = tuple(float(f(v)) for v in bounds)
        if not (b[0] < b[2] and b[1] < b[3]):
            return None
        narrowed = map_clip(clip, b, translate[0], translate[1])
        if narrowed == (0.0, 0.0, 0.0, 0.0):
            return None
        r = np.zeros((), LAYER_DTYPE)
        r["bounds"], r["translate"], r["clip"] = b, translate, clip
        r["start"], r["restore"] = len(self._paints), LAYER_OPEN
        r["alpha"], r["blend"] = alpha, blend
        self._layers.append(r)
        return narrowed

    def restore_layer(self):
        """Canvas::Restore of the innermost open layer: it is composited
        before the next draw."""
        for r in reversed(self._layers):
            if int(r["restore"]) == LAYER_OPEN:
                r["restore"] = len(self._paints)
                return

    def build(self) -> Scene:
        cat = lambda xs, dt, shp: (np.concatenate(xs).astype(dt) if xs else np.zeros(shp, dt))
        paints = (np.array(self._paints, PAINT_DTYPE) if self._paints
                  else np.zeros(0, PAINT_DTYPE))
        cstates = np.array(self._cstates, CLIP_STATE_DTYPE) if self._cstates else None
        clip_matrices = None
        if any(m is not None for m in self._cmatrices):
            # every state's matrix in the section; the translations move there
            clip_matrices = np.array([m if m is not None else
                                      (1.0, 0.0, float(c["translate"][0]), 0.0, 1.0,
                                       float(c["translate"][1]))
                                      for m, c in zip(self._cmatrices, cstates)], np.float32)
            cstates["translate"] = 0.0
        matrices = None
        if any(m is not None for m in self._matrices):
            # every draw's matrix in the section; the paints' translations move there
            matrices = np.array([m if m is not None else
                                 (1.0, 0.0, float(p["translate"][0]), 0.0, 1.0,
                                  float(p["translate"][1]))
                                 for m, p in zip(self._matrices, paints)], np.float32)
            paints["translate"] = 0.0
        return Scene(self.width, self.height, self.clear,
                     cat(self._verbs, np.uint8, 0), cat(self._pts, np.float32, (0, 2)),
                     cat(self._wts, np.float32, 0),
                     np.asarray(self._vo, np.uint32), np.asarray(self._po, np.uint32),
                     np.asarray(self._wo, np.uint32),
                     paints,
                     np.array(self._grads, GRADIENT_DTYPE) if self._grads else np.zeros(0, GRADIENT_DTYPE),
                     cat(self._sc, np.float32, (0, 4)), cat(self._so, np.float32, 0),
                     (np.array(self._clips, np.float32).reshape(-1, 4)
                      if any(c != NO_CLIP for c in self._clips) else None),
                     (np.array(self._filters, FILTER_DTYPE)
                      if any(int(f["type"]) != FILTER_NONE for f in self._filters) else None),
                     ((cstates, cat(self._cverbs, np.uint8, 0),
                       cat(self._cpts, np.float32, (0, 2)), cat(self._cwts, np.float32, 0),
                       np.asarray(self._draw_cstate, np.uint32))
                      if self._cstates else None),
                     ((np.array(self._images, IMAGE_DTYPE), cat(self._blobs, np.uint8, 0),
                       np.array(self._shaders, IMAGE_SHADER_DTYPE))
                      if self._images else None),
                     np.array(self._layers, LAYER_DTYPE) if self._layers else None,
                     matrices, clip_matrices)


def image_shader(image, filter=FILTER_NEAREST, tile_x=TILE_CLAMP, tile_y=TILE_CLAMP,
                 local=(1.0, 0.0, 0.0, 0.0, 1.0, 0.0)):
    """An IMAGE_SHADER_DTYPE record: Shader::MakeShader(image, sampling,
    tile_x, tile_y, local) with local = (sx, kx, tx, ky, sy, ty)."""
    r = np.zeros((), IMAGE_SHADER_DTYPE)
    r["image"], r["filter"], r["tile_x"], r["tile_y"] = image, filter, tile_x, tile_y
    r["local"] = local
    return r


def filter_record(kind, mode=0, color=0, matrix=None):
    """A FILTER_DTYPE record: kind FILTER_*, blend mode and ARGB colour for
    FILTER_BLEND, 20 row-major floats for FILTER_MATRIX."""
    r = np.zeros((), FILTER_DTYPE)
    r["type"], r["mode"], r["color"] = kind, mode, color
    if matrix is not None:
        r["matrix"] = np.asarray(matrix, np.float32).reshape(20)
    return r


# ---------------------------------------------------------------------------
# Seeded random streams: SplitMix64 -> xoshiro256**, vectorised over streams.
# ---------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _rotl(x, k):
    return (x << np.uint64(k)) | (x >> np.uint64(64 - k))


def _splitmix64(x):
    x = x + np.uint64(0x9E3779B97F4A7C15)
    z = x
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x, z ^ (z >> np.uint64(31))


def random_streams(seed: int, n_streams: int, n_draws: int) -> np.ndarray:
    """(n_streams, n_draws) uint64: stream i is xoshiro256** seeded by a
    SplitMix64 over (seed, i)."""
    with np.errstate(over="ignore"):
        x = (np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
             ^ (np.arange(n_streams, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03)))
        s = []
        for _ in range(4):
            x, z = _splitmix64(x)
            s.append(z)
        s0, s1, s2, s3 = s
        out = np.empty((n_streams, n_draws), np.uint64)
        for k in range(n_draws):
            out[:, k] = _rotl(s1 * np.uint64(5), 7) * np.uint64(9)
            t = s1 << np.uint64(17)
            s2 ^= s0; s3 ^= s1; s1 ^= s2; s0 ^= s3
            s2 ^= t
            s3 = _rotl(s3, 45)
    return out


def u01(u: np.ndarray) -> np.ndarray:
    """uint64 -> float32 in [0,1): (u >> 40) * 2^-24 (exact in float32)."""
    return ((u >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24))


def uniform(u, lo, hi) -> np.ndarray:
    return (np.float32(lo) + u01(u) * np.float32(hi - lo)).astype(np.float32)


def randint(u, lo, hi) -> np.ndarray:
    """Integer uniform on [lo, hi] inclusive (multiply-shift on the top 32 bits)."""
    span = np.uint64(hi - lo + 1)
    return (np.int64(lo) + ((u >> np.uint64(32)) * span >> np.uint64(32)).astype(np.int64))


def loguniform(u, lo, hi) -> np.ndarray:
    f = u01(u).astype(np.float64)
    return np.exp(np.log(lo) + f * (np.log(hi) - np.log(lo)))


def _color4f_from_rgb_bytes(r, g, b, a):
    """Paint::SetColor(ARGB(255,r,g,b)) -> Color4fFromColor (c / 255.f) then
    SetAlphaF(a) (src/graphic/paint.cc:77-101, src/graphic/color.cc:44-51)."""
    f = np.float32(255.0)
    return np.stack([np.asarray(r, np.float32) / f, np.asarray(g, np.float32) / f,
                     np.asarray(b, np.float32) / f, np.asarray(a, np.float32)], -1)


# ---------------------------------------------------------------------------
# Workloads (the five benchmark configurations, seeded synthetic data)
# ---------------------------------------------------------------------------
SEED_BASE = 0x5EED0000
_VERB_SLOTS = 7  # per verb: kind selector + up to 3 points


def random_paths_scene(seed, width, height, n_paths, verbs_lo, verbs_hi,
                       coord_lo=(0.0, 0.0), coord_hi=None, evenodd_frac=0.0,
                       gradient_frac=0.0, stroke_frac=0.0, clear=(1.0, 1.0, 1.0, 1.0)) -> Scene:
    """Random closed paths: MoveTo + n verbs (50% LineTo, 25% QuadTo,
    25% CubicTo) + Close, control points uniform over [coord_lo, coord_hi]."""
    if coord_hi is None:
        coord_hi = (float(width), float(height))
    base = 24
    K = base + _VERB_SLOTS * verbs_hi
    R = random_streams(seed, n_paths, K)
    nverb = randint(R[:, 0], verbs_lo, verbs_hi)
    fill_type = np.where(u01(R[:, 1]) < np.float32(evenodd_frac), EVEN_ODD, WINDING)
    kind_u = u01(R[:, 2])
    stroke = u01(R[:, 3]) < np.float32(stroke_frac)
    width_s = uniform(R[:, 4], 1.0, 8.0)
    cap = randint(R[:, 5], 0, 2)
    join = randint(R[:, 6], 0, 2)
    rgb = [randint(R[:, 7 + i], 0, 255) for i in range(3)]
    alpha = uniform(R[:, 10], 0.3, 1.0)
    colors = _color4f_from_rgb_bytes(*rgb, alpha)
    grad_kind = np.where(kind_u < np.float32(1.0 - gradient_frac), 0,
                         np.where(kind_u < np.float32(1.0 - gradient_frac / 2), GRAD_LINEAR, GRAD_RADIAL))
    mx = uniform(R[:, 22], coord_lo[0], coord_hi[0])
    my = uniform(R[:, 23], coord_lo[1], coord_hi[1])
    vsel = u01(R[:, base::_VERB_SLOTS][:, :verbs_hi])
    cx = [uniform(R[:, base + 1 + 2 * j::_VERB_SLOTS][:, :verbs_hi], coord_lo[0], coord_hi[0]) for j in range(3)]
    cy = [uniform(R[:, base + 2 + 2 * j::_VERB_SLOTS][:, :verbs_hi], coord_lo[1], coord_hi[1]) for j in range(3)]

    b = SceneBuilder(width, height, clear)
    gradR = random_streams(seed ^ 0x6A09E667F3BCC908, n_paths, 48) if gradient_frac > 0 else None
    for i in range(n_paths):
        n = int(nverb[i])
        sel = vsel[i, :n]
        kinds = np.where(sel < 0.5, LINE, np.where(sel < 0.75, QUAD, CUBIC)).astype(np.uint8)
        verbs = np.concatenate([[MOVE], kinds, [CLOSE]]).astype(np.uint8)
        npts = np.where(kinds == LINE, 1, np.where(kinds == QUAD, 2, 3))
        pts = [np.array([[mx[i], my[i]]], np.float32)]
        for j in range(n):
            k = int(npts[j])
            pts.append(np.stack([[cx[t][i, j], cy[t][i, j]] for t in range(k)]).astype(np.float32))
        pts = np.concatenate(pts)
        p = default_paint()
        p["fill_type"] = fill_type[i]
        p["fill_color"] = colors[i]
        p["stroke_color"] = colors[i]
        if stroke[i]:
            p["style"] = STROKE
            p["stroke_width"] = width_s[i]
            p["cap"] = cap[i]
            p["join"] = join[i]
        if grad_kind[i]:
            g = gradR[i]
            ns = int(randint(g[0], 2, 8))
            offs = np.sort(u01(g[1:1 + ns]))
            offs[0], offs[-1] = 0.0, 1.0
            sc = np.stack([randint(g[10 + 4 * s + c], 0, 255) for s in range(ns) for c in range(4)]
                          ).reshape(ns, 4).astype(np.float32) / np.float32(255.0)
            lo, hi = pts.min(0), pts.max(0)
            if grad_kind[i] == GRAD_LINEAR:
                p0 = (uniform(g[42], lo[0], hi[0]), uniform(g[43], lo[1], hi[1]))
                p1 = (uniform(g[44], lo[0], hi[0]), uniform(g[45], lo[1], hi[1]))
                gi = b.add_gradient(GRAD_LINEAR, p0, p1, (0.0, 0.0), sc, offs)
            else:
                c = (uniform(g[42], lo[0], hi[0]), uniform(g[43], lo[1], hi[1]))
                half_diag = np.float32(0.5) * np.float32(np.hypot(*(hi - lo).astype(np.float64)))
                r = np.float32(uniform(g[44], 0.25, 1.0) * half_diag)
                gi = b.add_gradient(GRAD_RADIAL, c, (0.0, 0.0), (r, 0.0), sc, offs)
            p["gradient"] = gi
        b.draw_path(verbs, pts, p)
    return b.build()


def with_layers(sc: Scene, specs) -> Scene:
    """`sc` with layers around runs of its draws.  specs: (start, restore,
    bounds, alpha, blend, translate, clip) per layer, in draw order, not
    overlapping; `clip` is the canvas's global clip bounds before the
    SaveLayer.  Draws inside a layer get their clip bounds narrowed by the
    layer's bounds, as Canvas::SaveLayer narrows them (src/render/canvas.cc:
    255-276); a layer the reference would not save (empty bounds, or bounds
    outside the clip) becomes an empty clip for its draws instead."""
    out = Scene(**{k: getattr(sc, k) for k in sc.__dataclass_fields__})
    clips = (np.array(sc.clips, np.float32) if sc.clips is not None
             else np.tile(np.array(NO_CLIP, np.float32), (sc.n_draws, 1)))
    recs = []
    for start, restore, bounds, alpha, blend, translate, clip in specs:
        b = SceneBuilder(sc.width, sc.height)
        narrowed = b.save_layer(bounds, alpha, blend, translate, clip)
        end = sc.n_draws if restore == LAYER_OPEN else restore
        for d in range(start, end):
            clips[d] = (0.0, 0.0, 0.0, 0.0) if narrowed is None else \
                map_clip(narrowed, tuple(float(v) for v in clips[d]))
        if narrowed is None:
            continue
        r = b._layers[0]
        r["start"], r["restore"] = start, restore
        recs.append(r)
    out.clips = clips
    out.layers = np.array(recs, LAYER_DTYPE) if recs else None
    return out


def layered_scene(seed, width, height, n_paths, n_layers, gradient_frac=0.3, stroke_frac=0.2,
                  blends=(BLEND_SRC_OVER,)) -> Scene:
    """Random paths (line/quad/cubic, both fill rules, gradients, strokes)
    with `n_layers` layers around runs of them: bounds over and past the
    canvas with fractional edges, alpha in [0.2, 1], blend modes from
    `blends`, some under a canvas translation and a narrowed clip."""
    sc = random_paths_scene(seed, width, height, n_paths, 2, 16,
                            coord_lo=(-16.0, -16.0), coord_hi=(width + 16.0, height + 16.0),
                            evenodd_frac=0.4, gradient_frac=gradient_frac,
                            stroke_frac=stroke_frac)
    R = random_streams(seed ^ 0x9E3779B97F4A7C15, max(n_layers, 1), 16)
    cuts = sorted(set(int(v) for v in randint(R[:, 0], 0, n_paths)))
    specs, prev = [], 0
    for i in range(n_layers):
        start = min(n_paths, prev + int(randint(R[i, 1:2], 0, max(1, n_paths // n_layers // 2))[0]))
        restore = min(n_paths, start + int(randint(R[i, 2:3], 0, max(1, n_paths // n_layers))[0]))
        prev = restore
        x0 = float(uniform(R[i, 3:4], -0.3 * width, 0.8 * width)[0])
        y0 = float(uniform(R[i, 4:5], -0.3 * height, 0.8 * height)[0])
        x1 = x0 + float(uniform(R[i, 5:6], 0.1 * width, 0.9 * width)[0])
        y1 = y0 + float(uniform(R[i, 6:7], 0.1 * height, 0.9 * height)[0])
        alpha = float(uniform(R[i, 7:8], 0.2, 1.0)[0])
        blend = blends[int(randint(R[i, 8:9], 0, len(blends) - 1)[0])]
        moved = u01(R[i, 9:10])[0] < 0.4
        tx = float(uniform(R[i, 10:11], -0.25 * width, 0.25 * width)[0]) if moved else 0.0
        ty = float(uniform(R[i, 11:12], -0.25 * height, 0.25 * height)[0]) if moved else 0.0
        clipped = u01(R[i, 12:13])[0] < 0.4
        clip = NO_CLIP if not clipped else (
            float(uniform(R[i, 13:14], -8.0, 0.4 * width)[0]),
            float(uniform(R[i, 14:15], -8.0, 0.4 * height)[0]),
            float(uniform(R[i, 15:16], 0.6 * width, width + 8.0)[0]), float(height) * 0.9)
        specs.append((start, restore, (x0, y0, x1, y1), alpha, blend, (tx, ty), clip))
    del cuts
    return with_layers(sc, specs)


def config1(seed=SEED_BASE + 1, n_paths=1000) -> Scene:
    """512x512, cleared white, 1,000 random filled paths of 3-32 verbs."""
    return random_paths_scene(seed, 512, 512, n_paths, 3, 32)


def config2(seed=SEED_BASE + 2, n_paths=20000, width=2048, height=2048) -> Scene:
    """2048x2048, 20,000 paths of 3-64 verbs over [-64,2112]^2; 30% even-odd;
    50% solid / 25% linear / 25% radial gradient; 20% stroked."""
    return random_paths_scene(seed, width, height, n_paths, 3, 64,
                              coord_lo=(-64.0, -64.0), coord_hi=(width + 64.0, height + 64.0),
                              evenodd_frac=0.3, gradient_frac=0.5, stroke_frac=0.2)


def config3(seed=SEED_BASE + 3, n_canvases=256, scale=1.0):
    """256 canvases with log-uniform sides in [64,1024] and log-uniform
    50-2,000 paths each, drawn as in config 1."""
    R = random_streams(seed, n_canvases, 4)
    out = []
    for i in range(n_canvases):
        w = int(round(float(loguniform(R[i, 0], 64, 1024))))
        h = int(round(float(loguniform(R[i, 1], 64, 1024))))
        n = max(1, int(round(float(loguniform(R[i, 2], 50, 2000)) * scale)))
        out.append(random_paths_scene(int(R[i, 3]), w, h, n, 3, 32))
    return out


def config4(seed=SEED_BASE + 4, n_outlines=100000, width=4096, height=4096,
            blur_frac=0.1) -> Scene:
    """4096x4096 glyph-dense scene: closed cubic outlines (8-40 verbs total,
    1-3 contours, inner contours smaller and wound the other way) scaled into
    8-48 px boxes at uniform positions, even-odd fill, solid colours; a tenth
    carry a kNormal blur mask filter with sigma ~ U[2,20] px, passed to
    MaskFilter::MakeBlur as the radius (sigma - 0.5) / 0.57735
    (src/effect/image_filter_base.hpp:32-41)."""
    A = 40
    K = 16 + 3 * A
    R = random_streams(seed, n_outlines, K)
    ncont = randint(R[:, 0], 1, 3)
    m = randint(R[:, 1], 8, 40)
    box = uniform(R[:, 2], 8.0, 48.0)
    px = u01(R[:, 3]) * (np.float32(width) - box)
    py = u01(R[:, 4]) * (np.float32(height) - box)
    rgb = [randint(R[:, 5 + i], 0, 255) for i in range(3)]
    alpha = uniform(R[:, 8], 0.3, 1.0)
    colors = _color4f_from_rgb_bytes(*rgb, alpha)
    blur = u01(R[:, 9]) < np.float32(blur_frac)
    sigma = uniform(R[:, 10], 2.0, 20.0)
    radius = ((sigma - np.float32(0.5)) / np.float32(0.57735)).astype(np.float32)
    rj = uniform(R[:, 16:16 + A], 0.75, 1.0)
    c1 = uniform(R[:, 16 + A:16 + 2 * A], 0.85, 1.15)
    c2 = uniform(R[:, 16 + 2 * A:16 + 3 * A], 0.85, 1.15)
    scales = np.array([1.0, 0.55, 0.3], np.float64)
    b = SceneBuilder(width, height)
    for i in range(n_outlines):
        k = int(ncont[i]); per = max(3, int(m[i]) // k)
        half = float(box[i]) * 0.5
        cx, cy = float(px[i]) + half, float(py[i]) + half
        verbs, pts, a0 = [], [], 0
        for j in range(k):
            rad = half * scales[j]
            direction = 1.0 if j == 0 else -1.0
            ang = direction * 2.0 * np.pi * np.arange(per + 1) / per
            rr = rj[i, a0:a0 + per].astype(np.float64)
            rr = np.concatenate([rr, rr[:1]])
            ax = cx + rad * rr * np.cos(ang); ay = cy + rad * rr * np.sin(ang)
            verbs.append(MOVE); pts.append((ax[0], ay[0]))
            for s in range(per):
                t1 = ang[s] + (ang[s + 1] - ang[s]) / 3.0
                t2 = ang[s] + 2.0 * (ang[s + 1] - ang[s]) / 3.0
                k1 = rad * float(c1[i, (a0 + s) % A]) * (rr[s] * 2 + rr[s + 1]) / 3.0
                k2 = rad * float(c2[i, (a0 + s) % A]) * (rr[s] + 2 * rr[s + 1]) / 3.0
                verbs.append(CUBIC)
                pts += [(cx + k1 * np.cos(t1), cy + k1 * np.sin(t1)),
                        (cx + k2 * np.cos(t2), cy + k2 * np.sin(t2)),
                        (ax[s + 1], ay[s + 1])]
            verbs.append(CLOSE)
            a0 += per
        p = default_paint()
        p["fill_type"] = EVEN_ODD
        p["fill_color"] = colors[i]
        p["stroke_color"] = colors[i]
        if blur[i]:
            p["blur_style"] = BLUR_NORMAL
            p["blur_radius"] = radius[i]
        b.draw_path(np.asarray(verbs, np.uint8), np.asarray(pts, np.float32), p)
    return b.build()
