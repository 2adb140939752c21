"""Python mirror of the skity drawing interface over the C ABI.

Names and argument meanings follow the reference's C++ API
(include/skity/graphic/path.hpp, paint.hpp, effect/shader.hpp,
effect/mask_filter.hpp, render/canvas.hpp) so tests read like the
reference's own: ``Path().MoveTo(..).LineTo(..)``, ``Paint().SetColor(..)``,
``Canvas.MakeCUDACanvas(bitmap)``, ``canvas.DrawPath(path, paint)``,
``canvas.Flush()``.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _lib
from . import scene as S

Style = type("Style", (), {"kFill_Style": 0, "kStroke_Style": 1, "kStrokeAndFill_Style": 2,
                           "kStrokeThenFill_Style": 3})
Cap = type("Cap", (), {"kButt_Cap": 0, "kRound_Cap": 1, "kSquare_Cap": 2})
Join = type("Join", (), {"kMiter_Join": 0, "kRound_Join": 1, "kBevel_Join": 2})
PathFillType = type("PathFillType", (), {"kWinding": 0, "kEvenOdd": 1})
# BlendMode (include/skity/graphic/blend_mode.hpp:45-80)
BlendMode = type("BlendMode", (), {n: i for i, n in enumerate(
    "kClear kSrc kDst kSrcOver kDstOver kSrcIn kDstIn kSrcOut kDstOut kSrcATop kDstATop kXor "
    "kPlus kModulate kScreen kOverlay kDarken kLighten kColorDodge kColorBurn kHardLight "
    "kSoftLight kDifference kExclusion kMultiply kHue kSaturation kColor kLuminosity".split())})
TileMode = type("TileMode", (), {"kClamp": 0, "kRepeat": 1, "kMirror": 2, "kDecal": 3})
BlurStyle = type("BlurStyle", (), {"kNormal": 1, "kSolid": 2, "kOuter": 3, "kInner": 4})


def ColorSetARGB(a, r, g, b) -> int:
    return ((a & 0xFF) << 24) | ((r & 0xFF) << 16) | ((g & 0xFF) << 8) | (b & 0xFF)


def Color4fFromColor(c: int) -> tuple:
    """src/graphic/color.cc:44-51: each channel / 255.f (float32)."""
    f = np.float32(255.0)
    return tuple(float(np.float32(v) / f) for v in
                 ((c >> 16) & 0xFF, (c >> 8) & 0xFF, c & 0xFF, (c >> 24) & 0xFF))


class Path:
    """skity::Path storage built with the same semantics as path.cc:494-569."""

    def __init__(self):
        self.verbs: list[int] = []
        self.points: list[tuple] = []
        self.weights: list[float] = []
        self.fill_type = PathFillType.kWinding
        self._last_move = ~0

    def _inject(self):
        if self._last_move < 0:
            p = (0.0, 0.0) if not self.verbs else self.points[~self._last_move]
            self.MoveTo(*p)

    def MoveTo(self, x, y):
        if self.verbs and self.verbs[-1] == S.MOVE:
            self.points[-1] = (x, y)
        else:
            self._last_move = len(self.points)
            self.verbs.append(S.MOVE)
            self.points.append((x, y))
        return self

    def LineTo(self, x, y):
        self._inject()
        self.verbs.append(S.LINE)
        self.points.append((x, y))
        return self

    def QuadTo(self, x1, y1, x2, y2):
        self._inject()
        self.verbs.append(S.QUAD)
        self.points += [(x1, y1), (x2, y2)]
        return self

    def ConicTo(self, x1, y1, x2, y2, w):
        if not w > 0:
            return self.LineTo(x2, y2)
        if np.isinf(w):
            return self.LineTo(x1, y1).LineTo(x2, y2)
        if w == 1.0:
            return self.QuadTo(x1, y1, x2, y2)
        self._inject()
        self.verbs.append(S.CONIC)
        self.weights.append(w)
        self.points += [(x1, y1), (x2, y2)]
        return self

    def CubicTo(self, x1, y1, x2, y2, x3, y3):
        self._inject()
        self.verbs.append(S.CUBIC)
        self.points += [(x1, y1), (x2, y2), (x3, y3)]
        return self

    def Close(self):
        if self.verbs and self.verbs[-1] != S.CLOSE:
            self.verbs.append(S.CLOSE)
        if self._last_move >= 0:
            self._last_move = ~self._last_move
        return self

    def AddRect(self, l, t, r, b):
        """Path::AddRect(rect) with the default direction (CW, start 0)."""
        return self.MoveTo(l, t).LineTo(r, t).LineTo(r, b).LineTo(l, b).Close()

    def AddOvalRRect(self, l, t, r, b):
        """Path::AddRRect of RRect::SetOval(rect) (src/geometry/rrect.cc:
        214-233, 353-367; src/graphic/path.cc:881-900, 1010-1040), the path
        Canvas::DrawOval and DrawCircle draw: the rect sorted; an empty one
        (or one with a zero half side) a rect path from its bottom-left
        corner (Path::AddRect, start index 3); otherwise four conics of
        weight FloatRoot2Over2, from (left, centre y) clockwise."""
        f = np.float32
        l, t, r, b = f(l), f(t), f(r), f(b)
        if not all(np.isfinite(v) for v in (l, t, r, b)):
            return self
        l, r = min(l, r), max(l, r)
        t, b = min(t, b), max(t, b)
        empty = not (l < r and t < b)
        half = f(0.5)
        if empty or f(r * half) - f(l * half) == 0 or f(b * half) - f(t * half) == 0:
            return self.MoveTo(l, b).LineTo(l, t).LineTo(r, t).LineTo(r, b).Close()
        cx, cy = f(half * f(r + l)), f(half * f(t + b))
        w = float(f(0.707106781))
        return (self.MoveTo(l, cy).ConicTo(l, t, cx, t, w).ConicTo(r, t, r, cy, w)
                .ConicTo(r, b, cx, b, w).ConicTo(l, b, l, cy, w).Close())

    def SetFillType(self, ft):
        self.fill_type = ft
        return self


class Image:
    """Image::MakeImage over an RGBA8 Pixmap: (height, width, 4) uint8
    pixels, AlphaType 2 (premultiplied) or 3 (unpremultiplied, the Pixmap
    default)."""
    def __init__(self, pixels, alpha_type=S.ALPHA_UNPREMUL):
        self.pixels = np.ascontiguousarray(pixels, np.uint8)
        assert self.pixels.ndim == 3 and self.pixels.shape[2] == 4
        self.alpha_type = alpha_type

    @staticmethod
    def MakeImage(pixels, alpha_type=S.ALPHA_UNPREMUL):
        return Image(pixels, alpha_type)

    def Width(self): return self.pixels.shape[1]

    def Height(self): return self.pixels.shape[0]

    def _struct(self, keep):
        im = _lib.Image_(self.Width(), self.Height(), self.alpha_type, 0, self.pixels.ctypes.data)
        keep += [self.pixels, im]
        return im


class FilterMode:
    kNearest, kLinear = 0, 1


class ImageShader:
    """Shader::MakeShader(image, sampling, x_tile_mode, y_tile_mode,
    local_matrix); local = (sx, kx, tx, ky, sy, ty), scale and translate."""
    def __init__(self, image, filter, tile_x, tile_y, local):
        self.image, self.filter, self.tile_x, self.tile_y = image, filter, tile_x, tile_y
        self.local = tuple(float(v) for v in local)


class Shader:
    @staticmethod
    def MakeShader(image, filter=FilterMode.kNearest, x_tile_mode=TileMode.kClamp,
                   y_tile_mode=TileMode.kClamp, local_matrix=(1.0, 0.0, 0.0, 0.0, 1.0, 0.0)):
        return ImageShader(image, filter, x_tile_mode, y_tile_mode, local_matrix)

    def __init__(self, kind, p0, p1, radius, colors, pos, tile):
        self.kind, self.p0, self.p1, self.radius = kind, p0, p1, radius
        self.colors = np.asarray(colors, np.float32).reshape(-1, 4)
        self.pos = None if pos is None else np.asarray(pos, np.float32)
        self.tile = tile

    @staticmethod
    def MakeLinear(pts, colors, pos, count, tile_mode=TileMode.kClamp):
        if count < 2:
            return None
        return Shader(S.GRAD_LINEAR, pts[0], pts[1], (0.0, 0.0), colors[:count], pos, tile_mode)

    @staticmethod
    def MakeRadial(center, radius, colors, pos, count, tile_mode=TileMode.kClamp):
        if count < 2 or radius < 0:
            return None
        return Shader(S.GRAD_RADIAL, center, (0.0, 0.0), (radius, 0.0), colors[:count], pos, tile_mode)

    @staticmethod
    def MakeSweep(cx, cy, start_angle, end_angle, colors, pos, count, tile_mode=TileMode.kClamp):
        """Shader::MakeSweep (src/effect/shader.cc:88-104): null for fewer
        than two stops or start >= end; the shader keeps bias = -start/360
        and scale = 1 / (end/360 - start/360), in float."""
        if count < 2 or not (start_angle < end_angle):
            return None
        f = np.float32
        t0, t1 = f(start_angle) / f(360), f(end_angle) / f(360)
        bias, scale = -t0, f(1) / (t1 - t0)
        return Shader(S.GRAD_SWEEP, (cx, cy), (0.0, 0.0), (float(bias), float(scale)),
                      colors[:count], pos, tile_mode)

    @staticmethod
    def MakeTwoPointConical(start, start_radius, end, end_radius, colors, pos, count,
                            tile_mode=TileMode.kClamp):
        """Shader::MakeTwoPointConical (src/effect/shader.cc:50-86): null for
        fewer than two stops or equal concentric circles; concentric with one
        radius zero is a radial gradient (reversed stops when the end radius
        is the zero one)."""
        if count < 2:
            return None
        f = np.float32
        near0 = lambda v: abs(f(v)) <= f(1.0 / (1 << 12))  # FloatNearlyZero
        same_radius = near0(f(start_radius) - f(end_radius))
        if near0(f(start[0]) - f(end[0])) and near0(f(start[1]) - f(end[1])):
            if same_radius:
                return None
            if near0(start_radius) or near0(end_radius):
                cols = np.asarray(colors, np.float32).reshape(-1, 4)[:count]
                if near0(end_radius):
                    rpos = None if pos is None else [float(f(1) - f(p)) for p in list(pos)[:count][::-1]]
                    return Shader(S.GRAD_RADIAL, start, (0.0, 0.0), (start_radius, 0.0),
                                  cols[::-1], rpos, tile_mode)
                return Shader(S.GRAD_RADIAL, start, (0.0, 0.0), (end_radius, 0.0), cols, pos,
                              tile_mode)
        return Shader(S.GRAD_CONICAL, start, end, (start_radius, end_radius), colors[:count], pos,
                      tile_mode)


class ColorFilter:
    """A colour filter as ColorFilterBase describes it (src/effect/
    color_filter_base.hpp): kind scene.FILTER_*, blend mode and ARGB colour,
    or the 20 row-major matrix terms."""

    def __init__(self, kind, mode=0, color=0, matrix=None):
        self.kind, self.mode, self.color = kind, mode, color
        self.matrix = None if matrix is None else [float(v) for v in np.asarray(matrix, np.float32).reshape(20)]

    def record(self):
        return S.filter_record(self.kind, self.mode, self.color, self.matrix)


class ColorFilters:
    """ColorFilters (include/skity/effect/color_filter.hpp; factories in
    src/effect/color_filter.cc:61-106)."""

    @staticmethod
    def Blend(color, mode):
        a = (int(color) >> 24) & 0xFF
        if mode == BlendMode.kDst or (mode == BlendMode.kDstIn and a == 255) or \
                (mode == BlendMode.kDstOut and a == 0):
            return None
        return ColorFilter(S.FILTER_BLEND, mode, int(color) & 0xFFFFFFFF)

    @staticmethod
    def Matrix(row_major):
        if row_major is None:
            return None
        m = np.asarray(row_major, np.float32).reshape(20)
        if np.array_equal(m, np.array([1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0],
                                      np.float32)):
            return None
        return ColorFilter(S.FILTER_MATRIX, matrix=m)

    @staticmethod
    def LinearToSRGBGamma():
        return ColorFilter(S.FILTER_LINEAR_TO_SRGB)

    @staticmethod
    def SRGBToLinearGamma():
        return ColorFilter(S.FILTER_SRGB_TO_LINEAR)

    @staticmethod
    def Compose(outer, inner):
        if inner is None:
            return outer
        if outer is None:
            return inner
        return ColorFilter(S.FILTER_COMPOSE)


class MaskFilter:
    def __init__(self, style, radius):
        self.style, self.radius = style, radius

    @staticmethod
    def MakeBlur(style, radius):
        return None if radius <= 0 else MaskFilter(style, radius)


class Paint:
    def __init__(self):
        self.rec = S.default_paint()
        self.shader: Shader | None = None
        self.mask_filter: MaskFilter | None = None
        self.color_filter: ColorFilter | None = None

    def SetStyle(self, s): self.rec["style"] = s; return self
    def SetStrokeWidth(self, w): self.rec["stroke_width"] = w; return self
    def SetStrokeMiter(self, m): self.rec["miter"] = m; return self
    def SetStrokeCap(self, c): self.rec["cap"] = c; return self
    def SetStrokeJoin(self, j): self.rec["join"] = j; return self
    def SetBlendMode(self, m): self.rec["blend"] = m; return self
    def SetColorFilter(self, f): self.color_filter = f; return self
    def SetShader(self, s): self.shader = s; return self
    def SetMaskFilter(self, m): self.mask_filter = m; return self

    def SetColor(self, c: int):
        self.rec["fill_color"] = self.rec["stroke_color"] = Color4fFromColor(c)
        return self

    def SetFillColor(self, r, g, b, a): self.rec["fill_color"] = (r, g, b, a); return self
    def SetStrokeColor(self, r, g, b, a): self.rec["stroke_color"] = (r, g, b, a); return self

    def SetAlphaF(self, a):
        a = float(np.clip(np.float32(a), 0, 1))
        self.rec["fill_color"][3] = a
        self.rec["stroke_color"][3] = a
        return self


class Context:
    """One CUDA device context (skity_cuda_context)."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        self.lib = _lib.load()
        info = _lib.ContextInfo_(ctypes.sizeof(_lib.ContextInfo_), device, budget_bytes)
        h = ctypes.c_void_p()
        _lib.check(self.lib.skity_cuda_context_create(ctypes.byref(info), ctypes.byref(h)),
                   "skity_cuda_context_create")
        self.handle = h
        # batches and canvases made on this context: closed before it is
        self._dependents = weakref.WeakSet()

    def stats(self) -> dict:
        st = _lib.Stats_()
        _lib.check(self.lib.skity_cuda_context_get_stats(self.handle, ctypes.byref(st)), "get_stats")
        return st.as_dict()

    def close(self):
        if self.handle:
            for d in list(self._dependents):
                d.close()
            self.lib.skity_cuda_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- batched form over scene streams
    def render_streams(self, scenes: list, out: list | None = None) -> list:
        """skity_cuda_render_streams: the scenes parsed, rendered and read
        back in one call.  `out`: the canvases' pixel arrays to fill
        ((height, width, 4) uint8, C-contiguous -- page-locked host memory
        makes the read-back a direct copy); new arrays when None."""
        bufs = [s.to_bytes() for s in scenes]
        if out is None:
            outs = [np.zeros((s.height, s.width, 4), np.uint8) for s in scenes]
        else:
            outs = list(out)
            if len(outs) != len(scenes) or any(
                    o.shape != (s.height, s.width, 4) or o.dtype != np.uint8 or
                    not o.flags["C_CONTIGUOUS"] for o, s in zip(outs, scenes)):
                raise ValueError("render_streams: out must hold one (height, width, 4) uint8 "
                                 "C-contiguous array per scene")
        n = len(bufs)
        cbufs = [ctypes.create_string_buffer(b, len(b)) for b in bufs]
        ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(c) for c in cbufs])
        lens = (ctypes.c_size_t * n)(*[len(b) for b in bufs])
        optr = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
        _lib.check(self.lib.skity_cuda_render_streams(self.handle, n, ptrs, lens, optr),
                   "skity_cuda_render_streams")
        return outs


class Batch:
    """Device-resident batch of scene streams (skity_cuda_batch)."""

    def __init__(self, ctx: Context, scenes: list):
        self.ctx, self.lib = ctx, ctx.lib
        self.sizes = [(s.height, s.width) for s in scenes]
        bufs = [s.to_bytes() for s in scenes]
        n = len(bufs)
        cbufs = [ctypes.create_string_buffer(b, len(b)) for b in bufs]
        ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(c) for c in cbufs])
        lens = (ctypes.c_size_t * n)(*[len(b) for b in bufs])
        h = ctypes.c_void_p()
        _lib.check(self.lib.skity_cuda_batch_create(ctx.handle, n, ptrs, lens, ctypes.byref(h)),
                   "skity_cuda_batch_create")
        self.handle = h
        ctx._dependents.add(self)

    def render(self) -> dict:
        _lib.check(self.lib.skity_cuda_batch_render(self.handle), "skity_cuda_batch_render")
        return self.ctx.stats()

    def render_per_draw(self) -> dict:
        """skity_cuda_batch_render_per_draw: the same canvases rendered one
        DrawPath at a time (the plain per-draw form)."""
        _lib.check(self.lib.skity_cuda_batch_render_per_draw(self.handle),
                   "skity_cuda_batch_render_per_draw")
        return self.ctx.stats()

    def set_config(self, tile_width: int = 256, ctas_per_sm: int = 4, band_rows: int = 16,
                   sweep_warps: int = 2):
        """skity_cuda_batch_set_config: the compositor's launch shape, bin
        granularity and the register sweeps' warps per CTA (the pixels do not
        change); the next render replans."""
        c = _lib.RasterConfig_(ctypes.sizeof(_lib.RasterConfig_), tile_width, ctas_per_sm,
                               band_rows, sweep_warps)
        _lib.check(self.lib.skity_cuda_batch_set_config(self.handle, ctypes.byref(c)),
                   "skity_cuda_batch_set_config")

    def config(self) -> dict:
        c = _lib.RasterConfig_()
        _lib.check(self.lib.skity_cuda_batch_get_config(self.handle, ctypes.byref(c)),
                   "skity_cuda_batch_get_config")
        return {"tile_width": c.tile_width, "ctas_per_sm": c.ctas_per_sm, "band_rows": c.band_rows,
                "sweep_warps": c.sweep_warps}

    def read(self, i: int, out: np.ndarray | None = None) -> np.ndarray:
        h, w = self.sizes[i]
        if out is None:
            out = np.zeros((h, w, 4), np.uint8)
        _lib.check(self.lib.skity_cuda_batch_read(self.handle, i, out.ctypes.data), "batch_read")
        return out

    def close(self):
        if self.handle:
            self.lib.skity_cuda_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Canvas:
    """A CUDA canvas over a caller-owned premultiplied RGBA8 bitmap
    (numpy array of shape (h, w, 4), uint8), created the way
    Canvas::MakeSoftwareCanvas(Bitmap*) creates the software canvas."""

    def __init__(self, ctx: Context, handle, bitmap: np.ndarray):
        self.ctx, self.lib, self.handle, self.bitmap = ctx, ctx.lib, handle, bitmap
        deps = getattr(ctx, "_dependents", None)  # a recorder's canvas has no context
        if deps is not None:
            deps.add(self)

    @staticmethod
    def MakeCUDACanvas(ctx: Context, bitmap: np.ndarray | None):
        """Returns None for a missing or empty bitmap, like MakeSoftwareCanvas."""
        if bitmap is None or bitmap.size == 0:
            return None
        assert bitmap.dtype == np.uint8 and bitmap.ndim == 3 and bitmap.shape[2] == 4
        assert bitmap.flags["C_CONTIGUOUS"]
        h = ctypes.c_void_p()
        rc = ctx.lib.skity_cuda_canvas_create(ctx.handle, bitmap.shape[1], bitmap.shape[0],
                                              bitmap.ctypes.data, bitmap.strides[0], ctypes.byref(h))
        if rc == -2:
            return None
        _lib.check(rc, "skity_cuda_canvas_create")
        return Canvas(ctx, h, bitmap)

    def Clear(self, color):
        c4 = Color4fFromColor(color) if isinstance(color, int) else tuple(color)
        arr = (ctypes.c_float * 4)(*c4)
        _lib.check(self.lib.skity_cuda_canvas_clear(self.handle, arr), "skity_cuda_canvas_clear")

    def DrawOval(self, left, top, right, bottom, paint: Paint):
        """Canvas::DrawOval(rect, paint) (canvas.cc:202-204, 418-430): the
        oval's RRect path (Path.AddOvalRRect), drawn as DrawPath."""
        self.DrawPath(Path().AddOvalRRect(left, top, right, bottom), paint)

    def DrawCircle(self, cx, cy, radius, paint: Paint):
        """Canvas::DrawCircle (canvas.cc:178-180, 407-416): a negative radius
        is 0; the oval of the circle's bounds."""
        f = np.float32
        cx, cy, radius = f(cx), f(cy), f(radius)
        if radius < 0:
            radius = f(0)
        self.DrawOval(cx - radius, cy - radius, cx + radius, cy + radius, paint)

    def DrawRect(self, left, top, right, bottom, paint: Paint):
        """Canvas::DrawRect (canvas.cc:206-208, 432-437): Path::AddRect."""
        self.DrawPath(Path().AddRect(left, top, right, bottom), paint)

    def DrawPath(self, path: Path, paint: Paint):
        verbs = np.asarray(path.verbs, np.uint8)
        pts = np.asarray(path.points, np.float32).reshape(-1, 2)
        wts = np.asarray(path.weights, np.float32)
        cp = _lib.Path_(verbs.ctypes.data if len(verbs) else None, len(verbs),
                        pts.ctypes.data if len(pts) else None, len(pts),
                        wts.ctypes.data if len(wts) else None, len(wts), path.fill_type)
        keep = []
        cpaint = self._paint_struct(paint, keep)
        _lib.check(self.lib.skity_cuda_canvas_draw_path(self.handle, ctypes.byref(cp),
                                                        ctypes.byref(cpaint)),
                   "skity_cuda_canvas_draw_path")

    def DrawImageRect(self, image, src, dst, filter=FilterMode.kNearest, paint=None):
        """Canvas::DrawImageRect(image, src, dst, sampling, paint); src and
        dst are (left, top, right, bottom)."""
        keep = []
        im = image._struct(keep) if image is not None else None
        s4 = (ctypes.c_float * 4)(*[float(v) for v in src])
        d4 = (ctypes.c_float * 4)(*[float(v) for v in dst])
        cpaint = self._paint_struct(paint, keep) if paint is not None else None
        _lib.check(self.lib.skity_cuda_canvas_draw_image_rect(
            self.handle, ctypes.byref(im) if im is not None else None, s4, d4, int(filter),
            ctypes.byref(cpaint) if cpaint is not None else None),
            "skity_cuda_canvas_draw_image_rect")

    def DrawImage(self, image, left, top, filter=FilterMode.kNearest, paint=None):
        """Canvas::DrawImage(image, x, y, sampling, paint): the whole image
        at (x, y)."""
        w, h = image.Width(), image.Height()
        self.DrawImageRect(image, (0, 0, w, h), (left, top, left + w, top + h), filter, paint)

    def _paint_struct(self, paint, keep):
        r = paint.rec
        cpaint = _lib.Paint_()
        cpaint.style, cpaint.cap, cpaint.join, cpaint.blend_mode = (int(r["style"]), int(r["cap"]),
                                                                    int(r["join"]), int(r["blend"]))
        cpaint.fill_color[:] = [float(v) for v in r["fill_color"]]
        cpaint.stroke_color[:] = [float(v) for v in r["stroke_color"]]
        cpaint.stroke_width = float(r["stroke_width"])
        cpaint.miter_limit = float(r["miter"])
        if isinstance(paint.shader, ImageShader):
            sh = paint.shader
            ish = _lib.ImageShader_()
            ish.image = ctypes.pointer(sh.image._struct(keep))
            ish.filter, ish.tile_x, ish.tile_y = sh.filter, sh.tile_x, sh.tile_y
            ish.local_matrix[:] = list(sh.local)
            keep.append(ish)
            cpaint.image_shader = ctypes.pointer(ish)
        elif paint.shader is not None:
            s = paint.shader
            colors = np.ascontiguousarray(s.colors, np.float32)
            offs = None if s.pos is None else np.ascontiguousarray(s.pos, np.float32)
            keep += [colors, offs]
            g = _lib.Gradient_()
            g.type, g.tile_mode, g.stop_count = s.kind, s.tile, len(colors)
            g.has_offsets = 0 if offs is None else 1
            g.p0[:] = list(s.p0)
            g.p1[:] = list(s.p1)
            g.radius[:] = list(s.radius)
            g.colors = colors.ctypes.data
            g.offsets = None if offs is None else offs.ctypes.data
            keep.append(g)
            cpaint.shader = ctypes.pointer(g)
        if paint.mask_filter is not None:
            cpaint.blur_style = paint.mask_filter.style
            cpaint.blur_radius = paint.mask_filter.radius
        if paint.color_filter is not None:
            cf = _lib.ColorFilter_()
            cf.type, cf.blend_mode, cf.color = (paint.color_filter.kind, paint.color_filter.mode,
                                                paint.color_filter.color)
            if paint.color_filter.matrix is not None:
                cf.matrix[:] = paint.color_filter.matrix
            keep.append(cf)
            cpaint.color_filter = ctypes.pointer(cf)
        return cpaint

    def Save(self):
        _lib.check(self.lib.skity_cuda_canvas_save(self.handle), "skity_cuda_canvas_save")

    def Restore(self):
        _lib.check(self.lib.skity_cuda_canvas_restore(self.handle), "skity_cuda_canvas_restore")

    def SaveLayer(self, bounds, paint: "Paint | None" = None):
        """Canvas::SaveLayer(bounds, paint): the draws until the matching
        Restore go to a layer, composited at the Restore with the paint's
        alpha and blend mode."""
        b = (ctypes.c_float * 4)(*[float(v) for v in bounds])
        keep = []
        cp = self._paint_struct(paint, keep) if paint is not None else None
        _lib.check(self.lib.skity_cuda_canvas_save_layer(
            self.handle, b, ctypes.byref(cp) if cp is not None else None),
            "skity_cuda_canvas_save_layer")

    def Translate(self, dx, dy):
        _lib.check(self.lib.skity_cuda_canvas_translate(self.handle, float(dx), float(dy)),
                   "skity_cuda_canvas_translate")

    def Scale(self, sx, sy):
        _lib.check(self.lib.skity_cuda_canvas_scale(self.handle, float(sx), float(sy)),
                   "skity_cuda_canvas_scale")

    def Rotate(self, degrees, px=0.0, py=0.0):
        """Canvas::Rotate(degrees) / Rotate(degrees, px, py)."""
        _lib.check(self.lib.skity_cuda_canvas_rotate(self.handle, float(degrees), float(px),
                                                     float(py)), "skity_cuda_canvas_rotate")

    def Skew(self, sx, sy):
        _lib.check(self.lib.skity_cuda_canvas_skew(self.handle, float(sx), float(sy)),
                   "skity_cuda_canvas_skew")

    def Concat(self, m9):
        """Canvas::Concat(matrix); m9 row-major as Matrix::Set9 takes it."""
        m = (ctypes.c_float * 9)(*[float(v) for v in m9])
        _lib.check(self.lib.skity_cuda_canvas_concat(self.handle, m), "skity_cuda_canvas_concat")

    def SetMatrix(self, m9):
        m = (ctypes.c_float * 9)(*[float(v) for v in m9])
        _lib.check(self.lib.skity_cuda_canvas_set_matrix(self.handle, m),
                   "skity_cuda_canvas_set_matrix")

    def Concat44(self, m16):
        """Canvas::Concat of a 4x4 Matrix given column-major."""
        m = (ctypes.c_float * 16)(*[float(v) for v in m16])
        _lib.check(self.lib.skity_cuda_canvas_concat44(self.handle, m),
                   "skity_cuda_canvas_concat44")

    def SetMatrix44(self, m16):
        m = (ctypes.c_float * 16)(*[float(v) for v in m16])
        _lib.check(self.lib.skity_cuda_canvas_set_matrix44(self.handle, m),
                   "skity_cuda_canvas_set_matrix44")

    def GetTotalMatrix(self):
        """The canvas matrix as Matrix::Get9 gives it (row-major 3x3)."""
        m = (ctypes.c_float * 9)()
        _lib.check(self.lib.skity_cuda_canvas_get_matrix(self.handle, m),
                   "skity_cuda_canvas_get_matrix")
        return tuple(float(v) for v in m)

    def ClipPath(self, path: Path, op=1):
        """Canvas::ClipPath(path, op): op 0 kDifference, 1 kIntersect."""
        verbs = np.asarray(path.verbs, np.uint8)
        pts = np.asarray(path.points, np.float32).reshape(-1, 2)
        wts = np.asarray(path.weights, np.float32)
        cp = _lib.Path_(verbs.ctypes.data if len(verbs) else None, len(verbs),
                        pts.ctypes.data if len(pts) else None, len(pts),
                        wts.ctypes.data if len(wts) else None, len(wts), path.fill_type)
        _lib.check(self.lib.skity_cuda_canvas_clip_path(self.handle, ctypes.byref(cp), int(op)),
                   "skity_cuda_canvas_clip_path")

    def ClipRect(self, left, top, right, bottom):
        """Canvas::ClipRect(rect, ClipOp::kIntersect) under the current
        translation; Save / Restore keep and restore the clip."""
        _lib.check(self.lib.skity_cuda_canvas_clip_rect(self.handle, float(left), float(top),
                                                        float(right), float(bottom)),
                   "skity_cuda_canvas_clip_rect")

    def Flush(self):
        _lib.check(self.lib.skity_cuda_canvas_flush(self.handle), "skity_cuda_canvas_flush")

    def close(self):
        if self.handle:
            self.lib.skity_cuda_canvas_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PictureRecorder:
    """PictureRecorder (include/skity/recorder/picture_recorder.hpp):
    BeginRecording returns a canvas whose calls are recorded, and
    FinishRecording the DisplayList holding them.  Needs no GPU."""

    def __init__(self):
        self.lib = _lib.load()
        self.canvas = None

    def BeginRecording(self, bounds):
        """bounds: (left, top, right, bottom) of the recording, as the
        reference takes it; the recorded canvas is right x bottom pixels."""
        w, h = int(round(bounds[2])), int(round(bounds[3]))
        hdl = ctypes.c_void_p()
        _lib.check(self.lib.skity_cuda_recorder_begin(w, h, ctypes.byref(hdl)),
                   "skity_cuda_recorder_begin")
        self.canvas = Canvas(_RecorderContext(self.lib), hdl, None)
        self.size = (w, h)
        return self.canvas

    def GetRecordingCanvas(self):
        return self.canvas

    def FinishRecording(self) -> "DisplayList":
        dl = ctypes.c_void_p()
        _lib.check(self.lib.skity_cuda_recorder_finish(self.canvas.handle, ctypes.byref(dl)),
                   "skity_cuda_recorder_finish")
        self.canvas.close()
        self.canvas = None
        return DisplayList(self.lib, dl, self.size)


class _RecorderContext:
    """Stands in for a Context for a recorder's canvas (it draws nothing)."""

    def __init__(self, lib):
        self.lib, self.handle = lib, None


class DisplayList:
    """DisplayList (include/skity/recorder/display_list.hpp): Draw(canvas)
    replays the recorded calls on a canvas; to_stream() / to_scene() give
    the scene stream the batched and serving forms take."""

    def __init__(self, lib, handle, size):
        self.lib, self.handle, self.size = lib, handle, size

    def GetOpCount(self) -> int:
        return int(self.lib.skity_cuda_display_list_op_count(self.handle))

    def Draw(self, canvas: "Canvas"):
        _lib.check(self.lib.skity_cuda_display_list_draw(self.handle, canvas.handle),
                   "skity_cuda_display_list_draw")

    def to_stream(self) -> bytes:
        n = ctypes.c_size_t(0)
        _lib.check(self.lib.skity_cuda_display_list_to_stream(self.handle, None, ctypes.byref(n)),
                   "skity_cuda_display_list_to_stream")
        buf = ctypes.create_string_buffer(n.value)
        _lib.check(self.lib.skity_cuda_display_list_to_stream(self.handle, buf, ctypes.byref(n)),
                   "skity_cuda_display_list_to_stream")
        return buf.raw[:n.value]

    def to_scene(self):
        from . import scene as S
        return S.Scene.from_bytes(self.to_stream())

    def close(self):
        if self.handle:
            self.lib.skity_cuda_display_list_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceCanvas:
    """The plain per-draw form: a premultiplied RGBA8 canvas held in device
    memory (any CUDA allocation, e.g. a torch uint8 tensor of shape
    (h, w, 4)) drawn one DrawPath at a time through
    skity_cuda_draw_path_static -- geometry, sweeps and composite launched
    for every draw, as the software canvas rasterises every draw on its own.
    Solid-colour paints only (no shader, no mask filter)."""

    def __init__(self, device_ptr: int, width: int, height: int, row_bytes: int | None = None,
                 device: int = 0, stream: int = 0):
        self.lib = _lib.load()
        self.ptr, self.width, self.height = int(device_ptr), int(width), int(height)
        self.row_bytes = int(row_bytes) if row_bytes else 4 * self.width
        self.device, self.stream = device, stream

    def draw_record(self, verbs, points, weights, rec) -> None:
        """DrawPath of one scene draw (path arrays + paint record)."""
        verbs = np.ascontiguousarray(verbs, np.uint8)
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 2)
        wts = np.ascontiguousarray(weights, np.float32)
        cp = _lib.Path_(verbs.ctypes.data if len(verbs) else None, len(verbs),
                        pts.ctypes.data if len(pts) else None, len(pts),
                        wts.ctypes.data if len(wts) else None, len(wts), int(rec["fill_type"]))
        p = _lib.Paint_()
        p.style, p.cap, p.join, p.blend_mode = (int(rec["style"]), int(rec["cap"]),
                                                int(rec["join"]), int(rec["blend"]))
        p.fill_color[:] = [float(v) for v in rec["fill_color"]]
        p.stroke_color[:] = [float(v) for v in rec["stroke_color"]]
        p.stroke_width = float(rec["stroke_width"])
        p.miter_limit = float(rec["miter"])
        _lib.check(self.lib.skity_cuda_draw_path_static(self.device, self.ptr, self.width,
                                                        self.height, self.row_bytes,
                                                        ctypes.byref(cp), ctypes.byref(p),
                                                        self.stream or None),
                   "skity_cuda_draw_path_static")

    def DrawPath(self, path: Path, paint: Paint) -> None:
        if paint.shader is not None or paint.mask_filter is not None:
            raise _lib.SkityCudaError(-5, "DeviceCanvas.DrawPath (solid colours only)")
        rec = paint.rec.copy()
        rec["fill_type"] = path.fill_type
        self.draw_record(path.verbs, path.points, path.weights, rec)

    def draw_scene(self, sc) -> int:
        """Every draw of a scene (solid colours) in order; returns the count."""
        for d in range(sc.n_draws):
            v0, v1 = int(sc.verb_off[d]), int(sc.verb_off[d + 1])
            p0, p1 = int(sc.point_off[d]), int(sc.point_off[d + 1])
            w0, w1 = int(sc.weight_off[d]), int(sc.weight_off[d + 1])
            self.draw_record(sc.verbs[v0:v1], sc.points[p0:p1], sc.weights[w0:w1], sc.paints[d])
        return sc.n_draws


class Server:
    """The serving loop (skity_cuda_server): requests are scene streams of
    one canvas each, admitted against a device-memory budget and rendered in
    continuously formed batches by `workers` concurrent workers."""

    def __init__(self, device: int = 0, budget_bytes: int = 0, workers: int = 0,
                 max_batch: int = 0):
        self.lib = _lib.load()
        info = _lib.ServerInfo_(ctypes.sizeof(_lib.ServerInfo_), device, budget_bytes, workers,
                                max_batch)
        h = ctypes.c_void_p()
        _lib.check(self.lib.skity_cuda_server_create(ctypes.byref(info), ctypes.byref(h)),
                   "skity_cuda_server_create")
        self.handle = h
        self.sizes = {}

    def submit(self, scene=None, stream: bytes | None = None) -> int:
        b = stream if stream is not None else scene.to_bytes()
        sc = scene if scene is not None else S.Scene.from_bytes(b)
        t = ctypes.c_uint64()
        _lib.check(self.lib.skity_cuda_server_submit(self.handle, b, len(b), ctypes.byref(t)),
                   "skity_cuda_server_submit")
        self.sizes[t.value] = (sc.height, sc.width)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000, want_pixels: bool = True):
        """(pixels or None, info dict); raises on error; returns (None, None)
        when the request is not done within the timeout."""
        if ticket not in self.sizes:  # unknown or released: the C ABI reports it
            want_pixels = False
        h, w = self.sizes.get(ticket, (0, 0))
        out = np.zeros((h, w, 4), np.uint8) if want_pixels else None
        info = _lib.RequestInfo_()
        rc = self.lib.skity_cuda_server_wait(self.handle, ticket, timeout_ms,
                                             out.ctypes.data if want_pixels else None,
                                             ctypes.byref(info))
        if rc == _lib.NOT_READY:
            return None, None
        self.sizes.pop(ticket, None)
        _lib.check(rc, "skity_cuda_server_wait")
        return out, {"queue_ms": info.queue_ms, "latency_ms": info.latency_ms,
                     "batch_size": info.batch_size}

    def close(self):
        if self.handle:
            self.lib.skity_cuda_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
