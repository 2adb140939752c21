"""SKP import: Skia picture files, as the reference's IO module reads them
(module/io/src/picture.cc, record/record_playback.cc, io/memory_read.cc,
io/flat/{paint,path,matrix}_flat.cc), played onto a canvas of this package.

The reader keeps the reference's reading of the format: the picture header
(magic, version 82..109, cull rect), the stream tags ('read' op data,
'fact' factory names, 'tpfc' typefaces, 'aray' the flattened buffers: 'pnt '
paints, 'pth ' paths), and op records of (op << 24 | size) words.  Paints
keep stroke width, miter, colour (Color4f -> Color -> Color4f, as
Paint::SetColor does), the packed anti-alias / blend / cap / join / style
bits; paths are rebuilt through Path's own builder calls (MoveTo / LineTo /
QuadTo / ConicTo / CubicTo / Close) with their fill type.

Ops taken: SAVE, RESTORE, CONCAT, CONCAT44, SET_MATRIX, SET_M44, TRANSLATE,
SCALE, ROTATE, SKEW, CLIP_RECT, CLIP_PATH, DRAW_PATH, DRAW_RECT, DRAW_CLEAR,
NOOP, FLUSH, PUSH_CULL, POP_CULL.  Anything else -- text, images, ovals and
round rects, pictures, paints with effects (shaders, filters, path effects),
inverse fill types -- raises SkpError naming it: the GPU path would not draw
it, so a partial scene is never passed off as the picture.
"""
from __future__ import annotations

import struct

import numpy as np

from . import scene as S

MAGIC = b"skiapict"
MIN_VERSION, MAX_VERSION = 82, 109  # Version::kMin_Version .. kCurrent_Version

# DrawType (module/io/src/record/draw_type.hpp): the values this reader takes
CLIP_PATH, CLIP_RECT, CONCAT, DRAW_CLEAR, DRAW_PATH, DRAW_RECT = 1, 3, 5, 10, 14, 21
RESTORE, ROTATE, SAVE, SCALE, SET_MATRIX, SKEW, TRANSLATE, NOOP = 28, 29, 30, 32, 33, 34, 35, 36
PUSH_CULL, POP_CULL, FLUSH, CONCAT44, SET_M44 = 41, 42, 63, 68, 71
OP_NAMES = {1: "CLIP_PATH", 2: "CLIP_REGION", 3: "CLIP_RECT", 4: "CLIP_RRECT", 5: "CONCAT",
            10: "DRAW_CLEAR", 11: "DRAW_DATA", 12: "DRAW_OVAL", 13: "DRAW_PAINT",
            14: "DRAW_PATH", 15: "DRAW_PICTURE", 16: "DRAW_POINTS", 21: "DRAW_RECT",
            22: "DRAW_RRECT", 28: "RESTORE", 29: "ROTATE", 30: "SAVE", 32: "SCALE",
            33: "SET_MATRIX", 34: "SKEW", 35: "TRANSLATE", 36: "NOOP", 40: "DRAW_DRRECT",
            41: "PUSH_CULL", 42: "POP_CULL", 43: "DRAW_PATCH", 44: "DRAW_PICTURE_MATRIX_PAINT",
            45: "DRAW_TEXT_BLOB", 46: "DRAW_IMAGE", 48: "DRAW_ATLAS", 49: "DRAW_IMAGE_NINE",
            50: "DRAW_IMAGE_RECT", 52: "SAVE_LAYER_SAVELAYERREC", 53: "DRAW_ANNOTATION",
            54: "DRAW_DRAWABLE", 55: "DRAW_DRAWABLE_MATRIX", 58: "DRAW_SHADOW_REC",
            59: "DRAW_IMAGE_LATTICE", 60: "DRAW_ARC", 61: "DRAW_REGION",
            62: "DRAW_VERTICES_OBJECT", 63: "FLUSH", 64: "DRAW_EDGEAA_IMAGE_SET",
            65: "SAVE_BEHIND", 66: "DRAW_EDGEAA_QUAD", 67: "DRAW_BEHIND_PAINT",
            68: "CONCAT44", 69: "CLIP_SHADER_IN_PAINT", 70: "MARK_CTM", 71: "SET_M44",
            72: "DRAW_IMAGE2", 73: "DRAW_IMAGE_RECT2", 74: "DRAW_IMAGE_LATTICE2",
            75: "DRAW_EDGEAA_IMAGE_SET2", 76: "RESET_CLIP", 77: "DRAW_SLUG"}


def _tag(a: str) -> int:
    return (ord(a[0]) << 24) | (ord(a[1]) << 16) | (ord(a[2]) << 8) | ord(a[3])


TAG_READER, TAG_FACTORY, TAG_TYPEFACE, TAG_PICTURE = _tag("read"), _tag("fact"), _tag("tpfc"), _tag("pctr")
TAG_ARRAY, TAG_PAINT, TAG_PATH, TAG_EOF = _tag("aray"), _tag("pnt "), _tag("pth "), _tag("eof ")
HAS_EFFECTS = 0x2  # paint flat flag: flattenables (shader, filters, path effect, blender) follow


class SkpError(ValueError):
    pass


class _Reader:
    """Little-endian reads over a byte string, 4-byte padded where the
    reference's ReadBuffer pads."""

    def __init__(self, data: bytes, off: int = 0, end: int | None = None):
        self.b, self.o = data, off
        self.end = len(data) if end is None else end

    def need(self, n):
        if self.o + n > self.end:
            raise SkpError("truncated picture data")

    def u8(self):
        self.need(1)
        v = self.b[self.o]
        self.o += 1
        return v

    def u32(self):
        self.need(4)
        v, = struct.unpack_from("<I", self.b, self.o)
        self.o += 4
        return v

    def i32(self):
        self.need(4)
        v, = struct.unpack_from("<i", self.b, self.o)
        self.o += 4
        return v

    def f32(self, n=1):
        self.need(4 * n)
        v = np.frombuffer(self.b, np.float32, n, self.o).copy()
        self.o += 4 * n
        return v

    def raw(self, n):
        self.need(n)
        v = self.b[self.o:self.o + n]
        self.o += n
        return v

    def align4(self):
        self.o = (self.o + 3) & ~3

    def packed_uint(self):  # ReadStream::ReadPackedUint (stream.cc:106-131)
        v = self.u8()
        if v == 0xFE:
            self.need(2)
            v, = struct.unpack_from("<H", self.b, self.o)
            self.o += 2
        elif v == 0xFF:
            v = self.u32()
        return v


def _color4f_to_color(c) -> int:
    """Color4fToColor (src/graphic/color.cc:53-59): each channel times 255 in
    float, clamped to [0, 255], truncated to a byte."""
    f = np.float32
    out = []
    for v in (c[3], c[0], c[1], c[2]):  # a, r, g, b
        x = f(f(v) * f(255))
        x = min(max(x, f(0)), f(255)) if not np.isnan(x) else f(0)
        out.append(int(x))
    a, r, g, b = out
    return (a << 24) | (r << 16) | (g << 8) | b


class SkpPaint:
    """A paint record as ReadFromMemory<Paint> (paint_flat.cc:145-186)
    leaves it."""

    def __init__(self, r: _Reader):
        self.stroke_width = float(r.f32()[0])
        self.miter = float(r.f32()[0])
        c4 = r.f32(4)
        self.color = _color4f_to_color(c4)  # Paint::SetColor(Color4fToColor(c))
        packed = r.u32()
        self.anti_alias = (packed & 1) != 0
        packed >>= 8
        mode = packed & 0xFF
        self.blend = 3 if mode == 0xFF else min(mode, 28)  # kSrcOver by default
        packed >>= 8
        self.cap = packed & 3
        packed >>= 2
        self.join = packed & 3
        packed >>= 2
        self.style = packed & 3
        packed >>= 4
        self.flat_flags = packed & 0xFF
        if self.flat_flags & HAS_EFFECTS:
            # the flattenables (path effect, shader, mask filter, colour filter,
            # image filter, blender) are not taken
            raise SkpError("paint with effects (shader, filter, path effect or blender)")

    def to_paint(self):
        from .canvas import Paint
        p = Paint()
        p.SetColor(self.color)
        p.SetStrokeWidth(self.stroke_width)
        p.SetStrokeMiter(self.miter)
        p.SetStyle(self.style)
        p.SetStrokeCap(self.cap)
        p.SetStrokeJoin(self.join)
        p.SetBlendMode(self.blend)
        return p


def _read_path(r: _Reader):
    """ReadFromMemory<Path> (path_flat.cc:226-305): packed version / type /
    fill type, then point, weight and verb counts, points, weights, verbs."""
    from .canvas import Path
    packed = r.u32()
    version = packed & 0xFF
    if version not in (4, 5):
        raise SkpError(f"path serialization version {version}")
    if (packed >> 28) & 0xF != 0:
        raise SkpError("round-rect path record")
    fill = (packed >> 8) & 0x3
    npts, ncnx, nvbs = r.i32(), r.i32(), r.i32()
    if min(npts, ncnx, nvbs) < 0:
        raise SkpError("bad path counts")
    path = Path()
    if nvbs == 0:
        if npts or ncnx:
            raise SkpError("path with points and no verbs")
        return path
    pts = r.f32(2 * npts).reshape(-1, 2)
    wts = r.f32(ncnx)
    verbs = r.raw(nvbs)
    r.align4()
    pi = wi = 0
    for v in verbs:  # fill_path (path_flat.cc:148-182)
        if v == S.MOVE:
            path.MoveTo(float(pts[pi][0]), float(pts[pi][1]))
            pi += 1
        elif v == S.LINE:
            path.LineTo(float(pts[pi][0]), float(pts[pi][1]))
            pi += 1
        elif v == S.QUAD:
            path.QuadTo(*(float(x) for x in pts[pi:pi + 2].reshape(-1)))
            pi += 2
        elif v == S.CUBIC:
            path.CubicTo(*(float(x) for x in pts[pi:pi + 3].reshape(-1)))
            pi += 3
        elif v == S.CONIC:
            path.ConicTo(*(float(x) for x in pts[pi:pi + 2].reshape(-1)), float(wts[wi]))
            pi += 2
            wi += 1
        elif v == S.CLOSE:
            path.Close()
    if fill > 1:
        raise SkpError("inverse fill type")
    path.SetFillType(fill)
    return path


class Picture:
    """An SKP file read as Picture::MakeFromStream reads it."""

    def __init__(self, data: bytes):
        if data[:8] != MAGIC:
            raise SkpError("not an SKP file")
        r = _Reader(data, 8)
        self.version = r.u32()
        if not MIN_VERSION <= self.version <= MAX_VERSION:
            raise SkpError(f"SKP version {self.version}")
        self.cull = tuple(float(v) for v in r.f32(4))
        if r.u8() != 1:  # kPictureData_TrailingStreamByteAfterPictInfo
            raise SkpError("no picture data")
        self.ops = b""
        self.paints: list[SkpPaint] = []
        self.paths = []
        self.factories: list[bytes] = []
        while True:
            tag = r.u32()
            if tag == TAG_EOF:
                break
            size = r.u32()
            if tag == TAG_READER:
                if size == 0:
                    raise SkpError("empty op data")
                self.ops = r.raw(size)
            elif tag == TAG_FACTORY:
                for _ in range(r.u32()):
                    self.factories.append(r.raw(r.packed_uint()))
            elif tag == TAG_TYPEFACE:
                if size:
                    raise SkpError("typefaces (text)")
            elif tag == TAG_PICTURE:
                raise SkpError("sub-pictures")
            elif tag == TAG_ARRAY:
                self._read_buffer(_Reader(r.raw(size)))
            else:
                raise SkpError(f"stream tag {tag:#x}")

    def _read_buffer(self, r: _Reader):  # ParseBufferTag (record_playback.cc:728-795)
        while r.o < r.end:
            tag, size = r.u32(), r.u32()
            if tag == TAG_PAINT:
                self.paints += [SkpPaint(r) for _ in range(size)]
            elif tag == TAG_PATH:
                if size > 0:
                    n = r.i32()
                    if n <= 0:
                        raise SkpError("bad path count")
                    self.paths += [_read_path(r) for _ in range(n)]
            elif tag == TAG_READER:
                self.ops = r.raw(size)
            elif size == 0:
                pass  # an empty table of text blobs, slugs, vertices or images
            else:
                raise SkpError(f"buffer tag {tag.to_bytes(4, 'big')!r} (text blobs, images, "
                               "vertices, ...)")

    def width_height(self):
        import math
        return int(math.ceil(self.cull[2])), int(math.ceil(self.cull[3]))

    def play(self, canvas) -> int:
        """Picture::PlayBack (picture.cc:215-247, HandleOp :313-1043) onto a
        canvas with the Canvas API of skity_gb300.canvas; returns the number
        of draws made."""
        r = _Reader(self.ops)
        canvas.Save()
        draws = 0

        def paint():
            i = r.i32()
            if not 0 < i <= len(self.paints):
                raise SkpError("paint index")
            return self.paints[i - 1].to_paint()

        def path():
            i = r.i32()
            if not 0 < i <= len(self.paths):
                raise SkpError("path index")
            return self.paths[i - 1]

        while r.o < r.end:
            start = r.o
            bits = r.u32()
            op, size = bits >> 24, bits & 0xFFFFFF
            if size == 0xFFFFFF:
                size = r.u32()
            if size == 0 or op == 0 or op > 77:
                raise SkpError("bad op record")
            if op in (NOOP,):
                r.o = start + size
            elif op in (FLUSH, PUSH_CULL, POP_CULL):
                pass
            elif op == SAVE:
                canvas.Save()
            elif op == RESTORE:
                canvas.Restore()
            elif op == TRANSLATE:
                dx, dy = r.f32(2)
                canvas.Translate(float(dx), float(dy))
            elif op == SCALE:
                sx, sy = r.f32(2)
                canvas.Scale(float(sx), float(sy))
            elif op == ROTATE:
                canvas.Rotate(float(r.f32()[0]))
            elif op == SKEW:
                sx, sy = r.f32(2)
                canvas.Skew(float(sx), float(sy))
            elif op in (CONCAT, SET_MATRIX):  # a 3x3, the Get9 order (matrix_flat.cc)
                m = [float(v) for v in r.f32(9)]
                (canvas.Concat if op == CONCAT else canvas.SetMatrix)(m)
            elif op in (CONCAT44, SET_M44):  # column-major 4x4
                m = [float(v) for v in r.f32(16)]
                (canvas.Concat44 if op == CONCAT44 else canvas.SetMatrix44)(m)
            elif op in (CLIP_RECT, CLIP_PATH):
                if op == CLIP_RECT:
                    rect = [float(v) for v in r.f32(4)]
                else:
                    cp = path()
                clip_op = 1 if (r.u32() & 0xF) != 0 else 0  # 0: kDifference
                r.i32()  # offset to the restore
                if op == CLIP_RECT:
                    if clip_op == 1:
                        canvas.ClipRect(*rect)
                    else:
                        from .canvas import Path
                        canvas.ClipPath(Path().AddRect(*rect), 0)
                else:
                    canvas.ClipPath(cp, clip_op)
            elif op == DRAW_PATH:
                p = paint()
                canvas.DrawPath(path(), p)
                draws += 1
            elif op == DRAW_RECT:
                p = paint()
                from .canvas import Path
                canvas.DrawPath(Path().AddRect(*(float(v) for v in r.f32(4))), p)
                draws += 1
            elif op == DRAW_CLEAR:
                from .canvas import Color4fFromColor
                canvas.Clear(Color4fFromColor(r.u32()))
            else:
                raise SkpError(f"op {OP_NAMES.get(op, op)}")
            r.o = start + size
        canvas.Restore()
        return draws


def load(data: bytes) -> Picture:
    return Picture(data)


def to_display_list(data: bytes, background=(1.0, 1.0, 1.0, 1.0)):
    """The picture recorded as a display list on a canvas of its cull rect
    (cleared to `background` first, None: not cleared); its to_stream() /
    to_scene() feed the batched and serving forms."""
    from .canvas import PictureRecorder
    pic = Picture(data)
    w, h = pic.width_height()
    rec = PictureRecorder()
    cv = rec.BeginRecording((0, 0, w, h))
    if background is not None:
        cv.Clear(background)
    pic.play(cv)
    return rec.FinishRecording()
