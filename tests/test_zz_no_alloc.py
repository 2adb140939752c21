"""skity_cuda_draw_path_static -- the entry point that draws without
allocating -- against skity_cuda_render_streams on the same draws, and
against the oracle.

Each static call draws one path onto a canvas held in a device tensor; after
every call the canvas must match render_streams of the draws so far (bar:
<= 1 LSB per channel and >= 99.9% exact pixels; bit-exact expected, the
passes run the same kernels).  The file sorts last, so the test runs both
alone in a fresh process and after every other GPU test.
"""
import ctypes

import numpy as np
import pytest

from skity_gb300 import _lib
from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999
SCRATCH_LIMIT = -9


# BlendMode values (include/skity/graphic/blend_mode.hpp): the Porter-Duff
# general path (kDstIn, kXor), a separable mode (kMultiply) and SoftLight
RARE_BLENDS = (6, 11, 24, 21)


def _scene():
    """Solid-colour paths over and around a 384x320 canvas: 30% even-odd, 40%
    stroked; some strokes turned into stroke-and-fill / stroke-then-fill, a
    few draws using kSrc and a few the rarer blend modes, so every pass kind
    and blend path is exercised."""
    sc = S.random_paths_scene(S.SEED_BASE + 77, 384, 320, 24, 3, 20,
                              coord_lo=(-32.0, -32.0), coord_hi=(416.0, 352.0),
                              evenodd_frac=0.3, stroke_frac=0.4)
    for d in range(sc.n_draws):
        p = sc.paints[d]
        if p["style"] == S.STROKE and d % 3 == 1:
            p["style"] = S.STROKE_AND_FILL
        elif p["style"] == S.STROKE and d % 3 == 2:
            p["style"] = S.STROKE_THEN_FILL
        if d % 7 == 5:
            p["blend"] = S.BLEND_SRC
        elif d % 5 == 3:
            p["blend"] = RARE_BLENDS[(d // 5) % len(RARE_BLENDS)]
    return sc


def _static_draw(lib, canvas, sc, d, stream):
    v0, v1 = int(sc.verb_off[d]), int(sc.verb_off[d + 1])
    p0, p1 = int(sc.point_off[d]), int(sc.point_off[d + 1])
    w0, w1 = int(sc.weight_off[d]), int(sc.weight_off[d + 1])
    verbs = np.ascontiguousarray(sc.verbs[v0:v1], np.uint8)
    pts = np.ascontiguousarray(sc.points[p0:p1], np.float32)
    wts = np.ascontiguousarray(sc.weights[w0:w1], np.float32)
    r = sc.paints[d]
    path = _lib.Path_(verbs.ctypes.data if len(verbs) else None, len(verbs),
                      pts.ctypes.data if len(pts) else None, len(pts),
                      wts.ctypes.data if len(wts) else None, len(wts), int(r["fill_type"]))
    paint = _paint(r)
    h, w = canvas.shape[0], canvas.shape[1]
    return lib.skity_cuda_draw_path_static(canvas.device.index or 0, canvas.data_ptr(), w, h,
                                           canvas.stride(0), ctypes.byref(path),
                                           ctypes.byref(paint), stream)


def _paint(r):
    p = _lib.Paint_()
    p.style, p.cap, p.join, p.blend_mode = (int(r["style"]), int(r["cap"]), int(r["join"]),
                                            int(r["blend"]))
    p.fill_color[:] = [float(v) for v in r["fill_color"]]
    p.stroke_color[:] = [float(v) for v in r["stroke_color"]]
    p.stroke_width = float(r["stroke_width"])
    p.miter_limit = float(r["miter"])
    return p


def _white_canvas(torch, h, w):
    # Clear(white) leaves premultiplied (255, 255, 255, 255) everywhere
    return torch.full((h, w, 4), 255, dtype=torch.uint8, device="cuda:0")


def _check(got, want):
    diff = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    exact = float((diff == 0).mean())
    assert int(diff.max()) <= TOL_LSB and exact >= MIN_EXACT, (int(diff.max()), exact)
    return exact


def test_static_draw_matches_render_streams(gpu_ctx):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    sc = _scene()
    canvas = _white_canvas(torch, sc.height, sc.width)
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row, each checked against the existing entry point
    for d in (0, 1):
        assert _static_draw(lib, canvas, sc, d, stream) == 0
        torch.cuda.synchronize()
        want = gpu_ctx.render_streams([sc.subset(0, d + 1)])[0]
        _check(canvas.cpu().numpy(), want)
    # the rest of the scene, checked once at the end
    for d in range(2, sc.n_draws):
        assert _static_draw(lib, canvas, sc, d, stream) == 0
    torch.cuda.synchronize()
    got = canvas.cpu().numpy()
    want = gpu_ctx.render_streams([sc])[0]
    assert _check(got, want) == 1.0
    # and against the oracle (the CPU restatement of the reference path)
    from oracle import oracle
    ref, _ = oracle.render(sc)
    _check(got, ref)


def test_static_draw_stroke_and_fill_is_all_or_nothing(gpu_ctx):
    """A stroke-and-fill draw whose fill fits the scratch but whose stroke
    does not: the call fails with the scratch limit and the canvas keeps
    every pixel it had (the fill pass is not blended on its own)."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    canvas = _white_canvas(torch, 64, 64)
    stream = torch.cuda.current_stream().cuda_stream
    # a zig-zag of 20k lines: its fill's edges fit, the stroke's outline
    # (several times the path) does not
    n = 20_000
    verbs = np.full(n, S.LINE, np.uint8)
    verbs[0] = S.MOVE
    pts = np.zeros((n, 2), np.float32)
    pts[:, 0] = (np.arange(n) % 2) * 60 + 2
    pts[:, 1] = np.linspace(2, 62, n, dtype=np.float32)
    path = _lib.Path_(verbs.ctypes.data, n, pts.ctypes.data, n, None, 0, 0)
    r = S.default_paint()
    r["fill_color"] = (0.2, 0.4, 0.6, 1.0)
    r["stroke_color"] = (0.9, 0.1, 0.1, 1.0)
    r["stroke_width"] = 3.0
    fill_only = _paint(r)
    assert lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 256, ctypes.byref(path),
                                           ctypes.byref(fill_only), stream) == 0
    torch.cuda.synchronize()
    assert not bool((canvas == 255).all())  # the fill alone fits and draws
    canvas.fill_(255)
    r["style"] = S.STROKE_AND_FILL
    both = _paint(r)
    rc = lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 256, ctypes.byref(path),
                                         ctypes.byref(both), stream)
    torch.cuda.synchronize()
    assert rc == SCRATCH_LIMIT
    assert bool((canvas == 255).all())


def test_static_draw_rejects_oversized_inputs(gpu_ctx):
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    canvas = _white_canvas(torch, 64, 64)
    stream = torch.cuda.current_stream().cuda_stream
    paint = _paint(S.default_paint())
    # path copy alone beyond the static scratch (2.5M points = 20 MB)
    n = 2_500_000
    verbs = np.full(n, S.LINE, np.uint8)
    verbs[0] = S.MOVE
    pts = np.zeros((n, 2), np.float32)
    pts[:, 0] = np.arange(n, dtype=np.float32) % 64
    path = _lib.Path_(verbs.ctypes.data, n, pts.ctypes.data, n, None, 0, 0)
    rc = lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 256, ctypes.byref(path),
                                         ctypes.byref(paint), stream)
    assert rc == SCRATCH_LIMIT
    # path copy fits, its edge buffers do not (400k lines)
    n = 400_000
    path = _lib.Path_(verbs.ctypes.data, n, pts.ctypes.data, n, None, 0, 0)
    rc = lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 256, ctypes.byref(path),
                                         ctypes.byref(paint), stream)
    assert rc == SCRATCH_LIMIT
    torch.cuda.synchronize()
    assert bool((canvas == 255).all())
    # unsupported / invalid arguments
    grad = _lib.Gradient_()
    paint.shader = ctypes.pointer(grad)
    small = _lib.Path_(verbs.ctypes.data, 2, pts.ctypes.data, 2, None, 0, 0)
    assert lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 256, ctypes.byref(small),
                                           ctypes.byref(paint), stream) == -5
    paint.shader = None
    assert lib.skity_cuda_draw_path_static(0, None, 64, 64, 256, ctypes.byref(small),
                                           ctypes.byref(paint), stream) == -2
    assert lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 100, ctypes.byref(small),
                                           ctypes.byref(paint), stream) == -2
    paint.blend_mode = 29  # past kLuminosity
    assert lib.skity_cuda_draw_path_static(0, canvas.data_ptr(), 64, 64, 256, ctypes.byref(small),
                                           ctypes.byref(paint), stream) == -2
