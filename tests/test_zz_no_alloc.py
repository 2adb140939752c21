"""skity_cuda_draw_path_static -- the entry point that draws without
allocating -- against skity_cuda_render_streams on the same draws.

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


def _scene():
    """Solid-colour paths over and around a 384x320 canvas: 30% even-odd, 40%
    stroked; some strokes turned into stroke-and-fill / stroke-then-fill and
    a few draws using kSrc, so every pass kind and blend path is exercised."""
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
    want = gpu_ctx.render_streams([sc])[0]
    assert _check(canvas.cpu().numpy(), want) == 1.0


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
