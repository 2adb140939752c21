"""GPU parity: the CUDA path through the C ABI against the oracle.
Bar: <= 1 LSB per channel and >= 99.9% of pixels exact (bit-exact expected)."""
import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999


def check(oracle_lib, got, sc, first=0, count=None):
    ref, _ = oracle_lib.render(sc, first, count)
    c = oracle_lib.compare(got, ref)
    assert c["max_abs_diff"] <= TOL_LSB and c["exact_frac"] >= MIN_EXACT, c
    return c


def test_config1_full(gpu_ctx, oracle_lib):
    sc = S.config1()
    got = gpu_ctx.render_streams([sc])[0]
    c = check(oracle_lib, got, sc)
    assert c["bad_pixels"] == 0


def test_config2_subset(gpu_ctx, oracle_lib):
    sc = S.config2(n_paths=400)
    got = gpu_ctx.render_streams([sc])[0]
    check(oracle_lib, got, sc)


def test_config4_blur_subset(gpu_ctx, oracle_lib):
    sc = S.config4(n_outlines=3000, width=1024, height=1024, blur_frac=0.2)
    got = gpu_ctx.render_streams([sc])[0]
    check(oracle_lib, got, sc)


def test_config3_batch(gpu_ctx, oracle_lib):
    scenes = S.config3(n_canvases=12, scale=0.2)
    outs = gpu_ctx.render_streams(scenes)
    for sc, got in zip(scenes, outs):
        check(oracle_lib, got, sc)


def test_batch_rerender_is_deterministic(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Batch
    scenes = S.config3(n_canvases=4, scale=0.1)
    b = Batch(gpu_ctx, scenes)
    b.render()
    first = [b.read(i) for i in range(len(scenes))]
    b.render()
    for i, sc in enumerate(scenes):
        again = b.read(i)
        assert np.array_equal(first[i], again)
        check(oracle_lib, again, sc)
    b.close()


def test_canvas_api_like_reference_test(gpu_ctx):
    """Restates the exact-pixel check of the reference's
    test/ut/render/sw_canvas_test.cc (StrokeThenFill order) on the CUDA
    canvas: a stroked-then-filled rect leaves white inside the fill and the
    stroke colour on the border."""
    from skity_gb300.canvas import Canvas, Paint, Path, Style, ColorSetARGB
    bitmap = np.zeros((40, 40, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear(ColorSetARGB(0xFF, 0, 0, 0))
    paint = Paint()
    paint.SetStyle(Style.kStrokeThenFill_Style)
    paint.SetStrokeWidth(10)
    paint.SetFillColor(1, 1, 1, 1)
    paint.SetStrokeColor(1, 0, 0, 1)
    canvas.DrawPath(Path().AddRect(10, 10, 30, 30), paint)
    canvas.Flush()
    assert tuple(bitmap[20, 12]) == (255, 255, 255, 255)  # fill drawn over the stroke
    assert tuple(bitmap[20, 7]) == (255, 0, 0, 255)       # stroke outside the rect


def test_canvas_matches_stream_and_oracle(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Canvas, Paint, Path, Shader, PathFillType, TileMode, MaskFilter, BlurStyle
    sb = S.SceneBuilder(120, 90)
    bitmap = np.zeros((90, 120, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    rng = np.random.default_rng(3)
    for i in range(30):
        path = Path().MoveTo(*rng.uniform(-10, 130, 2))
        for _ in range(5):
            path.CubicTo(*rng.uniform(-10, 130, 6))
        path.Close().SetFillType(PathFillType.kEvenOdd if i % 3 == 0 else PathFillType.kWinding)
        paint = Paint().SetColor(0xFF000000 | int(rng.integers(0, 1 << 24))).SetAlphaF(0.6)
        if i % 4 == 1:
            paint.SetStyle(1).SetStrokeWidth(3).SetStrokeCap(i % 3).SetStrokeJoin(i % 3)
        if i % 5 == 2:
            paint.SetShader(Shader.MakeLinear([(0, 0), (120, 90)], [[1, 0, 0, 1], [0, 0, 1, 0.5]], None, 2))
        if i % 7 == 3:
            paint.SetMaskFilter(MaskFilter.MakeBlur(BlurStyle.kNormal, 4.0))
        canvas.DrawPath(path, paint)
        g = -1
        if paint.shader is not None:
            s = paint.shader
            g = sb.add_gradient(s.kind, s.p0, s.p1, s.radius, s.colors, None, TileMode.kClamp)
        rec = paint.rec.copy(); rec["fill_type"] = path.fill_type; rec["gradient"] = g
        if paint.mask_filter is not None:
            rec["blur_style"] = paint.mask_filter.style
            rec["blur_radius"] = paint.mask_filter.radius
        sb.draw_path(path.verbs, path.points, rec)
    canvas.Flush()
    check(oracle_lib, bitmap, sb.build())


def test_flush_then_draw_blends_over_previous_pixels(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Canvas, Paint, Path
    bitmap = np.zeros((32, 32, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((0.0, 0.5, 1.0, 1.0))
    canvas.DrawPath(Path().MoveTo(2, 2).LineTo(30, 5).LineTo(8, 29).Close(),
                    Paint().SetFillColor(1, 0, 0, 0.5))
    canvas.Flush()
    canvas.DrawPath(Path().MoveTo(30, 2).LineTo(1, 16).LineTo(30, 30).Close(),
                    Paint().SetFillColor(0, 1, 0, 0.7))
    canvas.Flush()
    sb = S.SceneBuilder(32, 32, clear=(0.0, 0.5, 1.0, 1.0))
    p = S.default_paint(); p["fill_color"] = (1, 0, 0, 0.5)
    sb.draw_path([0, 1, 1, 5], [(2, 2), (30, 5), (8, 29)], p)
    p2 = S.default_paint(); p2["fill_color"] = (0, 1, 0, 0.7)
    sb.draw_path([0, 1, 1, 5], [(30, 2), (1, 16), (30, 30)], p2)
    check(oracle_lib, bitmap, sb.build())


def test_invalid_arguments_are_rejected(gpu_ctx):
    import ctypes
    from skity_gb300 import _lib
    from skity_gb300.canvas import Canvas
    assert Canvas.MakeCUDACanvas(gpu_ctx, None) is None
    assert Canvas.MakeCUDACanvas(gpu_ctx, np.zeros((0, 0, 4), np.uint8)) is None
    lib = gpu_ctx.lib
    assert lib.skity_cuda_canvas_flush(None) == -1
    bad = b"NOPE" + b"\0" * 100
    ptrs = (ctypes.c_void_p * 1)(ctypes.cast(ctypes.c_char_p(bad), ctypes.c_void_p))
    lens = (ctypes.c_size_t * 1)(len(bad))
    out = np.zeros(16, np.uint8)
    optr = (ctypes.c_void_p * 1)(out.ctypes.data)
    assert lib.skity_cuda_render_streams(gpu_ctx.handle, 1, ptrs, lens, optr) == -2
    bitmap = np.zeros((8, 8, 4), np.uint8)
    c = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    verbs = (ctypes.c_uint8 * 2)(0, 9)   # unknown verb
    pts = (ctypes.c_float * 2)(1, 1)
    cp = _lib.Path_(ctypes.cast(verbs, ctypes.c_void_p), 2, ctypes.cast(pts, ctypes.c_void_p), 1, None, 0, 0)
    paint = _lib.Paint_()
    assert lib.skity_cuda_canvas_draw_path(c.handle, ctypes.byref(cp), ctypes.byref(paint)) == -2


def test_canvas_translate_matches_oracle(gpu_ctx, oracle_lib):
    """Canvas::Save / Translate / Restore: the translated scene rendered
    as a batch and through the canvas API against the oracle (pinned to the
    reference's Canvas::Translate)."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import translated_scene
    from skity_gb300.canvas import Canvas, Paint, Path
    sc = translated_scene()
    check(oracle_lib, gpu_ctx.render_streams([sc])[0], sc)
    bitmap = np.zeros((40, 48, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    tri = Path().MoveTo(2, 2).LineTo(20, 5).LineTo(6, 19).Close()
    paint = Paint().SetFillColor(0.2, 0.3, 0.9, 0.8)
    canvas.DrawPath(tri, paint)
    canvas.Save()
    canvas.Translate(10.5, 3)
    canvas.Translate(4, 7.25)
    canvas.DrawPath(tri, paint)
    canvas.Restore()
    canvas.DrawPath(tri, Paint().SetFillColor(0.9, 0.1, 0.1, 0.5))
    canvas.Flush()
    sb = S.SceneBuilder(48, 40)
    for tr, col in [((0, 0), (0.2, 0.3, 0.9, 0.8)), ((14.5, 10.25), (0.2, 0.3, 0.9, 0.8)),
                    ((0, 0), (0.9, 0.1, 0.1, 0.5))]:
        p = S.default_paint()
        p["fill_color"] = col
        p["translate"] = tr
        sb.draw_path(tri.verbs, tri.points, p)
    check(oracle_lib, bitmap, sb.build())


@pytest.mark.gpu
def test_clip_rect_matches_oracle(gpu_ctx, oracle_lib):
    """Canvas::ClipRect (kIntersect) under Save / Translate / Restore: the
    clipped scenes rendered as a batch, and a draw sequence through the
    canvas API, against the oracle (pinned to the reference's ClipRect)."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import clipped_scene
    from skity_gb300.canvas import Canvas, Paint, Path
    scenes = [clipped_scene(S.SEED_BASE + 380 + k) for k in range(3)]
    for sc, got in zip(scenes, gpu_ctx.render_streams(scenes)):
        check(oracle_lib, got, sc)
    bitmap = np.zeros((40, 48, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    tri = Path().MoveTo(1, 1).LineTo(30, 4).LineTo(5, 33).Close()
    blue = Paint().SetFillColor(0.2, 0.3, 0.9, 0.8)
    red = Paint().SetFillColor(0.9, 0.1, 0.1, 0.5)
    canvas.Save()
    canvas.ClipRect(3.5, 2.25, 21, 18.75)
    canvas.DrawPath(tri, blue)
    canvas.Save()
    canvas.Translate(10.5, 3)
    canvas.ClipRect(-2, 0, 12, 40)  # device (8.5, 3, 22.5, 43): narrows the clip to x >= 8.5
    canvas.DrawPath(tri, red)
    canvas.Restore()
    canvas.DrawPath(tri, red)  # the first clip again
    canvas.Restore()
    canvas.Save()
    canvas.ClipRect(40, 0, 44, 5)
    canvas.ClipRect(0, 30, 5, 40)  # disjoint: empty clip, nothing drawn
    canvas.DrawPath(tri, blue)
    canvas.Restore()
    canvas.DrawPath(tri, Paint().SetFillColor(0.1, 0.8, 0.2, 0.4))  # unclipped
    canvas.Flush()
    c1 = S.map_clip(S.NO_CLIP, (3.5, 2.25, 21, 18.75))
    c2 = S.map_clip(c1, (-2, 0, 12, 40), 10.5, 3)
    c3 = S.map_clip(S.map_clip(S.NO_CLIP, (40, 0, 44, 5)), (0, 30, 5, 40))
    assert c3 == (0.0, 0.0, 0.0, 0.0)
    sb = S.SceneBuilder(48, 40)
    for tr, col, clip in [((0, 0), (0.2, 0.3, 0.9, 0.8), c1), ((10.5, 3), (0.9, 0.1, 0.1, 0.5), c2),
                          ((0, 0), (0.9, 0.1, 0.1, 0.5), c1), ((0, 0), (0.2, 0.3, 0.9, 0.8), c3),
                          ((0, 0), (0.1, 0.8, 0.2, 0.4), None)]:
        p = S.default_paint()
        p["fill_color"] = col
        p["translate"] = tr
        sb.draw_path(tri.verbs, tri.points, p, clip=clip)
    check(oracle_lib, bitmap, sb.build())


@pytest.mark.gpu
def test_every_blend_mode_matches_oracle(gpu_ctx, oracle_lib):
    """kClear .. kLuminosity (PorterDuffBlend with FastBlend, SoftLight in
    float, the rest as kSrcOver) over translucent and transparent pixels."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import blend_modes_scene
    sc = blend_modes_scene()
    check(oracle_lib, gpu_ctx.render_streams([sc])[0], sc)


@pytest.mark.gpu
def test_sweep_and_conical_gradients_match_oracle(gpu_ctx, oracle_lib):
    """Shader::MakeSweep and MakeTwoPointConical through the batch entry point
    and through the canvas API.  Bar as above; the sweep angle is the double
    atan2 rounded to float, the float atan2 of the reference in all but
    near-tie cases, so the run also records how many pixels are exact."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import sweep_conical_scene
    from skity_gb300.canvas import Canvas, Paint, Path, Shader
    sc = sweep_conical_scene()
    c = check(oracle_lib, gpu_ctx.render_streams([sc])[0], sc)
    print("sweep/conical parity", c)
    bitmap = np.zeros((60, 80, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    rect = Path().MoveTo(2, 2).LineTo(78, 3).LineTo(76, 58).LineTo(4, 55).Close()
    cols = np.array([[1, 0, 0, 1], [0, 1, 0, 0.6], [0, 0, 1, 1]], np.float32)
    shaders = [Shader.MakeSweep(40, 30, -30, 250, cols, None, 3),
               Shader.MakeTwoPointConical((20, 20), 5.0, (50, 35), 30.0, cols, [0, 0.3, 1], 3, 2)]
    sb = S.SceneBuilder(80, 60)
    for sh in shaders:
        paint = Paint().SetFillColor(0, 0, 0, 1)
        paint.shader = sh
        canvas.DrawPath(rect, paint)
        p = S.default_paint()
        p["gradient"] = sb.add_gradient(sh.kind, sh.p0, sh.p1, sh.radius, sh.colors, sh.pos,
                                        tile_mode=sh.tile)
        sb.draw_path(rect.verbs, rect.points, p)
    canvas.Flush()
    check(oracle_lib, bitmap, sb.build())


@pytest.mark.gpu
def test_blur_styles_match_oracle(gpu_ctx, oracle_lib):
    """MaskFilter::MakeBlur with kNormal, kSolid, kOuter and kInner."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import blur_styles_scene
    sc = blur_styles_scene()
    c = check(oracle_lib, gpu_ctx.render_streams([sc])[0], sc)
    assert c["bad_pixels"] == 0


@pytest.mark.gpu
def test_color_filters_match_oracle(gpu_ctx, oracle_lib):
    """ColorFilters::Blend / Matrix / LinearToSRGBGamma / SRGBToLinearGamma /
    Compose through the batch entry point and the canvas API."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import color_filters_scene
    from skity_gb300.canvas import BlendMode, Canvas, ColorFilters, Paint, Path
    sc = color_filters_scene()
    c = check(oracle_lib, gpu_ctx.render_streams([sc])[0], sc)
    assert c["bad_pixels"] == 0
    bitmap = np.zeros((40, 48, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    tri = Path().MoveTo(2, 2).LineTo(44, 5).LineTo(6, 37).Close()
    filters = [ColorFilters.Blend(0x80FF2040, BlendMode.kScreen),
               ColorFilters.Matrix([0, 1, 0, 0, 0.1, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0.5, 0]),
               ColorFilters.SRGBToLinearGamma()]
    sb = S.SceneBuilder(48, 40)
    for k, f in enumerate(filters):
        paint = Paint().SetFillColor(0.3 + 0.2 * k, 0.6, 0.2, 0.7).SetColorFilter(f)
        canvas.DrawPath(tri, paint)
        sb.draw_path(tri.verbs, tri.points, paint.rec.copy(), color_filter=f.record())
    canvas.Flush()
    check(oracle_lib, bitmap, sb.build())


@pytest.mark.gpu
def test_clip_path_matches_oracle(gpu_ctx, oracle_lib):
    """Canvas::ClipPath (intersect and difference, nested under Save /
    Restore, with ClipRect and Translate) through the batch entry point, and
    through the canvas API with a Clear under a path clip."""
    import sys, os
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from test_oracle_pin import clip_path_cases_scene, path_clips_scene
    from skity_gb300.canvas import Canvas, Paint, Path
    scenes = [path_clips_scene(S.SEED_BASE + 399 + k) for k in range(4)] + [clip_path_cases_scene()]
    for sc, got in zip(scenes, gpu_ctx.render_streams(scenes)):
        c = check(oracle_lib, got, sc)
        assert c["bad_pixels"] == 0, c
    bitmap = np.zeros((40, 48, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    tri = Path().MoveTo(2, 2).LineTo(46, 6).LineTo(8, 38).Close()
    band = Path().MoveTo(0, 12).LineTo(48, 12).LineTo(48, 24).LineTo(0, 24).Close()
    canvas.Save()
    canvas.ClipPath(tri, 1)
    canvas.Clear((0.2, 0.4, 0.9, 1.0))  # DrawPaint under the clip
    canvas.Save()
    canvas.Translate(1.5, 0.5)
    canvas.ClipPath(band, 0)
    canvas.DrawPath(Path().MoveTo(0, 0).LineTo(48, 0).LineTo(48, 40).LineTo(0, 40).Close(),
                    Paint().SetFillColor(0.9, 0.2, 0.1, 0.7))
    canvas.Restore()
    canvas.Restore()
    canvas.DrawPath(band, Paint().SetFillColor(0.1, 0.8, 0.2, 0.5))
    canvas.Flush()
    sb = S.SceneBuilder(48, 40)
    sb.save()
    sb.clip_path(tri.verbs, tri.points, S.CLIP_INTERSECT)
    glob = S.map_clip(S.NO_CLIP, (2, 2, 46, 38))
    p = S.default_paint()
    p["blend"], p["fill_color"] = S.BLEND_SRC, (0.2, 0.4, 0.9, 1.0)
    sb.draw_path([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE], [[0, 0], [48, 0], [48, 40], [0, 40]], p)
    sb.save()
    sb.clip_path(band.verbs, band.points, S.CLIP_DIFFERENCE, translate=(1.5, 0.5), bounds=glob)
    q = S.default_paint()
    q["fill_color"], q["translate"] = (0.9, 0.2, 0.1, 0.7), (1.5, 0.5)
    sb.draw_path([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE], [[0, 0], [48, 0], [48, 40], [0, 40]], q,
                 clip=glob)
    sb.restore()
    sb.restore()
    r = S.default_paint()
    r["fill_color"] = (0.1, 0.8, 0.2, 0.5)
    sb.draw_path(band.verbs, band.points, r)
    check(oracle_lib, bitmap, sb.build())
