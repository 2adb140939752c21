"""Canvas matrices on the GPU (Canvas::Scale / Rotate / Skew / Concat /
SetMatrix; RastePath's CopyWithMatrix and GenerateBrush's inverse) through
the C ABI against the oracle, pinned to the reference's software canvas.
Bit-exact expected (tolerance: <= 1 LSB per channel, >= 99.9% exact)."""
import os
import sys

import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def check(oracle_lib, got, sc):
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["max_abs_diff"] <= TOL_LSB and c["exact_frac"] >= MIN_EXACT, c
    return c


def test_matrix_scenes_match_oracle(gpu_ctx, oracle_lib):
    """Fills and strokes under scales, flips, rotations, skews and general
    affine maps; gradients under scale and translation; one batch."""
    from test_oracle_pin import matrix_scene
    scenes = [matrix_scene(S.SEED_BASE + 365 + k) for k in range(4)]
    scenes.append(matrix_scene(S.SEED_BASE + 369, 640, 480))
    for got, sc in zip(gpu_ctx.render_streams(scenes), scenes):
        assert check(oracle_lib, got, sc)["bad_pixels"] == 0


def _shapes():
    from skity_gb300.canvas import Path
    tri = Path().MoveTo(2, 2).LineTo(30, 6).LineTo(8, 28).Close()
    blob = (Path().MoveTo(5, 5).QuadTo(40, 0, 35, 20).CubicTo(30, 40, 10, 45, 3, 30)
            .ConicTo(0, 20, 5, 5, 0.7).Close())
    return tri, blob


def test_canvas_transforms_match_oracle(gpu_ctx, oracle_lib):
    """The canvas API: Translate, Scale, Rotate (about a point), Skew and
    Concat between Save / Restore; each draw's matrix (GetTotalMatrix, the
    reference Canvas's own product, pinned on the CPU) replayed by the
    oracle."""
    from skity_gb300.canvas import Canvas, Paint, Shader
    tri, blob = _shapes()
    W, H = 96, 80
    bitmap = np.zeros((H, W, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    sb = S.SceneBuilder(W, H)
    colors = [(1, 0, 0, 1), (0, 0.5, 1, 1), (0.2, 0.9, 0.1, 0.8)]

    def draw(path, paint, shader=None):
        canvas.DrawPath(path, paint)
        m9 = canvas.GetTotalMatrix()
        p = paint.rec.copy()
        if shader is not None:
            p["gradient"] = sb.add_gradient(shader.kind, shader.p0, shader.p1, shader.radius,
                                            shader.colors, shader.pos, shader.tile)
        sb.draw_path(path.verbs, path.points, p, path.weights,
                     matrix=(m9[0], m9[1], m9[2], m9[3], m9[4], m9[5]))

    red = Paint().SetFillColor(0.9, 0.1, 0.1, 0.8)
    blue = Paint().SetFillColor(0.1, 0.2, 0.9, 0.6)
    stroke = Paint().SetStyle(1).SetStrokeWidth(2.5).SetStrokeJoin(1).SetFillColor(0, 0, 0, 1)
    stroke.SetStrokeColor(0.1, 0.6, 0.2, 0.9)
    draw(tri, red)
    canvas.Save()
    canvas.Translate(20, 10)
    canvas.Scale(1.5, 0.75)
    grad = Shader.MakeLinear([(0, 0), (30, 20)], colors, None, 3)
    draw(blob, Paint().SetShader(grad).SetFillColor(0, 0, 0, 1), grad)
    canvas.Rotate(25, 10, 10)
    draw(blob, blue)
    draw(tri, stroke)
    canvas.Skew(0.3, -0.1)
    draw(tri, red)
    canvas.Restore()
    canvas.Save()
    canvas.Concat((0.8, -0.4, 50, 0.3, 1.1, 20, 0, 0, 1))
    draw(blob, stroke)
    canvas.Rotate(-60)
    draw(tri, blue)
    canvas.Restore()
    draw(tri, blue)
    canvas.Flush()
    check(oracle_lib, bitmap, sb.build())


def test_canvas_transform_limits(gpu_ctx):
    """A gradient or a blur under a rotation, and draws under perspective,
    return NOT_SUPPORTED and draw nothing."""
    from skity_gb300 import _lib
    from skity_gb300.canvas import Canvas, MaskFilter, Paint, Shader
    tri, _ = _shapes()
    bitmap = np.full((40, 48, 4), 7, np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    grad = Shader.MakeLinear([(0, 0), (30, 20)], [(1, 0, 0, 1), (0, 0, 1, 1)], None, 2)
    canvas.Rotate(30)
    with pytest.raises(_lib.SkityCudaError) as e:
        canvas.DrawPath(tri, Paint().SetShader(grad))
    assert e.value.code == -5  # SKITY_CUDA_ERROR_NOT_SUPPORTED
    with pytest.raises(_lib.SkityCudaError) as e:
        canvas.DrawPath(tri, Paint().SetMaskFilter(MaskFilter.MakeBlur(1, 3.0)))
    assert e.value.code == -5
    canvas.SetMatrix((1, 0, 0, 0, 1, 0, 0.01, 0, 1))
    with pytest.raises(_lib.SkityCudaError):
        canvas.DrawPath(tri, Paint())
    canvas.Flush()
    assert (bitmap == 7).all()


def test_clips_and_blurs_under_matrices(gpu_ctx, oracle_lib):
    """ClipPath and rotated ClipRect under canvas matrices, rotated draws
    under path clips, blurs under scales, clip rects and path clips; one
    batch."""
    from test_oracle_pin import matrix_clips_scene
    scenes = [matrix_clips_scene(S.SEED_BASE + 470 + k) for k in range(6)]
    scenes.append(matrix_clips_scene(S.SEED_BASE + 476, 512, 384, 120))
    for got, sc in zip(gpu_ctx.render_streams(scenes), scenes):
        assert check(oracle_lib, got, sc)["bad_pixels"] == 0


def test_canvas_clips_under_matrices(gpu_ctx, oracle_lib):
    """The canvas API: ClipRect under a rotation (a rect path clip),
    ClipPath under a scale and a skew, a blur under a scale, a clip rect and
    a path clip; the expected scene built with the reference's rules
    (global clip bounds by the mapped bounds, Path::AddRect) and rendered by
    the oracle."""
    from skity_gb300.canvas import Canvas, MaskFilter, Paint
    tri, blob = _shapes()
    W, H = 120, 96
    bitmap = np.zeros((H, W, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    sb = S.SceneBuilder(W, H)
    state = {"glob": S.NO_CLIP, "stack": []}

    def m6():
        m9 = canvas.GetTotalMatrix()
        return (m9[0], m9[1], m9[2], m9[3], m9[4], m9[5])

    def draw(path, paint):
        canvas.DrawPath(path, paint)
        p = paint.rec.copy()
        if paint.mask_filter is not None:
            p["blur_style"], p["blur_radius"] = paint.mask_filter.style, paint.mask_filter.radius
        sb.draw_path(path.verbs, path.points, p, path.weights, clip=state["glob"], matrix=m6())

    def save():
        canvas.Save()
        sb.save()
        state["stack"].append(state["glob"])

    def restore():
        canvas.Restore()
        sb.restore()
        state["glob"] = state["stack"].pop()

    def clip_rect(rect):
        canvas.ClipRect(*rect)
        m = m6()
        state["glob"] = S.map_clip_matrix(state["glob"], rect, m)
        if m[1] != 0.0 or m[3] != 0.0:
            sb.clip_path(S.RECT_VERBS, S.rect_points(rect), S.CLIP_INTERSECT, S.WINDING,
                         bounds=state["glob"], matrix=m)

    def clip_path(path, op):
        canvas.ClipPath(path, op)
        m = m6()
        pts = np.asarray(path.points, np.float32).reshape(-1, 2)
        if op == S.CLIP_INTERSECT:
            pb = (pts[:, 0].min(), pts[:, 1].min(), pts[:, 0].max(), pts[:, 1].max())
            state["glob"] = S.map_clip_matrix(state["glob"], pb, m)
        sb.clip_path(path.verbs, pts, op, path.fill_type, path.weights, bounds=state["glob"],
                     matrix=m)

    red = Paint().SetFillColor(0.9, 0.1, 0.1, 0.8)
    blue = Paint().SetFillColor(0.1, 0.2, 0.9, 0.6)
    stroke = Paint().SetStyle(1).SetStrokeWidth(3.0).SetFillColor(0, 0, 0, 1)
    stroke.SetStrokeColor(0.1, 0.6, 0.2, 0.9)
    blur = Paint().SetFillColor(0.2, 0.2, 0.7, 0.9).SetMaskFilter(MaskFilter.MakeBlur(1, 4.0))
    save()
    canvas.Rotate(20, 60, 48)
    clip_rect((20.0, 15.0, 100.0, 80.0))
    canvas.Translate(30, 20)
    draw(blob, red)
    canvas.Skew(0.25, 0.0)
    draw(tri, stroke)
    restore()
    save()
    canvas.Scale(2.0, 1.5)
    clip_path(blob, S.CLIP_INTERSECT)
    draw(tri, blue)
    canvas.Translate(3, 4)
    draw(blob, blur)
    canvas.Skew(0.3, -0.2)
    clip_path(tri, S.CLIP_DIFFERENCE)
    draw(blob, stroke)
    restore()
    clip_rect((5.0, 5.0, 70.0, 60.0))
    canvas.Scale(1.25, 1.25)
    draw(blob, Paint().SetFillColor(0.8, 0.5, 0.1, 0.9).SetMaskFilter(MaskFilter.MakeBlur(3, 2.5)))
    canvas.Flush()
    sc = sb.build()
    assert sc.clip_matrices is not None
    check(oracle_lib, bitmap, sc)


def test_canvas_shapes_match_oracle(gpu_ctx, oracle_lib):
    """Canvas::DrawOval / DrawCircle / DrawRect on the CUDA canvas (fills and
    strokes, under a scale and a rotation) against the oracle rendering the
    same paths (the reference's RRect and rect paths, tests/test_shapes.py)."""
    from skity_gb300.canvas import Canvas, Paint, Path
    W, H = 128, 96
    bitmap = np.zeros((H, W, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    sb = S.SceneBuilder(W, H)

    def m6():
        m9 = canvas.GetTotalMatrix()
        return (m9[0], m9[1], m9[2], m9[3], m9[4], m9[5])

    fill = Paint().SetFillColor(0.8, 0.2, 0.3, 0.8)
    stroke = Paint().SetStyle(1).SetStrokeWidth(2.5).SetFillColor(0, 0, 0, 1)
    stroke.SetStrokeColor(0.1, 0.4, 0.9, 0.9)
    calls = [("oval", (8.0, 6.0, 60.5, 40.0), fill), ("circle", (90.0, 30.0, 18.25), stroke),
             ("rect", (10.0, 50.0, 50.0, 90.0), fill), ("circle", (70.0, 70.0, 0.0), stroke)]
    for k, (kind, a, paint) in enumerate(calls):
        if k == 2:
            canvas.Scale(1.2, 0.9)
        if k == 3:
            canvas.Rotate(15, 64, 48)
        if kind == "oval":
            canvas.DrawOval(*a, paint)
            path = Path().AddOvalRRect(*a)
        elif kind == "circle":
            canvas.DrawCircle(*a, paint)
            cx, cy, r = (np.float32(v) for v in a)
            path = Path().AddOvalRRect(cx - r, cy - r, cx + r, cy + r)
        else:
            canvas.DrawRect(*a, paint)
            path = Path().AddRect(*a)
        sb.draw_path(path.verbs, path.points, paint.rec, path.weights, matrix=m6())
    canvas.Flush()
    check(oracle_lib, bitmap, sb.build())
