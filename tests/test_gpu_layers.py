"""Canvas::SaveLayer / Restore on the GPU against the oracle (itself pinned
to the reference's software backend on the same scenes): layer temp canvases
and their restore image passes.  Bar: <= 1 LSB per channel and >= 99.9% of
pixels exact (bit-exact expected)."""
import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999


def _check(oracle_lib, got, sc):
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["max_abs_diff"] <= TOL_LSB and c["exact_frac"] >= MIN_EXACT, c
    return c


def test_layered_scenes_match_oracle(gpu_ctx, oracle_lib):
    scenes = [S.layered_scene(S.SEED_BASE + 700 + seed, 120 + 8 * seed, 96 + 4 * seed, 30, 3,
                              blends=(3, 1, 24, 6, 11, 21)) for seed in range(8)]
    scenes.append(S.layered_scene(S.SEED_BASE + 799, 640, 480, 400, 6))
    for sc, got in zip(scenes, gpu_ctx.render_streams(scenes)):
        assert _check(oracle_lib, got, sc)["bad_pixels"] == 0


def test_canvas_save_layer_like_reference(gpu_ctx, oracle_lib):
    """The C ABI canvas: a half-transparent layer under a translation and a
    clip, draws inside and after it, against the same calls recorded as a
    scene for the oracle."""
    from skity_gb300.canvas import Canvas, Paint, Path
    w, h = 160, 120
    bitmap = np.zeros((h, w, 4), np.uint8)
    cv = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    cv.Clear((1.0, 1.0, 1.0, 1.0))
    b = S.SceneBuilder(w, h)
    tri = ([S.MOVE, S.LINE, S.LINE, S.CLOSE], [(10, 10), (150, 30), (40, 110)])
    quad = ([S.MOVE, S.QUAD, S.LINE, S.CLOSE], [(0, 60), (80, -20), (160, 60), (80, 118)])
    red, blue = Paint().SetColor(0xFFCC2020), Paint().SetColor(0xFF2040DD).SetAlphaF(0.8)

    def draw(verbs_pts, paint, clip, t):
        p = Path()
        p.MoveTo(*verbs_pts[1][0])
        if verbs_pts[0][1] == S.QUAD:
            p.QuadTo(*verbs_pts[1][1], *verbs_pts[1][2]).LineTo(*verbs_pts[1][3])
        else:
            for q in verbs_pts[1][1:]:
                p.LineTo(*q)
        p.Close()
        cv.DrawPath(p, paint)
        rec = paint.rec.copy()
        rec["translate"] = t
        b.draw_path(p.verbs, p.points, rec, clip=clip)

    draw(tri, red, None, (0.0, 0.0))
    cv.Save()
    cv.Translate(7.5, -3.25)
    cv.ClipRect(-5, 0, 130, 100)
    clip = S.map_clip(S.NO_CLIP, (-5, 0, 130, 100), 7.5, -3.25)
    layer_paint = Paint().SetAlphaF(0.55)
    cv.SaveLayer((3.5, 4.25, 120.75, 90.5), layer_paint)
    inner = b.save_layer((3.5, 4.25, 120.75, 90.5), float(np.float32(0.55)), S.BLEND_SRC_OVER,
                         (7.5, -3.25), clip)
    draw(quad, blue, inner, (7.5, -3.25))
    draw(tri, red, inner, (7.5, -3.25))
    cv.Restore()
    b.restore_layer()
    cv.Restore()
    draw(quad, Paint().SetColor(0x8020A040), None, (0.0, 0.0))
    cv.Flush()
    sc = b.build()
    assert sc.layers is not None and len(sc.layers) == 1
    assert _check(oracle_lib, bitmap, sc)["bad_pixels"] == 0


def test_canvas_save_layer_limits(gpu_ctx):
    from skity_gb300 import _lib
    from skity_gb300.canvas import Canvas
    bitmap = np.zeros((32, 32, 4), np.uint8)
    cv = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    cv.SaveLayer((0, 0, 16, 16))
    with pytest.raises(_lib.SkityCudaError) as e:  # a layer inside a layer
        cv.SaveLayer((2, 2, 8, 8))
    assert e.value.code == -5
    with pytest.raises(_lib.SkityCudaError) as e:  # a flush with the layer open
        cv.Flush()
    assert e.value.code == -5
    cv.Restore()
    cv.Flush()
