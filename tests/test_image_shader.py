"""Image shaders and DrawImageRect (PixmapBrush over BitmapSampler,
sw_canvas.cc:641-677 and :755-786, sw_span_brush.cc:555-579,
bitmap_sampler.cc:12-108).

The oracle's sampler is pinned to the known answers of the reference's own
sampler tests (test/ut/graphic/bitmap_test.cc:141-228); the device path is
compared with the oracle on seeded scenes, through the CPU build of the
device code here and on the GPU."""
import os
import sys

import numpy as np
import pytest

from skity_gb300 import scene as S

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

RED, GREEN, BLUE, YELLOW, MAGENTA = 0xFFFF0000, 0xFF00FF00, 0xFF0000FF, 0xFFFFFF00, 0xFFFF00FF


def _pixmap(colors, w, h):
    """Bitmap::SetPixel of ARGB colours into RGBA8 rows."""
    px = np.zeros((h, w, 4), np.uint8)
    for i, c in enumerate(colors):
        y, x = divmod(i, w)
        px[y, x] = ((c >> 16) & 255, (c >> 8) & 255, c & 255, c >> 24)
    return px


def test_sampler_known_answers(oracle_lib):
    """The reference's BitmapSampler tests, value for value."""
    quad = _pixmap([RED, GREEN, BLUE, YELLOW], 2, 2)
    s = lambda px, f, t, u, v: oracle_lib.sample(px, S.ALPHA_PREMUL, f, t, t, u, v)
    # NearestNeighborSample
    assert s(quad, 0, S.TILE_CLAMP, 0.25, 0.25) == RED
    assert s(quad, 0, S.TILE_CLAMP, 0.75, 0.25) == GREEN
    assert s(quad, 0, S.TILE_CLAMP, 0.25, 0.75) == BLUE
    assert s(quad, 0, S.TILE_CLAMP, 0.75, 0.75) == YELLOW
    # LinearSample: the centre averages the four, truncated
    c = s(quad, 1, S.TILE_CLAMP, 0.5, 0.5)
    assert ((c >> 16) & 255, (c >> 8) & 255, c & 255) == (127, 127, 63)
    # TileModeClamp
    one = _pixmap([MAGENTA], 1, 1)
    for uv in (-1.0, 0.5, 2.0):
        assert s(one, 0, S.TILE_CLAMP, uv, uv) == MAGENTA
    # TileModeRepeat
    assert s(quad, 0, S.TILE_REPEAT, 1.25, 1.25) == RED
    assert s(quad, 0, S.TILE_REPEAT, -0.25, -0.75) == GREEN
    # TileModeMirror
    row = _pixmap([RED, GREEN], 2, 1)
    assert s(row, 0, S.TILE_MIRROR, 0.25, 0.0) == RED
    assert s(row, 0, S.TILE_MIRROR, 0.75, 0.0) == GREEN
    assert s(row, 0, S.TILE_MIRROR, 1.25, 0.0) == GREEN
    assert s(row, 0, S.TILE_MIRROR, 1.75, 0.0) == RED
    assert s(row, 0, S.TILE_MIRROR, 2.25, 0.0) == RED
    # decal: transparent outside [0, 1)
    assert s(quad, 0, S.TILE_DECAL, 1.0, 0.5) == 0
    assert s(quad, 0, S.TILE_DECAL, -0.01, 0.5) == 0


def image_scene(seed=S.SEED_BASE + 410, width=150, height=120):
    """Image-shaded fills and strokes (every tile mode, nearest / linear /
    cubic, premultiplied and unpremultiplied pixels, scaled and translated
    local matrices, canvas translations, blend modes, paint alpha) and
    DrawImageRect calls."""
    rng = np.random.default_rng(seed)
    b = S.SceneBuilder(width, height, clear=(0.9, 0.95, 1.0, 1.0))
    imgs = []
    for k in range(4):
        w, h = int(rng.integers(1, 24)), int(rng.integers(1, 24))
        px = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
        premul = k % 2 == 0
        if premul:  # valid premultiplied pixels
            px[..., :3] = np.minimum(px[..., :3], px[..., 3:4])
        imgs.append(b.add_image(px, S.ALPHA_PREMUL if premul else S.ALPHA_UNPREMUL))
    for i in range(36):
        p = S.default_paint()
        p["fill_color"] = (0.0, 0.0, 0.0, float(rng.choice([1.0, 0.6, 0.3])))
        p["blend"] = int(rng.choice([3, 3, 3, 1, 12, 14]))
        p["translate"] = (float(rng.integers(-6, 7)), float(rng.integers(-6, 7))) \
            if i % 3 == 0 else (0.0, 0.0)
        img = int(rng.choice(imgs))
        if i % 4 == 3:
            w = float(rng.uniform(2, 20)); h = float(rng.uniform(2, 20))
            src = (float(rng.uniform(-2, 4)), float(rng.uniform(-2, 4)))
            src = (src[0], src[1], src[0] + float(rng.uniform(1, 20)), src[1] + float(rng.uniform(1, 20)))
            x0, y0 = float(rng.uniform(-10, width - 10)), float(rng.uniform(-10, height - 10))
            dst = (x0, y0, x0 + float(rng.uniform(4, 70)), y0 + float(rng.uniform(4, 60)))
            b.draw_image_rect(img, src, dst, p, filter=int(rng.integers(0, 3)))
            continue
        sx, sy = float(rng.uniform(0.3, 5)), float(rng.uniform(0.3, 5))
        local = (sx, 0.0, float(rng.uniform(-30, 60)), 0.0, sy, float(rng.uniform(-30, 60)))
        rec = S.image_shader(img, int(rng.integers(0, 3)), int(rng.integers(0, 4)),
                             int(rng.integers(0, 4)), local)
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        n = int(rng.integers(3, 7))
        ang = np.sort(rng.uniform(0, 2 * np.pi, n))
        rad = rng.uniform(8, 45, n)
        pts = np.stack([cx + rad * np.cos(ang), cy + rad * np.sin(ang)], 1).astype(np.float32)
        verbs = [S.MOVE] + [S.LINE] * (n - 1) + [S.CLOSE]
        if i % 5 == 1:
            p["style"], p["stroke_width"] = S.STROKE, float(rng.uniform(1, 8))
            p["stroke_color"] = (0.0, 0.0, 0.0, float(rng.choice([1.0, 0.5])))
        b.draw_path(verbs, pts, p, image_shader=rec)
    return b.build()


def test_image_scene_oracle_runs(oracle_lib):
    px, st = oracle_lib.render(image_scene())
    assert px.shape == (120, 150, 4) and st.fragments > 0


def test_image_scene_cpu_pipeline(cpu_pipeline, oracle_lib):
    from test_cpu_pipeline import cpu_render
    for seed in range(3):
        sc = image_scene(S.SEED_BASE + 410 + seed)
        got, _ = cpu_render(cpu_pipeline, sc)
        ref, _ = oracle_lib.render(sc)
        assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


@pytest.mark.gpu
def test_image_scene_gpu(gpu_ctx, oracle_lib):
    from test_gpu_parity import check
    for seed in range(3):
        sc = image_scene(S.SEED_BASE + 410 + seed)
        c = check(oracle_lib, gpu_ctx.render_streams([sc])[0], sc)
        assert c["bad_pixels"] == 0, c


@pytest.mark.gpu
def test_draw_image_rect_canvas_api(gpu_ctx, oracle_lib):
    """Canvas.DrawImageRect / DrawImage and an image-shaded DrawPath through
    the C ABI, against the same draws as a scene for the oracle."""
    from skity_gb300.canvas import Canvas, FilterMode, Image, Paint, Path, Shader, TileMode
    rng = np.random.default_rng(S.SEED_BASE + 420)
    px = rng.integers(0, 256, (9, 13, 4), dtype=np.uint8)
    bitmap = np.zeros((60, 80, 4), np.uint8)
    canvas = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    canvas.Clear((1.0, 1.0, 1.0, 1.0))
    img = Image.MakeImage(px)  # unpremultiplied, the Pixmap default
    canvas.DrawImageRect(img, (1, 2, 11, 8), (5, 4, 47, 33), FilterMode.kLinear)
    canvas.DrawImage(img, 50, 30)
    paint = Paint()
    paint.SetShader(Shader.MakeShader(img, FilterMode.kNearest, TileMode.kMirror,
                                      TileMode.kRepeat, (2.0, 0.0, 3.0, 0.0, 1.5, -4.0)))
    canvas.DrawPath(Path().MoveTo(40, 2).LineTo(78, 20).LineTo(52, 58).Close(), paint)
    canvas.Flush()
    sb = S.SceneBuilder(80, 60, clear=(1.0, 1.0, 1.0, 1.0))
    i = sb.add_image(px, S.ALPHA_UNPREMUL)
    sb.draw_image_rect(i, (1, 2, 11, 8), (5, 4, 47, 33), S.default_paint(), S.FILTER_LINEAR)
    sb.draw_image_rect(i, (0, 0, 13, 9), (50, 30, 63, 39), S.default_paint())
    sb.draw_path([S.MOVE, S.LINE, S.LINE, S.CLOSE], [(40, 2), (78, 20), (52, 58)],
                 S.default_paint(),
                 image_shader=S.image_shader(i, S.FILTER_NEAREST, S.TILE_MIRROR, S.TILE_REPEAT,
                                             (2.0, 0.0, 3.0, 0.0, 1.5, -4.0)))
    ref, _ = oracle_lib.render(sb.build())
    assert oracle_lib.compare(bitmap, ref)["bad_pixels"] == 0
