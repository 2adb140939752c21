"""Pins the oracle (oracle/sw_oracle.cc) to the reference software backend
compiled from the reference's own sources (oracle/ref/Makefile ->
oracle/_ref/ref_render): identical pixels on seeded scenes that cover every
behaviour of the path.  Runs where the reference build exists (it needs the
reference checkout to compile); CPU only."""
import numpy as np
import pytest

from skity_gb300 import scene as S


@pytest.fixture(scope="module")
def ref(oracle_lib):
    try:
        ok = oracle_lib.build_reference()
    except RuntimeError as e:
        pytest.skip(f"reference build failed: {e}")
    if not ok and not oracle_lib.reference_available():
        pytest.skip("reference checkout not present")
    return oracle_lib


def _pin(oracle_lib, sc):
    want = oracle_lib.render_reference(sc)
    got, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, want)
    assert c["bad_pixels"] == 0, c


@pytest.mark.parametrize("seed", range(8))
def test_random_fills(ref, seed):
    sc = S.random_paths_scene(S.SEED_BASE + 300 + seed, 96 + 16 * seed, 80 + 8 * seed, 40,
                              1, 24, coord_lo=(-20.0, -20.0),
                              coord_hi=(116.0 + 16 * seed, 100.0 + 8 * seed),
                              evenodd_frac=0.5)
    _pin(ref, sc)


@pytest.mark.parametrize("seed", range(6))
def test_random_strokes_and_gradients(ref, seed):
    sc = S.random_paths_scene(S.SEED_BASE + 320 + seed, 200, 150, 50, 2, 40,
                              coord_lo=(-30.0, -30.0), coord_hi=(230.0, 180.0),
                              evenodd_frac=0.3, gradient_frac=0.6, stroke_frac=0.5)
    _pin(ref, sc)


def test_config2_subset(ref):
    _pin(ref, S.config2(n_paths=200, width=2048, height=2048))


def test_blur_outlines(ref):
    _pin(ref, S.config4(seed=S.SEED_BASE + 340, n_outlines=400, width=384, height=384,
                        blur_frac=0.5))


def test_batch_canvases(ref):
    for sc in S.config3(n_canvases=6, scale=0.1):
        _pin(ref, sc)


def test_styles_blend_modes_and_tile_modes(ref):
    """Every Paint::Style, the four supported blend modes, all gradient tile
    modes and evenly spaced stops (no offsets), no clear colour."""
    b = S.SceneBuilder(120, 100, clear=None)
    rng = np.random.default_rng(11)
    for i in range(48):
        n = 3 + i % 5
        verbs = [S.MOVE] + [[S.LINE, S.QUAD, S.CUBIC][j % 3] for j in range(n)] + [S.CLOSE]
        npts = 1 + sum({S.LINE: 1, S.QUAD: 2, S.CUBIC: 3}[v] for v in verbs[1:-1])
        pts = rng.uniform(-10, 130, (npts, 2)).astype(np.float32)
        p = S.default_paint()
        p["style"] = i % 4
        p["stroke_width"] = float(1 + i % 6)
        p["cap"], p["join"] = i % 3, (i // 3) % 3
        p["blend"] = [S.BLEND_SRC_OVER, S.BLEND_SRC, S.BLEND_CLEAR, S.BLEND_DST][i % 4] \
            if i % 5 == 0 else S.BLEND_SRC_OVER
        p["fill_color"] = tuple(rng.uniform(0, 1, 4).astype(np.float32))
        p["stroke_color"] = tuple(rng.uniform(0, 1, 4).astype(np.float32))
        if i % 3 == 1:
            cols = rng.uniform(0, 1, (2 + i % 4, 4)).astype(np.float32)
            offs = None if i % 2 else np.sort(rng.uniform(0, 1, len(cols))).astype(np.float32)
            kind = S.GRAD_LINEAR if i % 6 == 1 else S.GRAD_RADIAL
            p["gradient"] = b.add_gradient(kind, (float(pts[0, 0]), float(pts[0, 1])),
                                           (float(pts[1, 0]), float(pts[1, 1])),
                                           (float(5 + i), 0.0), cols, offs, tile_mode=i % 4)
        b.draw_path(verbs, pts, p)
    _pin(ref, b.build())


def translated_scene(seed=S.SEED_BASE + 360):
    """Draws under Canvas::Translate: fills, strokes and gradients with
    per-draw translations (some fractional, some moving paths off-canvas)."""
    sc = S.random_paths_scene(seed, 180, 140, 40, 2, 24, coord_lo=(-20.0, -20.0),
                              coord_hi=(160.0, 120.0), evenodd_frac=0.4, gradient_frac=0.5,
                              stroke_frac=0.3)
    rng = np.random.default_rng(seed & 0xFFFF)
    for d in range(sc.n_draws):
        if d % 4 != 3:
            sc.paints[d]["translate"] = rng.uniform(-40, 40, 2).astype(np.float32)
    return sc


def test_canvas_translate(ref):
    _pin(ref, translated_scene())


def matrix_scene(seed=S.SEED_BASE + 365, width=180, height=140, shaded=True):
    """Draws under canvas matrices (Canvas::Scale / Rotate / Skew / Concat):
    fills (both fill rules) and strokes under scales (non-uniform, flipped,
    fractional), rotations, skews and their products, plus translations and
    the identity; gradients under the scale-and-translate matrices only
    (`shaded`)."""
    base = S.random_paths_scene(seed, width, height, 36, 2, 20, coord_lo=(-20.0, -20.0),
                                coord_hi=(width - 20.0, height - 20.0), evenodd_frac=0.4,
                                gradient_frac=0.5 if shaded else 0.0, stroke_frac=0.3)
    rng = np.random.default_rng(seed & 0xFFFF)
    b = S.SceneBuilder(width, height)
    gi = {}
    for d in range(base.n_draws):
        v0, v1 = int(base.verb_off[d]), int(base.verb_off[d + 1])
        p0, p1 = int(base.point_off[d]), int(base.point_off[d + 1])
        p = base.paints[d].copy()
        kind = d % 6
        f = np.float32
        if kind == 0:    # scale and translate
            sx, sy = rng.uniform(0.3, 1.8), rng.uniform(0.3, 1.8)
            m = (sx, 0.0, rng.uniform(-30, 60), 0.0, sy, rng.uniform(-30, 50))
        elif kind == 1:  # flip and scale
            m = (-rng.uniform(0.5, 1.5), 0.0, width * 0.9, 0.0, rng.uniform(0.5, 1.5), 5.5)
        elif kind == 2:  # rotation about a point
            a = f(rng.uniform(-3.1, 3.1))
            c, s_ = np.cos(a), np.sin(a)
            cx, cy = f(width / 2), f(height / 2)
            m = (c, -s_, f(cx - (c * cx - s_ * cy)), s_, c, f(cy - (s_ * cx + c * cy)))
        elif kind == 3:  # skew
            m = (1.0, rng.uniform(-0.6, 0.6), rng.uniform(-20, 20), rng.uniform(-0.4, 0.4), 1.0,
                 rng.uniform(-20, 20))
        elif kind == 4:  # a general affine map
            m = tuple(rng.uniform(-1.2, 1.2, 6) * (1, 1, 80, 1, 1, 60) + (0.2, 0, 60, 0, 0.2, 50))
        else:            # translation or identity
            m = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0) if d % 12 == 5 else \
                (1.0, 0.0, rng.uniform(-40, 40), 0.0, 1.0, rng.uniform(-40, 40))
        m = tuple(float(f(v)) for v in m)
        g = int(p["gradient"])
        if g >= 0 and (m[1] != 0.0 or m[3] != 0.0):
            g = -1  # shaders are taken under scale and translation only
        if g >= 0:
            if g not in gi:
                gr = base.gradients[g]
                s0, n = int(gr["stop_start"]), int(gr["stop_count"])
                gi[g] = b.add_gradient(int(gr["type"]), tuple(gr["p0"]), tuple(gr["p1"]),
                                       tuple(gr["radius"]), base.stop_colors[s0:s0 + n],
                                       base.stop_offsets[s0:s0 + n] if gr["has_offsets"] else None,
                                       int(gr["tile_mode"]))
            g = gi[g]
        p["gradient"] = g
        b.draw_path(base.verbs[v0:v1], base.points[p0:p1], p, matrix=m)
    return b.build()


@pytest.mark.parametrize("seed", range(3))
def test_canvas_matrices(ref, seed):
    _pin(ref, matrix_scene(S.SEED_BASE + 365 + seed))


def clipped_scene(seed=S.SEED_BASE + 380, width=180, height=140):
    """Draws under Canvas::ClipRect (kIntersect) and Translate, as a canvas
    sees them between Save and Restore: one or two nested clip rects per
    draw (fractional, unordered, partly off-canvas, disjoint = empty clip),
    some under a translation, some draws with the canvas's initial bounds."""
    sc = S.random_paths_scene(seed, width, height, 48, 2, 24, coord_lo=(-20.0, -20.0),
                              coord_hi=(width - 20.0, height - 20.0), evenodd_frac=0.4,
                              gradient_frac=0.5, stroke_frac=0.3)
    rng = np.random.default_rng(seed & 0xFFFF)
    clips = np.zeros((sc.n_draws, 4), np.float32)
    for d in range(sc.n_draws):
        tx, ty = (rng.uniform(-30, 30, 2).astype(np.float32) if d % 3 == 1 else (0.0, 0.0))
        sc.paints[d]["translate"] = (tx, ty)
        clip = S.NO_CLIP
        if d % 6 != 5:
            for _ in range(1 + (d % 4 == 0)):
                x0, x1 = rng.uniform(-30, width + 30, 2)
                y0, y1 = rng.uniform(-30, height + 30, 2)
                if d % 5 == 2:  # whole-pixel rects
                    x0, x1, y0, y1 = np.round([x0, x1, y0, y1])
                clip = S.map_clip(clip, (x0, y0, x1, y1), tx, ty)
        clips[d] = clip
    sc.clips = clips
    return sc


@pytest.mark.parametrize("seed", range(3))
def test_canvas_clip_rect(ref, seed):
    sc = clipped_scene(S.SEED_BASE + 380 + seed)
    assert np.any(sc.clips[:, 2] == 0)  # some draws under an empty clip
    _pin(ref, sc)



def blend_modes_scene(seed=S.SEED_BASE + 395, width=120, height=96):
    """Every BlendMode (kClear .. kLuminosity; the modes past kScreen other
    than kSoftLight blend as kSrcOver) with solid and gradient paints,
    fills and strokes, over a canvas cleared to a translucent colour so the
    destination alpha varies (opaque, translucent and transparent pixels)."""
    rng = np.random.default_rng(seed & 0xFFFF)
    b = S.SceneBuilder(width, height, clear=(0.3, 0.6, 0.2, 0.5))
    for i in range(3 * 29):
        mode = i % 29
        n = 3 + i % 6
        verbs = [S.MOVE] + [[S.LINE, S.QUAD, S.CUBIC][j % 3] for j in range(n)] + [S.CLOSE]
        npts = 1 + sum({S.LINE: 1, S.QUAD: 2, S.CUBIC: 3}[v] for v in verbs[1:-1])
        pts = rng.uniform(-10, width + 10, (npts, 2)).astype(np.float32)
        p = S.default_paint()
        p["blend"] = mode
        p["style"] = [S.FILL, S.STROKE, S.FILL][i // 29]
        p["stroke_width"] = float(2 + i % 5)
        alpha = [1.0, 0.0, rng.uniform(0.05, 0.95)][i % 3]
        p["fill_color"] = tuple(np.append(rng.uniform(0, 1, 3), alpha).astype(np.float32))
        p["stroke_color"] = p["fill_color"]
        if i % 4 == 3:
            cols = rng.uniform(0, 1, (3, 4)).astype(np.float32)
            p["gradient"] = b.add_gradient(S.GRAD_LINEAR if i % 8 == 3 else S.GRAD_RADIAL,
                                           (float(pts[0, 0]), float(pts[0, 1])),
                                           (float(pts[1, 0]), float(pts[1, 1])),
                                           (float(10 + i), 0.0), cols)
        b.draw_path(verbs, pts, p)
    return b.build()


def test_every_blend_mode(ref):
    _pin(ref, blend_modes_scene())


def sweep_conical_scene(seed=S.SEED_BASE + 396, width=140, height=110):
    """Sweep gradients (angle ranges within and past a turn, every tile
    mode) and two-point conical gradients in each of the brush's cases --
    general with the focal circle inside and outside, swapped ends (zero end
    radius), equal radii (strip), concentric (radial), a negative radius
    (transparent) -- on fills and strokes, some under a translation."""
    from skity_gb300.canvas import Shader
    rng = np.random.default_rng(seed & 0xFFFF)
    b = S.SceneBuilder(width, height)
    cases = ["sweep", "general", "general_big", "swap", "strip", "radial", "negative"]
    for i in range(6 * len(cases)):
        case = cases[i % len(cases)]
        n = 3 + i % 5
        verbs = [S.MOVE] + [[S.LINE, S.QUAD, S.CUBIC][j % 3] for j in range(n)] + [S.CLOSE]
        npts = 1 + sum({S.LINE: 1, S.QUAD: 2, S.CUBIC: 3}[v] for v in verbs[1:-1])
        pts = rng.uniform(-10, [width + 10, height + 10], (npts, 2)).astype(np.float32)
        p = S.default_paint()
        p["style"] = S.STROKE if i % 5 == 4 else S.FILL
        p["stroke_width"] = 3.0
        if i % 4 == 1:
            p["translate"] = tuple(rng.uniform(-15, 15, 2).astype(np.float32))
        k = 2 + i % 4
        cols = rng.uniform(0, 1, (k, 4)).astype(np.float32)
        offs = None if i % 3 == 0 else np.sort(rng.uniform(0, 1, k)).astype(np.float32)
        tile = (i // len(cases)) % 4
        c0 = tuple(rng.uniform(0, [width, height]).astype(np.float32))
        c1 = tuple(rng.uniform(0, [width, height]).astype(np.float32))
        if case == "sweep":
            a0 = float(rng.uniform(-180, 180))
            sh = Shader.MakeSweep(c0[0], c0[1], a0, a0 + float(rng.uniform(20, 500)), cols, offs, k,
                                  tile)
        elif case == "general":
            sh = Shader.MakeTwoPointConical(c0, float(rng.uniform(5, 20)), c1,
                                            float(rng.uniform(25, 60)), cols, offs, k, tile)
        elif case == "general_big":  # the start circle not inside the end one
            sh = Shader.MakeTwoPointConical(c0, float(rng.uniform(30, 60)), c1,
                                            float(rng.uniform(2, 10)), cols, offs, k, tile)
        elif case == "swap":
            sh = Shader.MakeTwoPointConical(c0, float(rng.uniform(10, 40)), c1, 0.0, cols, offs,
                                            k, tile)
        elif case == "strip":
            r = float(rng.uniform(5, 30))
            sh = Shader.MakeTwoPointConical(c0, r, c1, r, cols, offs, k, tile)
        elif case == "radial":
            sh = Shader.MakeTwoPointConical(c0, float(rng.uniform(5, 15)), c0,
                                            float(rng.uniform(20, 50)), cols, offs, k, tile)
        else:
            sh = Shader.MakeTwoPointConical(c0, -5.0, c1, 30.0, cols, offs, k, tile)
        assert sh is not None and sh.kind in (S.GRAD_SWEEP, S.GRAD_CONICAL), case
        p["gradient"] = b.add_gradient(sh.kind, sh.p0, sh.p1, sh.radius, sh.colors, sh.pos,
                                       tile_mode=sh.tile)
        b.draw_path(verbs, pts, p)
    return b.build()


def test_sweep_and_conical_gradients(ref):
    _pin(ref, sweep_conical_scene())


def blur_styles_scene(seed=S.SEED_BASE + 397):
    """Blurred outlines with every BlurStyle (kNormal, kSolid, kOuter,
    kInner) and their fills, over a cleared canvas."""
    sc = S.config4(seed=seed, n_outlines=240, width=256, height=256, blur_frac=0.6)
    blurred = np.nonzero(sc.paints["blur_style"] != 0)[0]
    sc.paints["blur_style"][blurred] = 1 + (np.arange(len(blurred)) % 4)
    return sc


def test_blur_styles(ref):
    sc = blur_styles_scene()
    assert set(np.unique(sc.paints["blur_style"])) >= {1, 2, 3, 4}
    _pin(ref, sc)


def color_filters_scene(seed=S.SEED_BASE + 398, width=128, height=100):
    """Every colour filter: Blend (all 29 modes, opaque, translucent and
    transparent colours), Matrix (channel swaps, negative terms, biases,
    saturating terms), LinearToSRGBGamma, SRGBToLinearGamma and Compose, on
    solid and gradient fills, strokes and blurred draws."""
    rng = np.random.default_rng(seed & 0xFFFF)
    b = S.SceneBuilder(width, height, clear=(0.8, 0.7, 0.3, 0.9))
    for i in range(96):
        n = 3 + i % 5
        verbs = [S.MOVE] + [[S.LINE, S.QUAD, S.CUBIC][j % 3] for j in range(n)] + [S.CLOSE]
        npts = 1 + sum({S.LINE: 1, S.QUAD: 2, S.CUBIC: 3}[v] for v in verbs[1:-1])
        pts = rng.uniform(-10, [width + 10, height + 10], (npts, 2)).astype(np.float32)
        p = S.default_paint()
        p["style"] = S.STROKE if i % 7 == 3 else S.FILL
        p["stroke_width"] = 3.0
        p["fill_color"] = tuple(np.append(rng.uniform(0, 1, 3), rng.uniform(0.2, 1)).astype(np.float32))
        p["stroke_color"] = p["fill_color"]
        if i % 5 == 2:
            cols = rng.uniform(0, 1, (3, 4)).astype(np.float32)
            p["gradient"] = b.add_gradient(S.GRAD_LINEAR, (float(pts[0, 0]), float(pts[0, 1])),
                                           (float(pts[1, 0]), float(pts[1, 1])), (0.0, 0.0), cols)
        if i % 11 == 6:
            p["blur_style"], p["blur_radius"] = 1 + i % 4, float(rng.uniform(1, 6))
        kind = [S.FILTER_BLEND, S.FILTER_MATRIX, S.FILTER_LINEAR_TO_SRGB, S.FILTER_SRGB_TO_LINEAR,
                S.FILTER_COMPOSE, S.FILTER_BLEND][i % 6]
        if kind == S.FILTER_BLEND:
            a = [255, 0, int(rng.integers(1, 255))][i % 3]
            argb = (a << 24) | int(rng.integers(0, 1 << 24))
            f = S.filter_record(kind, mode=(i // 6 + 7 * (i % 2)) % 29, color=argb)
        elif kind == S.FILTER_MATRIX:
            m = rng.uniform(-1.2, 1.2, 20).astype(np.float32)
            m[[4, 9, 14, 19]] = rng.uniform(-0.5, 0.5, 4)
            if i % 4 == 1:  # a channel swap with the alpha kept
                m = np.array([0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 0], np.float32)
            f = S.filter_record(kind, matrix=m)
        else:
            f = S.filter_record(kind)
        b.draw_path(verbs, pts, p, color_filter=f)
    return b.build()


def test_color_filters(ref):
    sc = color_filters_scene()
    assert set(np.unique(sc.filters["type"])) == {1, 2, 3, 4, 5}
    _pin(ref, sc)


def _random_closed_path(rng, lo, hi, n_verbs):
    verbs = [S.MOVE] + [[S.LINE, S.QUAD, S.CUBIC][int(rng.integers(0, 3))] for _ in range(n_verbs)]
    verbs.append(S.CLOSE)
    npts = 1 + sum({S.LINE: 1, S.QUAD: 2, S.CUBIC: 3}[v] for v in verbs[1:-1])
    return verbs, rng.uniform(lo, hi, (npts, 2)).astype(np.float32)


def path_clips_scene(seed=S.SEED_BASE + 399, width=160, height=120, n_ops=90):
    """Canvas::ClipPath with kIntersect and kDifference (curved and polygon
    paths, both fill rules, rects), nested under Save / Restore, mixed with
    ClipRect and Translate, over fills, strokes and gradients; the draws
    replay the canvas's clip state as the software canvas keeps it."""
    rng = np.random.default_rng(seed & 0xFFFF)
    b = S.SceneBuilder(width, height, clear=(1.0, 1.0, 1.0, 1.0))
    glob, t = S.NO_CLIP, (0.0, 0.0)
    stack = []
    for i in range(n_ops):
        r = rng.random()
        if r < 0.08 and stack:
            b.restore()
            glob, t = stack.pop()
        elif r < 0.16:
            b.save()
            stack.append((glob, t))
        elif r < 0.30:
            op = S.CLIP_INTERSECT if rng.random() < 0.6 else S.CLIP_DIFFERENCE
            if rng.random() < 0.3:
                x0, y0 = rng.uniform(-20, [width, height])
                x1, y1 = x0 + rng.uniform(10, 90), y0 + rng.uniform(10, 70)
                verbs = [S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE]
                pts = np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1]], np.float32)
            else:
                verbs, pts = _random_closed_path(rng, [-20, -20], [width + 20, height + 20],
                                                 int(rng.integers(3, 9)))
            fill = S.EVEN_ODD if rng.random() < 0.3 else S.WINDING
            b.clip_path(verbs, pts, op, fill, translate=t, bounds=glob)
            if op == S.CLIP_INTERSECT:  # ClipPath narrows the global clip bounds too
                pb = (pts[:, 0].min(), pts[:, 1].min(), pts[:, 0].max(), pts[:, 1].max())
                glob = S.map_clip(glob, pb, t[0], t[1])
        elif r < 0.34:
            t = (float(np.float32(t[0]) + np.float32(rng.uniform(-12, 12))),
                 float(np.float32(t[1]) + np.float32(rng.uniform(-12, 12))))
        elif r < 0.38:
            x0, y0 = rng.uniform(-10, [width, height])
            glob = S.map_clip(glob, (x0, y0, x0 + rng.uniform(20, 120), y0 + rng.uniform(20, 90)),
                              t[0], t[1])
        else:
            verbs, pts = _random_closed_path(rng, [-10, -10], [width + 10, height + 10],
                                             int(rng.integers(2, 12)))
            p = S.default_paint()
            p["style"] = S.STROKE if rng.random() < 0.2 else S.FILL
            p["stroke_width"] = float(rng.uniform(1, 6))
            p["fill_type"] = S.EVEN_ODD if rng.random() < 0.3 else S.WINDING
            p["fill_color"] = tuple(np.append(rng.uniform(0, 1, 3), rng.uniform(0.3, 1)).astype(np.float32))
            p["stroke_color"] = p["fill_color"]
            p["translate"] = t
            if rng.random() < 0.15:
                p["blend"] = S.BLEND_SRC
            if rng.random() < 0.2:
                cols = rng.uniform(0, 1, (3, 4)).astype(np.float32)
                p["gradient"] = b.add_gradient(S.GRAD_RADIAL, (float(pts[0, 0]), float(pts[0, 1])),
                                               (0.0, 0.0), (float(rng.uniform(10, 60)), 0.0), cols)
            b.draw_path(verbs, pts, p, clip=glob)
    return b.build()


@pytest.mark.parametrize("seed", range(4))
def test_clip_path(ref, seed):
    sc = path_clips_scene(S.SEED_BASE + 399 + seed)
    assert sc.path_clips is not None and (sc.path_clips[4] != 0).any()
    _pin(ref, sc)


def clip_path_cases_scene():
    """The path-clip combinations one by one (intersect, difference, and each
    op nested in each, an even-odd star, a clip under a translation), each
    between Save and Restore, over a rect and a stroked curve."""
    b = S.SceneBuilder(96, 72)
    tri = ([S.MOVE, S.LINE, S.LINE, S.CLOSE], [[5, 5], [90, 12], [30, 68]])
    band = ([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE], [[0, 28], [96, 28], [96, 44], [0, 44]])
    star = ([S.MOVE, S.LINE, S.LINE, S.LINE, S.LINE, S.CLOSE],
            [[48, 2], [70, 66], [10, 24], [86, 24], [26, 66]])
    rect = ([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE], [[3, 3], [93, 3], [93, 69], [3, 69]])
    curve = ([S.MOVE, S.CUBIC], [[4, 60], [30, -20], [60, 100], [92, 8]])
    cases = [((tri, S.CLIP_INTERSECT, S.WINDING), None), ((tri, S.CLIP_DIFFERENCE, S.WINDING), None),
             ((tri, S.CLIP_INTERSECT, S.WINDING), (band, S.CLIP_INTERSECT)),
             ((tri, S.CLIP_INTERSECT, S.WINDING), (band, S.CLIP_DIFFERENCE)),
             ((tri, S.CLIP_DIFFERENCE, S.WINDING), (band, S.CLIP_DIFFERENCE)),
             ((tri, S.CLIP_DIFFERENCE, S.WINDING), (band, S.CLIP_INTERSECT)),
             ((star, S.CLIP_INTERSECT, S.EVEN_ODD), None)]
    for k, (first, second) in enumerate(cases):
        b.save()
        t = (float(k % 3) * 0.5, float(k % 2) * 1.25)
        (verbs, pts), op, fill = first
        b.clip_path(verbs, pts, op, fill, translate=t)
        if second is not None:
            (v2, p2), op2 = second
            b.clip_path(v2, p2, op2)
        p = S.default_paint()
        p["fill_color"] = (0.1 * k, 0.9 - 0.1 * k, 0.5, 0.6)
        b.draw_path(*rect, p)
        q = S.default_paint()
        q["style"], q["stroke_width"] = S.STROKE, 3.0
        q["stroke_color"] = (0.9, 0.1, 0.1 * k, 0.8)
        b.draw_path(*curve, q)
        b.restore()
    return b.build()


def test_clip_path_cases(ref):
    _pin(ref, clip_path_cases_scene())


def _random_matrix(rng, width, height, kind):
    """A canvas matrix (sx, kx, tx, ky, sy, ty) of one of five kinds:
    0 translation, 1 scale and translate, 2 rotation about the centre,
    3 skew, 4 general affine."""
    f = np.float32
    if kind == 0:
        m = (1.0, 0.0, rng.uniform(-20, 20), 0.0, 1.0, rng.uniform(-20, 20))
    elif kind == 1:
        m = (rng.uniform(0.5, 1.6) * rng.choice([-1, 1]), 0.0, rng.uniform(-20, 40), 0.0,
             rng.uniform(0.5, 1.6), rng.uniform(-20, 40))
        if m[0] < 0:
            m = (m[0], 0.0, m[2] + width, 0.0, m[4], m[5])
    elif kind == 2:
        a = f(rng.uniform(-3.1, 3.1))
        c, s_ = np.cos(a), np.sin(a)
        cx, cy = f(width / 2), f(height / 2)
        m = (c, -s_, f(cx - (c * cx - s_ * cy)), s_, c, f(cy - (s_ * cx + c * cy)))
    elif kind == 3:
        m = (1.0, rng.uniform(-0.5, 0.5), rng.uniform(-15, 15), rng.uniform(-0.4, 0.4), 1.0,
             rng.uniform(-15, 15))
    else:
        m = tuple(rng.uniform(-1.1, 1.1, 6) * (1, 1, 60, 1, 1, 50) + (0.3, 0, width / 2, 0, 0.3,
                                                                   height / 2))
    return tuple(float(f(v)) for v in m)


def matrix_clips_scene(seed=S.SEED_BASE + 470, width=150, height=110, n_ops=70):
    """ClipPath under canvas matrices of every kind, ClipRect under them (a
    rect path clip under a rotation or skew, Canvas::OnClipRect), nested
    under Save / Restore; fills and strokes under any matrix beneath those
    clips; blurs (every style) under scale-and-translate matrices, clip
    rects and path clips."""
    rng = np.random.default_rng(seed & 0xFFFF)
    b = S.SceneBuilder(width, height, clear=(1.0, 1.0, 1.0, 1.0))
    glob, m = S.NO_CLIP, (1.0, 0.0, 0.0, 0.0, 1.0, 0.0)
    stack = []
    for i in range(n_ops):
        r = rng.random()
        st = m[1] == 0.0 and m[3] == 0.0
        if r < 0.07 and stack:
            b.restore()
            glob, m = stack.pop()
        elif r < 0.14:
            b.save()
            stack.append((glob, m))
        elif r < 0.24:
            m = _random_matrix(rng, width, height, int(rng.integers(0, 5)))
        elif r < 0.34:
            op = S.CLIP_INTERSECT if rng.random() < 0.7 else S.CLIP_DIFFERENCE
            verbs, pts = _random_closed_path(rng, [-10, -10], [width + 10, height + 10],
                                             int(rng.integers(3, 8)))
            if op == S.CLIP_INTERSECT:  # Canvas::ClipPath narrows the bounds first
                pb = (pts[:, 0].min(), pts[:, 1].min(), pts[:, 0].max(), pts[:, 1].max())
                glob = S.map_clip_matrix(glob, pb, m)
            fill = S.EVEN_ODD if rng.random() < 0.3 else S.WINDING
            b.clip_path(verbs, pts, op, fill, bounds=glob, matrix=m)
        elif r < 0.42:
            x0, y0 = rng.uniform(-10, [width * 0.7, height * 0.7])
            rect = tuple(float(np.float32(v)) for v in
                         (x0, y0, x0 + rng.uniform(30, 120), y0 + rng.uniform(25, 90)))
            glob = S.map_clip_matrix(glob, rect, m)
            if not st:  # SWCanvas::OnClipRect -> Canvas::OnClipRect: the rect as a path
                b.clip_path(S.RECT_VERBS, S.rect_points(rect), S.CLIP_INTERSECT, S.WINDING,
                            bounds=glob, matrix=m)
        else:
            verbs, pts = _random_closed_path(rng, [-10, -10], [width + 10, height + 10],
                                             int(rng.integers(2, 10)))
            p = S.default_paint()
            p["style"] = S.STROKE if rng.random() < 0.2 else S.FILL
            p["stroke_width"] = float(rng.uniform(1, 6))
            p["fill_type"] = S.EVEN_ODD if rng.random() < 0.3 else S.WINDING
            p["fill_color"] = tuple(np.append(rng.uniform(0, 1, 3),
                                              rng.uniform(0.3, 1)).astype(np.float32))
            p["stroke_color"] = p["fill_color"]
            if st and rng.random() < 0.35:
                p["blur_style"] = int(rng.integers(1, 5))
                p["blur_radius"] = float(np.float32(rng.uniform(1.0, 6.0)))
            elif st and rng.random() < 0.2:
                cols = rng.uniform(0, 1, (3, 4)).astype(np.float32)
                p["gradient"] = b.add_gradient(S.GRAD_LINEAR,
                                               (float(pts[0, 0]), float(pts[0, 1])),
                                               (float(pts[1, 0]), float(pts[1, 1])), (0.0, 0.0),
                                               cols)
            b.draw_path(verbs, pts, p, clip=glob, matrix=m)
    return b.build()


@pytest.mark.parametrize("seed", range(6))
def test_clips_and_blurs_under_matrices(ref, seed):
    sc = matrix_clips_scene(S.SEED_BASE + 470 + seed)
    assert sc.clip_matrices is not None
    assert (sc.paints["blur_style"] != 0).any()
    _pin(ref, sc)


@pytest.mark.parametrize("seed", range(8))
def test_layers(ref, seed):
    """Canvas::SaveLayer / Restore: layers over and past the canvas with
    fractional bounds, alpha, several blend modes, under translations and
    narrowed clips, with fills, strokes and gradients inside and outside."""
    sc = S.layered_scene(S.SEED_BASE + 700 + seed, 120 + 8 * seed, 96 + 4 * seed, 30, 3,
                         blends=(3, 1, 24, 6, 11, 21))
    _pin(ref, sc)
