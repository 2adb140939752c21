"""The CUDA kernels' per-thread bodies, executed on the CPU, against the
oracle: geometry, introsort, sweep, span layout, compositing and blur are
checked bit-exact before any GPU run (tests/cpu_pipeline.cc)."""
import ctypes

import numpy as np
import pytest

from skity_gb300 import scene as S


def cpu_render(lib, sc, mode=0):
    """mode 0: register sweep (generic sweep for passes it gives up on), as
    the GPU pipeline runs it; mode 1: generic sweep for every pass; mode 2:
    every pass forced through the 32-edge register form (the wider ones give
    up and are swept again after the register forms, as k_sweep_retry does)."""
    b = sc.to_bytes()
    out = np.zeros((sc.height, sc.width, 4), np.uint8)
    st = (ctypes.c_uint64 * 6)()
    rc = lib.skc_cpu_render_mode(b, len(b), out.ctypes.data, st, mode, 0)
    assert rc == 0, rc
    return out, list(st)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_fill_paths_bit_exact(cpu_pipeline, oracle_lib, seed):
    sc = S.random_paths_scene(S.SEED_BASE + 100 + seed, 200, 160, 60, 3, 32)
    got, st = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0
    assert st[3] == 0 or st[3] > 0  # retries are allowed, results must match


def test_config2_mix_bit_exact(cpu_pipeline, oracle_lib):
    """Strokes (all caps and joins), gradients, both fill rules, clipping."""
    sc = S.config2(n_paths=120, width=512, height=512)
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def test_blur_bit_exact(cpu_pipeline, oracle_lib):
    sc = S.config4(n_outlines=400, width=256, height=256, blur_frac=0.5)
    got, st = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert st[4] > 0
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def test_introsort_matches_std_sort(cpu_pipeline):
    """Tied keys must come out in std::sort's order (the reference sorts its
    edges with std::sort, sw_raster.cc:679-704)."""
    rng = np.random.default_rng(7)
    for n in list(range(0, 40)) + [64, 100, 257, 1000, 4096]:
        for distinct in (1, 2, 5, 50, 10**6):
            keys = rng.integers(0, distinct, n).astype(np.int32)
            a = np.zeros(n, np.int32)
            b = np.zeros(n, np.int32)
            cpu_pipeline.skc_cpu_introsort(keys.ctypes.data, a.ctypes.data, n)
            cpu_pipeline.skc_std_sort(keys.ctypes.data, b.ctypes.data, n)
            assert np.array_equal(a, b), (n, distinct)
    # adversarial inputs that drive introsort into its heapsort fallback
    for n in (100, 1000, 5000):
        keys = np.concatenate([np.arange(n // 2), np.arange(n // 2)[::-1]]).astype(np.int32) % 7
        a = np.zeros(len(keys), np.int32)
        b = np.zeros(len(keys), np.int32)
        cpu_pipeline.skc_cpu_introsort(keys.ctypes.data, a.ctypes.data, len(keys))
        cpu_pipeline.skc_std_sort(keys.ctypes.data, b.ctypes.data, len(keys))
        assert np.array_equal(a, b)


def test_edge_cases_bit_exact(cpu_pipeline, oracle_lib):
    b = S.SceneBuilder(64, 48)
    p = S.default_paint()
    p["fill_color"] = (0.2, 0.4, 0.6, 0.8)
    b.draw_path([S.MOVE], [(1, 1)], p)                              # lone move
    b.draw_path([S.MOVE, S.LINE, S.CLOSE], [(2, 2), (30, 2)], p)    # horizontal line
    b.draw_path([S.MOVE, S.LINE, S.LINE, S.CLOSE], [(-50, -50), (200, 10), (10, 300)], p)
    b.draw_path([S.MOVE, S.LINE, S.LINE], [(5, 5), (40, 5.5), (20, 40)], p)  # no close
    b.draw_path([S.MOVE, S.QUAD, S.CUBIC, S.CLOSE],
                [(3, 40), (30, -20), (60, 40), (10, 10), (50, 10), (3, 40)], p)
    q = p.copy(); q["fill_type"] = S.EVEN_ODD
    b.draw_path([S.MOVE, S.LINE, S.LINE, S.LINE, S.LINE, S.CLOSE],
                [(10, 10), (50, 40), (50, 10), (10, 40), (30, 0)], q)
    s = p.copy(); s["style"] = S.STROKE; s["stroke_width"] = 0.0
    b.draw_path([S.MOVE, S.LINE], [(1, 30), (60, 31)], s)           # hairline width 0
    s2 = p.copy(); s2["style"] = S.STROKE_AND_FILL; s2["stroke_width"] = 3; s2["cap"] = S.ROUND
    b.draw_path([S.MOVE, S.CONIC, S.CLOSE], [(10, 20), (30, 0), (50, 20)], s2, weights=[0.5])
    sc = b.build()
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def _stripes(b, paint, n, x0, y0s, w, h):
    verbs, pts = [], []
    for i in range(n):
        x, y = x0 + 2.5 * i, y0s[i]
        verbs += [S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE]
        pts += [(x, y), (x + w, y + 0.3), (x + w, y + h), (x, y + h - 0.4)]
    b.draw_path(verbs, pts, paint)


def test_long_active_lists_fall_back_to_generic_sweep(cpu_pipeline, oracle_lib):
    """More active edges than the register sweep holds (128): at the first
    step and at an insertion; a path just under the limit stays in it.
    Both sweep forms must give the oracle's pixels."""
    b = S.SceneBuilder(420, 140)
    p = S.default_paint()
    p["fill_color"] = (0.1, 0.5, 0.9, 0.7)
    _stripes(b, p, 90, 3.0, [5.0] * 90, 1.7, 60.0)                        # 180 at once
    _stripes(b, p, 90, 5.0, [70.0 + 0.25 * i for i in range(90)], 1.3, 50.0)  # grows past 128
    q = p.copy()
    q["fill_type"] = S.EVEN_ODD
    _stripes(b, q, 62, 40.0, [30.0 + 0.5 * i for i in range(62)], 2.1, 70.0)  # 124 at most
    sc = b.build()
    ref, _ = oracle_lib.render(sc)
    got, st = cpu_render(cpu_pipeline, sc)
    assert st[5] == 2, st
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0
    generic, st1 = cpu_render(cpu_pipeline, sc, mode=1)
    assert st1[5] == 3
    assert np.array_equal(got, generic)


def test_register_give_up_path(cpu_pipeline, oracle_lib):
    """Passes whose active list outgrows the register form they were given
    are swept again by the generic form after every register form; the
    pixels do not change."""
    sc = S.config2(n_paths=80, width=384, height=384)
    a, st0 = cpu_render(cpu_pipeline, sc, 0)
    f, st2 = cpu_render(cpu_pipeline, sc, 2)
    assert st2[5] > st0[5], (st0, st2)  # some passes gave up
    assert np.array_equal(a, f)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(f, ref)["bad_pixels"] == 0


def test_register_and_generic_sweeps_agree(cpu_pipeline):
    sc = S.config2(n_paths=60, width=384, height=384)
    a, _ = cpu_render(cpu_pipeline, sc, 0)
    g, _ = cpu_render(cpu_pipeline, sc, 1)
    assert np.array_equal(a, g)


def test_canvas_translate_bit_exact(cpu_pipeline, oracle_lib):
    from test_oracle_pin import translated_scene
    sc = translated_scene()
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


@pytest.mark.parametrize("seed", range(3))
def test_canvas_matrices_bit_exact(cpu_pipeline, oracle_lib, seed):
    """Canvas::Scale / Rotate / Skew / Concat: fills and strokes under every
    kind of affine canvas matrix, gradients under scale and translation."""
    from test_oracle_pin import matrix_scene
    sc = matrix_scene(S.SEED_BASE + 365 + seed)
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def test_matrix_limits_refused(cpu_pipeline, oracle_lib):
    """Under a rotation or skew a gradient is refused (its device_to_local
    needs the general inverse), as is a blur (its filtered bitmap's image
    draw inverts the matrix the same way); the oracle refuses the same
    draws."""
    from test_oracle_pin import matrix_scene
    sc = matrix_scene(S.SEED_BASE + 365, shaded=False)
    g = S.SceneBuilder(sc.width, sc.height)
    gi = g.add_gradient(S.GRAD_LINEAR, (0.0, 0.0), (50.0, 20.0), (0.0, 0.0),
                        [(1, 0, 0, 1), (0, 0, 1, 1)])
    p = S.default_paint()
    p["gradient"] = gi
    tri = ([S.MOVE, S.LINE, S.LINE, S.CLOSE], [(5, 5), (60, 10), (20, 50)])
    g.draw_path(*tri, p, matrix=(0.9, 0.3, 4.0, -0.3, 0.9, 6.0))
    blur = S.default_paint()
    blur["blur_style"], blur["blur_radius"] = 1, 3.0
    h = S.SceneBuilder(sc.width, sc.height)
    h.draw_path(*tri, blur, matrix=(0.9, 0.3, 4.0, -0.3, 0.9, 6.0))
    for bad in (g.build(), h.build()):
        b = bad.to_bytes()
        out = np.zeros((bad.height, bad.width, 4), np.uint8)
        st = (ctypes.c_uint64 * 6)()
        assert cpu_pipeline.skc_cpu_render_mode(b, len(b), out.ctypes.data, st, 0, 0) == -5
        with pytest.raises(RuntimeError):
            oracle_lib.render(bad)


@pytest.mark.parametrize("seed", range(3))
def test_clip_rect_bit_exact(cpu_pipeline, oracle_lib, seed):
    """Canvas::ClipRect bounds the scan of every later draw (fills, strokes,
    gradients, under translations, empty clips included)."""
    from test_oracle_pin import clipped_scene
    sc = clipped_scene(S.SEED_BASE + 380 + seed)
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def test_blur_under_clip_bit_exact(cpu_pipeline, oracle_lib):
    """A blurred draw under a narrowed clip: the temp canvas is unclipped,
    the filtered bitmap's image draw is clipped."""
    sc = S.config4(seed=S.SEED_BASE + 390, n_outlines=20, width=96, height=96, blur_frac=1.0)
    sc.clips = np.tile(np.array([[4, 4, 60, 60]], np.float32), (sc.n_draws, 1))
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0
    assert (got[61:] == got[95, 95]).all()  # nothing below the clip


@pytest.mark.parametrize("seed", range(6))
def test_clips_and_blurs_under_matrices_bit_exact(cpu_pipeline, oracle_lib, seed):
    """ClipPath and rotated ClipRect under canvas matrices, rotated draws
    under path clips, blurs under scales, clip rects and path clips."""
    from test_oracle_pin import matrix_clips_scene
    sc = matrix_clips_scene(S.SEED_BASE + 470 + seed)
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["bad_pixels"] == 0, c


def test_every_blend_mode_bit_exact(cpu_pipeline, oracle_lib):
    from test_oracle_pin import blend_modes_scene
    sc = blend_modes_scene()
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def test_sweep_and_conical_gradients_bit_exact(cpu_pipeline, oracle_lib):
    from test_oracle_pin import sweep_conical_scene
    sc = sweep_conical_scene()
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["bad_pixels"] == 0, c


def test_blur_styles_bit_exact(cpu_pipeline, oracle_lib):
    from test_oracle_pin import blur_styles_scene
    sc = blur_styles_scene()
    got, st = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert st[4] > 0  # temp canvases
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


def test_color_filters_bit_exact(cpu_pipeline, oracle_lib):
    from test_oracle_pin import color_filters_scene
    sc = color_filters_scene()
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0


@pytest.mark.parametrize("seed", range(4))
def test_clip_path_bit_exact(cpu_pipeline, oracle_lib, seed):
    """Canvas::ClipPath states (intersect / difference, nested) computed row
    by row and applied to the draws' rows, against the oracle."""
    from test_oracle_pin import path_clips_scene
    sc = path_clips_scene(S.SEED_BASE + 399 + seed)
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["bad_pixels"] == 0, c


def test_clip_path_cases_bit_exact(cpu_pipeline, oracle_lib):
    from test_oracle_pin import clip_path_cases_scene
    sc = clip_path_cases_scene()
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["bad_pixels"] == 0, c


def test_fixed_div_matches_64bit_quotient(cpu_pipeline):
    """The device FixedDiv (three 32-bit divisions for divisors below 2^24)
    against the 64-bit truncated quotient: random pairs over every magnitude,
    the extremes, and the small FDot6 values the raster divides most."""
    rng = np.random.default_rng(7)
    n = 2_000_000
    mags = rng.integers(0, 32, size=n)
    numer = (rng.integers(0, 2**31, size=n, dtype=np.int64) >> (31 - mags)).astype(np.int64)
    numer *= np.where(rng.random(n) < 0.5, -1, 1)
    dm = rng.integers(0, 32, size=n)
    denom = (rng.integers(1, 2**31, size=n, dtype=np.int64) >> (31 - dm)).astype(np.int64)
    denom = np.maximum(denom, 1) * np.where(rng.random(n) < 0.5, -1, 1)
    edge = np.array([-2**31, 2**31 - 1, 0, 1, -1, 2**24 - 1, 2**24, -(2**24) + 1], np.int64)
    en, ed = np.meshgrid(edge, np.array([1, -1, 2, 3, 2**24 - 1, -(2**24 - 1), 2**24, 2**31 - 1,
                                         -2**31, 16, -64], np.int64))
    numer = np.concatenate([numer, en.ravel()]).astype(np.int32)
    denom = np.concatenate([denom, ed.ravel()]).astype(np.int32)
    assert cpu_pipeline.skc_cpu_fixed_div_check(numer.ctypes.data, denom.ctypes.data, len(numer)) == 0


@pytest.mark.parametrize("seed", range(6))
def test_layers_bit_exact(cpu_pipeline, oracle_lib, seed):
    """Canvas::SaveLayer / Restore: layer temp canvases and their restore
    image passes (alpha, blend modes, translations, clips, fractional
    bounds) against the oracle."""
    sc = S.layered_scene(S.SEED_BASE + 700 + seed, 120 + 8 * seed, 96 + 4 * seed, 30, 3,
                         blends=(3, 1, 24, 6, 11))
    got, _ = cpu_render(cpu_pipeline, sc)
    ref, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, ref)["bad_pixels"] == 0
