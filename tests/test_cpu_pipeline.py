"""The CUDA kernels' per-thread bodies, executed on the CPU, against the
oracle: geometry, introsort, sweep, span layout, compositing and blur are
checked bit-exact before any GPU run (tests/cpu_pipeline.cc)."""
import ctypes

import numpy as np
import pytest

from skity_gb300 import scene as S


def cpu_render(lib, sc):
    b = sc.to_bytes()
    out = np.zeros((sc.height, sc.width, 4), np.uint8)
    st = (ctypes.c_uint64 * 6)()
    rc = lib.skc_cpu_render(b, len(b), out.ctypes.data, st)
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
