"""The FP64 exact-area coverage oracle (oracle/exact_area.cc): exact on
polygons, union semantics for nonzero and even-odd, and the coverage-error
report of the reference rasteriser (the oracle, pinned to it) against true
area on a seeded scene.  CPU only."""
import pytest

from skity_gb300 import scene as S


def _one(verbs, pts, even_odd=False, w=32, h=32):
    b = S.SceneBuilder(w, h, clear=(0.0, 0.0, 0.0, 0.0))
    p = S.default_paint()
    p["fill_color"] = (1.0, 1.0, 1.0, 1.0)
    p["fill_type"] = S.EVEN_ODD if even_odd else S.WINDING
    b.draw_path(verbs, pts, p)
    return b.build()


def test_polygon_areas_are_exact(oracle_lib):
    rect = _one([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE],
                [(2.25, 3.5), (10.75, 3.5), (10.75, 9.25), (2.25, 9.25)])
    cov = oracle_lib.exact_coverage(rect, 0)
    assert cov[3, 2] == pytest.approx(0.75 * 0.5)
    assert cov[5, 5] == 1.0 and cov[0, 0] == 0.0
    assert cov.sum() == pytest.approx(8.5 * 5.75, abs=1e-9)
    tri = _one([S.MOVE, S.LINE, S.LINE, S.CLOSE], [(1, 1), (30, 5), (7, 29)])
    assert oracle_lib.exact_coverage(tri, 0).sum() == pytest.approx(394.0, abs=1e-9)


def test_fill_rules_union_and_parity(oracle_lib):
    sq = [(2, 2), (10, 2), (10, 10), (2, 10)]
    twice = [S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE] * 2
    nz = oracle_lib.exact_coverage(_one(twice, sq + sq), 0)
    eo = oracle_lib.exact_coverage(_one(twice, sq + sq, even_odd=True), 0)
    assert nz.sum() == pytest.approx(64.0) and eo.sum() == pytest.approx(0.0, abs=1e-9)
    # a pentagram: the centre has winding 2 -- covered by nonzero, not even-odd
    star = [(16, 1), (25, 29), (2, 11), (30, 11), (7, 29)]
    v = [S.MOVE] + [S.LINE] * 4 + [S.CLOSE]
    nzs = oracle_lib.exact_coverage(_one(v, star), 0)
    eos = oracle_lib.exact_coverage(_one(v, star, even_odd=True), 0)
    assert nzs[16, 16] == 1.0 and eos[16, 16] == 0.0
    assert nzs.sum() > eos.sum() > 0


def test_curves_converge(oracle_lib):
    # flattening within tol moves the area by at most (2/3) * tol * curve
    # length (each chord cuts off a parabolic segment of area
    # (2/3) * chord * sagitta); the curves here are under 150 px long
    q = _one([S.MOVE, S.QUAD, S.QUAD, S.CLOSE], [(2, 16), (16, -10), (30, 16), (16, 42), (2, 16)])
    a = oracle_lib.exact_coverage(q, 0, tol=1e-2).sum()
    b = oracle_lib.exact_coverage(q, 0, tol=1e-5).sum()
    assert abs(a - b) < (2 / 3) * 1e-2 * 150


def test_reference_coverage_error_report(oracle_lib):
    """Max and mean |reference coverage - exact area| (1/255 units) over the
    fills of a seeded 128x128 scene: the fixed-point AAA is close on average
    and bounded everywhere."""
    sc = S.random_paths_scene(S.SEED_BASE + 900, 128, 128, 24, 3, 32)
    cs = oracle_lib.coverage_scenes(sc)
    alphas = [oracle_lib.render(s)[0][..., 3] for _, s in cs]
    rep = oracle_lib.coverage_error(sc, alphas)
    print("reference coverage error:", rep)
    assert rep["pixels"] > 0 and rep["edge_pixels"] > 0
    assert rep["mean_err_255"] < 8.0
    assert rep["max_err_255"] <= 255.0
