"""Canvas::DrawOval / DrawCircle / DrawRect in the Python mirror: the paths
they draw are the reference's (RRect::SetOval + Path::AddRRect), point for
point, against the reference build (oracle/_ref/ref_shapes); CPU only."""
import os
import subprocess

import numpy as np
import pytest

from skity_gb300 import scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SHAPES = os.path.join(ROOT, "oracle", "_ref", "ref_shapes")


def _ref(args):
    out = subprocess.check_output([REF_SHAPES] + args, text=True).splitlines()
    verbs = [int(v) for v in out[0].split()[1:]]
    pts = np.array([float.fromhex(v) for v in out[1].split()[1:]], np.float32).reshape(-1, 2)
    wts = np.array([float.fromhex(v) for v in out[2].split()[1:]], np.float32)
    return verbs, pts, wts


def _mine(path):
    return (list(path.verbs), np.asarray(path.points, np.float32).reshape(-1, 2),
            np.asarray(path.weights, np.float32))


@pytest.fixture(scope="module")
def ref_shapes(oracle_lib):
    oracle_lib.build_reference()
    if not os.path.exists(REF_SHAPES):
        pytest.skip("reference build not present")
    return REF_SHAPES


def test_ovals_and_circles_match_reference(ref_shapes):
    from skity_gb300.canvas import Path
    rng = np.random.default_rng(0x0FA1)
    f = np.float32
    cases = [("o", (10.0, 20.0, 50.5, 44.0)), ("o", (50.0, 40.0, 10.0, 5.0)),
             ("o", (3.0, 3.0, 3.0, 9.0)), ("o", (0.0, 0.0, 0.0, 0.0)),
             ("c", (30.0, 30.0, 0.0)), ("c", (12.5, 7.25, -3.0)), ("c", (100.0, 50.0, 1e-3))]
    for _ in range(40):
        if rng.random() < 0.5:
            cases.append(("o", tuple(float(f(v)) for v in rng.uniform(-300, 300, 4))))
        else:
            cases.append(("c", tuple(float(f(v)) for v in
                                     (*rng.uniform(-300, 300, 2), rng.uniform(-5, 200)))))
    for kind, a in cases:
        want = _ref([kind] + [float(v).hex() for v in a])
        if kind == "o":
            got = _mine(Path().AddOvalRRect(*a))
        else:
            cx, cy, r = (f(v) for v in a)
            r = max(r, f(0))
            got = _mine(Path().AddOvalRRect(cx - r, cy - r, cx + r, cy + r))
        assert got[0] == want[0], (kind, a)
        assert got[1].tobytes() == want[1].tobytes(), (kind, a)
        assert got[2].tobytes() == want[2].tobytes(), (kind, a)


def test_draw_oval_circle_rect_record_their_paths(oracle_lib):
    """The canvas calls record those paths as DrawPath does."""
    from skity_gb300.canvas import Paint, Path, PictureRecorder
    r = PictureRecorder()
    cv = r.BeginRecording((0, 0, 96, 80))
    cv.Clear((1.0, 1.0, 1.0, 1.0))
    cv.DrawOval(10, 8, 70, 50, Paint().SetColor(0xFFC03060))
    cv.DrawCircle(48, 40, 20.5, Paint().SetStyle(1).SetStrokeWidth(3).SetColor(0xFF3060C0))
    cv.DrawRect(5, 60, 90, 75, Paint().SetColor(0xFF20A040))
    sc = r.FinishRecording().to_scene()
    assert sc.n_draws == 3
    b = S.SceneBuilder(96, 80)
    for path, paint in ((Path().AddOvalRRect(10, 8, 70, 50), Paint().SetColor(0xFFC03060)),
                        (Path().AddOvalRRect(27.5, 19.5, 68.5, 60.5),
                         Paint().SetStyle(1).SetStrokeWidth(3).SetColor(0xFF3060C0)),
                        (Path().AddRect(5, 60, 90, 75), Paint().SetColor(0xFF20A040))):
        b.draw_path(path.verbs, path.points, paint.rec, path.weights)
    got, _ = oracle_lib.render(sc)
    want, _ = oracle_lib.render(b.build())
    assert np.array_equal(got, want)
    assert (got != 255).any()
