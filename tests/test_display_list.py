"""PictureRecorder / DisplayList (the reference's src/recorder): calls made on
a recorder's canvas replay, through DisplayList::Draw, the way they were
made -- on a CUDA canvas, or written as a scene stream for the batched and
serving forms.  CPU: the recorded scene against the same calls made on a
scene builder, rendered by the oracle (and by the reference build where it
exists).  The GPU half is in test_gpu_display_list.py."""
import numpy as np
import pytest

from skity_gb300 import scene as S


def _record(rec_canvas_ops):
    from skity_gb300.canvas import PictureRecorder
    r = PictureRecorder()
    cv = r.BeginRecording((0, 0, 144, 112))
    rec_canvas_ops(cv)
    return r.FinishRecording()


def scene_ops(cv):
    """A scene of every recorded call: Clear, fills and strokes with a
    gradient, Save / Translate / ClipRect / Restore, a layer, a path clip."""
    from skity_gb300.canvas import Paint, Path, Shader
    cv.Clear((1.0, 1.0, 1.0, 1.0))
    tri = Path().MoveTo(10, 10).LineTo(130, 25).QuadTo(90, 120, 20, 100).Close()
    cub = Path().MoveTo(5, 60).CubicTo(40, -10, 100, 130, 140, 50).LineTo(70, 105).Close()
    cv.DrawPath(tri, Paint().SetColor(0xFF3060C0).SetAlphaF(0.7))
    cv.Save()
    cv.Translate(6.5, -4.25)
    cv.ClipRect(0, 8, 120, 90)
    g = Shader.MakeLinear([(0, 0), (140, 110)], [(1, 0, 0, 1), (0, 0, 1, 1)], None, 2)
    cv.DrawPath(cub, Paint().SetShader(g))
    cv.SaveLayer((12.5, 9.75, 100.25, 80.5), Paint().SetAlphaF(0.5))
    cv.DrawPath(tri, Paint().SetColor(0xFF20A040))
    cv.Restore()
    cv.Restore()
    cv.ClipPath(Path().MoveTo(0, 0).LineTo(144, 0).LineTo(0, 112).Close(), 1)
    p = Paint().SetColor(0xC0C02020)
    p.SetStyle(1)
    p.SetStrokeWidth(5)
    cv.DrawPath(cub, p)


def test_recorded_ops_and_stream(oracle_lib):
    dl = _record(scene_ops)
    assert dl.GetOpCount() == 12
    sc = dl.to_scene()
    assert sc.width == 144 and sc.height == 112 and sc.n_draws == 4
    assert sc.layers is not None and len(sc.layers) == 1 and sc.path_clips is not None
    # the same display list replayed onto another recorder records the same scene
    from skity_gb300.canvas import PictureRecorder
    r = PictureRecorder()
    dl.Draw(r.BeginRecording((0, 0, 144, 112)))
    again = r.FinishRecording()
    assert again.GetOpCount() == dl.GetOpCount()
    assert again.to_stream() == dl.to_stream()
    got, _ = oracle_lib.render(sc)
    assert int(got[..., 3].min()) == 255 and len(np.unique(got.reshape(-1, 4), axis=0)) > 50


def test_stream_matches_reference(oracle_lib):
    """The display list's scene, replayed by the reference's own software
    backend (oracle/_ref), equals the oracle's render of it."""
    try:
        ok = oracle_lib.build_reference()
    except RuntimeError as e:
        pytest.skip(f"reference build failed: {e}")
    if not ok and not oracle_lib.reference_available():
        pytest.skip("reference checkout not present")
    sc = _record(scene_ops).to_scene()
    want = oracle_lib.render_reference(sc)
    got, _ = oracle_lib.render(sc)
    assert oracle_lib.compare(got, want)["bad_pixels"] == 0


def test_recorded_transforms_write_matrices(oracle_lib):
    """Scale / Rotate / Skew / Concat / SetMatrix are recorded and replayed:
    the scene gets each draw's canvas matrix, the one the reference's own
    Canvas computes for the same calls (oracle/_ref/ref_matrix, where the
    reference build exists)."""
    import os
    import subprocess
    from skity_gb300.canvas import Paint, Path
    tri = Path().MoveTo(10, 10).LineTo(60, 20).LineTo(20, 70).Close()
    calls = [("t", (12.0, 7.5)), ("s", (1.25, 0.8)), ("r", (33.0, 20.0, 10.0)),
             ("k", (0.2, -0.15)), ("c", (0.9, 0.1, 5.0, -0.2, 1.1, -3.0, 0.0, 0.0, 1.0))]

    def ops(cv):
        cv.Clear((1.0, 1.0, 1.0, 1.0))
        for name, a in calls:
            {"t": cv.Translate, "s": cv.Scale, "r": cv.Rotate, "k": cv.Skew}.get(
                name, lambda *v: cv.Concat(v))(*a)
            cv.DrawPath(tri, Paint().SetColor(0xFF3060C0).SetAlphaF(0.7))
        cv.SetMatrix((2.0, 0.0, 1.0, 0.0, 2.0, 1.0, 0.0, 0.0, 1.0))
        cv.DrawPath(tri, Paint().SetColor(0xFF20A040))
    dl = _record(ops)
    sc = dl.to_scene()
    assert sc.matrices is not None and sc.matrices.shape == (6, 6)
    assert (sc.paints["translate"] == 0).all()
    assert tuple(sc.matrices[5]) == (2.0, 0.0, 1.0, 0.0, 2.0, 1.0)
    got, _ = oracle_lib.render(sc)
    assert len(np.unique(got.reshape(-1, 4), axis=0)) > 20
    ref_matrix = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                              "oracle", "_ref", "ref_matrix")
    if not os.path.exists(ref_matrix):
        return
    args = []
    for k, (name, a) in enumerate(calls):
        args += [name] + [float(np.float32(v)).hex() for v in a]
        out = subprocess.check_output([ref_matrix] + args, text=True).split()
        want = np.array([float.fromhex(v) for v in out], np.float32)
        assert want[[0, 1, 2, 3, 4, 5]].tobytes() == sc.matrices[k].tobytes(), k


def test_recorded_clips_under_matrices(oracle_lib):
    """ClipRect under a rotation becomes a kIntersect path clip of the rect
    (Path::AddRect) under that matrix, after the global clip bounds narrow
    to the rotated rect's bounds; ClipPath under a scale keeps its matrix;
    the draws carry the narrowed bounds.  The recorded scene renders as the
    same calls made on a scene builder (the oracle is pinned to the
    reference for these cases)."""
    from skity_gb300.canvas import Paint, Path
    blob = Path().MoveTo(5, 5).QuadTo(40, 0, 35, 20).CubicTo(30, 40, 10, 45, 3, 30).Close()

    def ops(cv):
        cv.Clear((1.0, 1.0, 1.0, 1.0))
        cv.Save()
        cv.Rotate(20, 60, 48)
        cv.ClipRect(20, 15, 100, 80)
        cv.DrawPath(blob, Paint().SetColor(0xFFC03060))
        cv.Restore()
        cv.Scale(2.0, 1.5)
        cv.ClipPath(blob, S.CLIP_INTERSECT)
        cv.DrawPath(blob, Paint().SetColor(0xFF3060C0).SetAlphaF(0.7))
    sc = _record(ops).to_scene()
    states, _, _, _, per_draw = sc.path_clips
    assert sc.clip_matrices is not None and len(states) == 2
    rot = tuple(float(v) for v in sc.matrices[0])
    assert tuple(float(v) for v in sc.clip_matrices[0]) == rot
    assert int(states[0]["op"]) == S.CLIP_INTERSECT and int(states[0]["nv"]) == 5
    glob = S.map_clip_matrix(S.NO_CLIP, (20.0, 15.0, 100.0, 80.0), rot)
    assert tuple(float(v) for v in states[0]["bounds"]) == glob
    assert tuple(float(v) for v in sc.clips[0]) == glob
    sm = (2.0, 0.0, 0.0, 0.0, 1.5, 0.0)
    assert tuple(float(v) for v in sc.clip_matrices[1]) == sm
    pts = np.asarray(blob.points, np.float32).reshape(-1, 2)
    g2 = S.map_clip_matrix(S.NO_CLIP, (pts[:, 0].min(), pts[:, 1].min(), pts[:, 0].max(),
                                       pts[:, 1].max()), sm)
    assert tuple(float(v) for v in states[1]["bounds"]) == g2 and g2[0] == 6.0
    assert list(per_draw) == [1, 2]
    b = S.SceneBuilder(sc.width, sc.height)
    b.save()
    b.clip_path(S.RECT_VERBS, S.rect_points((20.0, 15.0, 100.0, 80.0)), S.CLIP_INTERSECT,
                bounds=glob, matrix=rot)
    b.draw_path(blob.verbs, blob.points, Paint().SetColor(0xFFC03060).rec, clip=glob,
                matrix=rot)
    b.restore()
    b.clip_path(blob.verbs, blob.points, S.CLIP_INTERSECT, bounds=g2, matrix=sm)
    b.draw_path(blob.verbs, blob.points, Paint().SetColor(0xFF3060C0).SetAlphaF(0.7).rec,
                clip=g2, matrix=sm)
    got, _ = oracle_lib.render(sc)
    want, _ = oracle_lib.render(b.build())
    assert np.array_equal(got, want)


@pytest.mark.parametrize("seed", range(12))
def test_recorded_matrices_inside_layers_match_reference(seed):
    """Translations, Save / Restore and SaveLayer in random order: the matrix
    of a draw inside a layer is the layer's world matrix times the matrix
    the calls after SaveLayer built (the reference's CanvasState layer
    states), bit for bit the reference Canvas's GetTotalMatrix
    (oracle/_ref/ref_matrix) -- not the product taken call by call."""
    import os
    import subprocess
    from skity_gb300.canvas import Paint, Path
    ref_matrix = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                              "oracle", "_ref", "ref_matrix")
    if not os.path.exists(ref_matrix):
        pytest.skip("reference build not present")
    rng = np.random.default_rng(0x1A7E + seed)
    f = np.float32
    seq, depth_layers, depth = [], 0, 0
    for _ in range(24):
        r = rng.random()
        if r < 0.45:
            seq.append(("t", (f(rng.uniform(-9, 9)), f(rng.uniform(-9, 9)))))
        elif r < 0.6:
            seq.append(("S", ()))
            depth += 1
        elif r < 0.75 and depth_layers == 0:
            seq.append(("L", (f(-50), f(-50), f(200), f(200))))
            depth += 1
            depth_layers = depth
        elif depth > 0:
            seq.append(("R", ()))
            if depth == depth_layers:
                depth_layers = 0
            depth -= 1
    tri = Path().MoveTo(10, 10).LineTo(60, 20).LineTo(20, 70).Close()

    def ops(cv):
        cv.Clear((1.0, 1.0, 1.0, 1.0))
        for name, a in seq:
            if name == "t":
                cv.Translate(float(a[0]), float(a[1]))
            elif name == "S":
                cv.Save()
            elif name == "L":
                cv.SaveLayer(tuple(float(v) for v in a), Paint())
            else:
                cv.Restore()
            cv.DrawPath(tri, Paint().SetColor(0xFF3060C0))
        for _ in range(depth):  # close what is open (a layer is drawn at its restore)
            cv.Restore()
    sc = _record(ops).to_scene()
    m = sc.matrices if sc.matrices is not None else None
    args = []
    for k, (name, a) in enumerate(seq):
        args += [name] + [float(v).hex() for v in a]
        out = subprocess.check_output([ref_matrix] + args, text=True).split()
        want = np.array([float.fromhex(v) for v in out], np.float32)
        got = (m[k][[2, 5]] if m is not None else sc.paints[k]["translate"]).astype(np.float32)
        assert want[[2, 5]].tobytes() == got.tobytes(), (k, seq[:k + 1], want, got)
