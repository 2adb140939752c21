"""A recorded display list on the GPU: DisplayList::Draw onto a CUDA canvas,
its scene stream through the batched form and through the serving loop --
each against the oracle's render of the recorded scene.  Bar: <= 1 LSB per
channel and >= 99.9% of pixels exact (bit-exact expected)."""
import numpy as np
import pytest

from skity_gb300 import scene as S
from test_display_list import _record, scene_ops

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999


def _check(oracle_lib, got, ref):
    c = oracle_lib.compare(got, ref)
    assert c["max_abs_diff"] <= TOL_LSB and c["exact_frac"] >= MIN_EXACT, c
    return c


def test_display_list_draw_batch_and_server(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Batch, Canvas, Server
    dl = _record(scene_ops)
    sc = dl.to_scene()
    ref, _ = oracle_lib.render(sc)
    # DisplayList::Draw onto a CUDA canvas, then Flush
    bitmap = np.zeros((sc.height, sc.width, 4), np.uint8)
    cv = Canvas.MakeCUDACanvas(gpu_ctx, bitmap)
    dl.Draw(cv)
    cv.Flush()
    assert _check(oracle_lib, bitmap, ref)["bad_pixels"] == 0
    # the scene stream in a batch with other canvases
    b = Batch(gpu_ctx, [S.config1(n_paths=50), sc])
    b.render()
    assert _check(oracle_lib, b.read(1), ref)["bad_pixels"] == 0
    b.close()
    # and submitted to the serving loop
    srv = Server(0, workers=1, max_batch=4)
    t = srv.submit(stream=dl.to_stream())
    px, info = srv.wait(t, 60000)
    srv.close()
    assert _check(oracle_lib, px, ref)["bad_pixels"] == 0
