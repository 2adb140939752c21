"""The plain per-draw form (skity_cuda_batch_render_per_draw): every DrawPath
rasterised and blended on its own, against the batched render of the same
batch and against the oracle.  Bar: <= 1 LSB per channel and >= 99.9% of
pixels exact (bit-exact expected: the same kernels run)."""
import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999


def _check(oracle_lib, got, sc):
    ref, _ = oracle_lib.render(sc)
    c = oracle_lib.compare(got, ref)
    assert c["max_abs_diff"] <= TOL_LSB and c["exact_frac"] >= MIN_EXACT, c


def test_per_draw_matches_batched_and_oracle(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Batch
    scenes = S.config3(n_canvases=10, scale=0.25) + [S.config2(n_paths=300, width=512, height=384)]
    b = Batch(gpu_ctx, scenes)
    b.render()
    batched = [b.read(i) for i in range(len(scenes))]
    st = b.render_per_draw()
    assert st["host_syncs"] == 1
    assert st["kernel_launches"] >= 7 * sum(sc.n_draws for sc in scenes)
    for i, sc in enumerate(scenes):
        got = b.read(i)
        assert np.array_equal(got, batched[i])
        _check(oracle_lib, got, sc)
    b.close()


def test_per_draw_rejects_blur(gpu_ctx):
    """Blur mask filters need the batch's temp canvases: not taken."""
    from skity_gb300.canvas import Batch
    from skity_gb300 import _lib
    sc = S.config4(n_outlines=50, width=256, height=256, blur_frac=0.5)
    b = Batch(gpu_ctx, [sc])
    with pytest.raises(_lib.SkityCudaError) as e:
        b.render_per_draw()
    assert e.value.code == -5
    b.close()
