"""The coverage-error report (FP64 exact area, oracle/exact_area.cc) for the
CUDA path: every fill of a seeded scene rendered alone through the C ABI
(opaque white on transparent, one canvas per draw in one batch); its max and
mean error against true area must equal the reference rasteriser's (the
oracle's), since the pixels are bit-exact."""
import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu


def test_gpu_coverage_error_matches_reference(gpu_ctx, oracle_lib):
    sc = S.random_paths_scene(S.SEED_BASE + 901, 160, 128, 30, 3, 32, evenodd_frac=0.5)
    cs = oracle_lib.coverage_scenes(sc)
    gpu = gpu_ctx.render_streams([s for _, s in cs])
    ref = [oracle_lib.render(s)[0] for _, s in cs]
    for g, r in zip(gpu, ref):
        assert np.array_equal(g, r)
    rg = oracle_lib.coverage_error(sc, [g[..., 3] for g in gpu])
    rr = oracle_lib.coverage_error(sc, [r[..., 3] for r in ref])
    print("coverage error vs exact area: gpu", rg, "reference", rr)
    assert rg == rr
