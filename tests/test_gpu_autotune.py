"""Raster configurations (compositor tile width, persistent CTAs per SM,
pass-bin band height, register-sweep warps per CTA) change the time, never
the pixels; the autotuner
picks one from its space and persists it."""
import os

import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu


def test_every_config_gives_the_same_pixels(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Batch
    scenes = S.config3(n_canvases=6, scale=0.15)
    scenes.append(S.config4(n_outlines=300, width=300, height=200, blur_frac=0.3))
    refs = [oracle_lib.render(sc)[0] for sc in scenes]
    b = Batch(gpu_ctx, scenes)
    for cfg in [dict(tile_width=64, ctas_per_sm=1, band_rows=8, sweep_warps=1),
                dict(tile_width=512, ctas_per_sm=0, band_rows=64, sweep_warps=4),
                dict(tile_width=128, ctas_per_sm=2, band_rows=32, sweep_warps=2),
                dict(tile_width=256, ctas_per_sm=4, band_rows=16, sweep_warps=4)]:
        b.set_config(**cfg)
        assert b.config() == cfg
        for _ in range(2):  # planned render, then a graph replay
            b.render()
            for i, ref in enumerate(refs):
                assert np.array_equal(b.read(i), ref), (cfg, i)
    b.close()


def test_autotune_picks_and_persists(gpu_ctx, tmp_path, monkeypatch):
    from skity_gb300 import autotune
    from skity_gb300.canvas import Batch
    monkeypatch.setenv("SKITY_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    scenes = S.config3(n_canvases=4, scale=0.1)
    b = Batch(gpu_ctx, scenes)
    key = autotune.signature(scenes, "test")
    r = autotune.tune(b, key, reps=1)
    assert not r["cached"] and r["config"]["tile_width"] in autotune.TILE_WIDTHS
    assert r["config"]["sweep_warps"] in autotune.SWEEP_WARPS
    assert b.config() == r["config"]
    assert os.path.exists(tmp_path / "tune.json")
    again = autotune.tune(b, key)
    assert again["cached"] and again["config"] == r["config"]
    b.close()


def test_invalid_config_rejected(gpu_ctx):
    from skity_gb300 import _lib
    from skity_gb300.canvas import Batch
    b = Batch(gpu_ctx, S.config3(n_canvases=1, scale=0.05))
    for bad in [dict(tile_width=16), dict(band_rows=12), dict(ctas_per_sm=1000),
                dict(sweep_warps=3)]:
        with pytest.raises(_lib.SkityCudaError):
            b.set_config(**bad)
    b.close()
