"""Autotuner of the raster launch shapes for a resident batch.

The pixels never depend on the configuration (skity_cuda_raster_config);
only the time does.  The searched space:

* row-tile width in pixels {128, 256, 512, 1024, 2048} -- the compositor gives each
  warp one canvas row segment, so a tile is (width x 1 row) and its width,
  a multiple of the 32 lanes, is the shape parameter;
* persistent CTAs per SM {1, 2, 4, 6, 8} (the grid is that many CTAs per SM,
  pulling tiles from a work counter in most-work-first order);
* pass-bin granularity: bands of {8, 16, 32} rows;
* warps per CTA of the register-resident AAA sweeps {1, 2, 4} (one pass a
  warp; fewer warps a CTA spread a batch's few long passes over more SMs,
  more warps share one CTA's launch and shared-memory carve-out).

Tile width x CTAs per SM are swept together on the compositing time, then
the band height with the best pair on the same time, then the sweep's warps
on the whole render's device time.  Each point re-plans the batch (one
planned render), then times `reps` CUDA-graph replays and keeps the fastest.
Results
persist as JSON keyed by a workload signature, in the file named by
SKITY_GB300_TUNE_CACHE (default ~/.cache/skity_gb300/autotune.json).
"""
from __future__ import annotations

import json
import os

TILE_WIDTHS = (128, 256, 512, 1024, 2048)
CTAS_PER_SM = (1, 2, 4, 6, 8)
BAND_ROWS = (8, 16, 32)
SWEEP_WARPS = (1, 2, 4)


def cache_path() -> str:
    return os.environ.get("SKITY_GB300_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "skity_gb300",
                                       "autotune.json"))


def signature(scenes, device_name: str = "") -> str:
    """Workload key: canvas count, pixels and draws, rounded, plus the device."""
    px = sum(s.width * s.height for s in scenes)
    draws = sum(s.n_draws for s in scenes)
    return f"canvases={len(scenes)};mpix={px / 1e6:.1f};draws={draws};dev={device_name}"


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(d: dict) -> None:
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        with open(p, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
    except OSError:
        pass


def _time(batch, cfg: dict, reps: int, key: str = "composite_ms") -> float:
    batch.set_config(**cfg)
    batch.render()  # plan + record the replay graphs
    return min(batch.render()[key] for _ in range(reps))


def tune(batch, key: str, reps: int = 3, use_cache: bool = True) -> dict:
    """Finds (or loads) the fastest configuration for `batch`, applies it and
    returns {"config": ..., "composite_ms": ..., "trials": [...], "cached": bool}."""
    cache = _load() if use_cache else {}
    if key in cache:
        ent = cache[key]
        batch.set_config(**ent["config"])
        return dict(ent, cached=True)
    trials = []
    for tw in TILE_WIDTHS:
        for ctas in CTAS_PER_SM:
            cfg = {"tile_width": tw, "ctas_per_sm": ctas, "band_rows": 16, "sweep_warps": 2}
            trials.append((_time(batch, cfg, reps), cfg))
    best_ms, best = min(trials, key=lambda t: t[0])
    for rows in BAND_ROWS:
        if rows == best["band_rows"]:
            continue
        cfg = dict(best, band_rows=rows)
        ms = _time(batch, cfg, reps)
        trials.append((ms, cfg))
        if ms < best_ms:
            best_ms, best = ms, cfg
    sweeps = []
    for warps in SWEEP_WARPS:
        cfg = dict(best, sweep_warps=warps)
        sweeps.append((_time(batch, cfg, reps, "device_ms"), cfg))
    best_dev, best = min(sweeps, key=lambda t: t[0])
    batch.set_config(**best)
    ent = {"config": best, "composite_ms": best_ms, "device_ms": best_dev,
           "trials": [{"composite_ms": ms, **c} for ms, c in trials]
           + [{"device_ms": ms, **c} for ms, c in sweeps]}
    if use_cache:
        cache = _load()
        cache[key] = ent
        _store(cache)
    return dict(ent, cached=False)
