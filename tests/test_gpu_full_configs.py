"""GPU parity at the timed sizes: the full 2048x2048 scene (20,000 paths),
all 256 canvases of the batching workload and the full 4096x4096 glyph-dense
scene with blur, each rendered as the bench renders it (a resident batch
replayed from its CUDA graphs) and checked against the oracle.

The oracle's pixels of these workloads are committed as SHA-256 digests
(tests/golden/full_digests.json, written by tests/golden/make_full_digests.py);
a render whose digest matches is bit-exact.  On a mismatch the oracle renders
the workload on every host core and the bar is applied to the difference:
<= 1 LSB per channel and >= 99.9% of pixels exact."""
import hashlib
import json
import os

import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999
HERE = os.path.dirname(os.path.abspath(__file__))


def _digests(name):
    with open(os.path.join(HERE, "golden", "full_digests.json")) as f:
        return json.load(f)[name]


def _check(oracle_lib, name, scenes, got):
    want = _digests(name)
    assert len(want) == len(got)
    mismatched = [i for i, g in enumerate(got)
                  if hashlib.sha256(g.tobytes()).hexdigest() != want[i]]
    if not mismatched:
        return
    threads = os.cpu_count() or 1
    worst, bad, px = 0, 0, 0
    for i in mismatched:
        ref, _ = oracle_lib.render_mt(scenes[i], threads)
        c = oracle_lib.compare(got[i], ref)
        worst = max(worst, c["max_abs_diff"])
        bad += c["bad_pixels"]
    px = sum(g.shape[0] * g.shape[1] for g in got)
    exact = 1.0 - bad / px
    assert worst <= TOL_LSB and exact >= MIN_EXACT, (name, worst, exact, len(mismatched))


def _render(gpu_ctx, scenes):
    from skity_gb300.canvas import Batch
    b = Batch(gpu_ctx, scenes)
    b.render()   # planned render (capacities found, replay graphs recorded)
    st = b.render()  # graph replay, as the bench times it
    assert st["graph_replays"] == 1 and st["host_syncs"] == 1
    got = [b.read(i) for i in range(len(scenes))]
    b.close()
    return got


def test_config2_full(gpu_ctx, oracle_lib):
    scenes = [S.config2()]
    _check(oracle_lib, "config2", scenes, _render(gpu_ctx, scenes))


def test_config3_all_canvases(gpu_ctx, oracle_lib):
    scenes = S.config3()
    _check(oracle_lib, "config3", scenes, _render(gpu_ctx, scenes))


def test_config4_full(gpu_ctx, oracle_lib):
    scenes = [S.config4()]
    _check(oracle_lib, "config4", scenes, _render(gpu_ctx, scenes))


def test_config1_full_end_to_end(gpu_ctx, oracle_lib):
    """The 512x512 scene through skity_cuda_render_streams (host buffers in
    and out, one call)."""
    scenes = [S.config1()]
    _check(oracle_lib, "config1", scenes, gpu_ctx.render_streams(scenes))
