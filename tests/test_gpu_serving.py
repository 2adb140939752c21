"""The serving loop (skity_cuda_server_*) through the C ABI: requests that
arrive while others are in flight land in different, overlapping batches,
and every request's pixels are the same as rendering it alone and as the
oracle's (bar: <= 1 LSB per channel, >= 99.9% exact; bit-exact expected)."""
import threading

import numpy as np
import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999


def _requests(n):
    R = S.random_streams(S.SEED_BASE + 500, n, 3)
    out = []
    for i in range(n):
        side_w = int(round(float(S.loguniform(R[i, 0], 48, 320))))
        side_h = int(round(float(S.loguniform(R[i, 1], 48, 320))))
        paths = int(round(float(S.loguniform(R[i, 2], 3, 120))))
        out.append(S.random_paths_scene(S.SEED_BASE + 600 + i, side_w, side_h, paths, 3, 32))
    return out


def _check(got, want):
    d = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=-1)
    assert int(d.max()) <= TOL_LSB and float((d == 0).mean()) >= MIN_EXACT


def test_results_same_alone_and_in_the_mix(gpu_ctx, oracle_lib):
    from skity_gb300.canvas import Server
    reqs = _requests(24)
    alone = [gpu_ctx.render_streams([sc])[0] for sc in reqs]
    srv = Server(0, workers=2, max_batch=8)
    tickets = [None] * len(reqs)

    def producer(idx):
        for i in idx:
            tickets[i] = srv.submit(reqs[i])

    th = [threading.Thread(target=producer, args=(range(k, len(reqs), 3),)) for k in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    batch_sizes = []
    for i, t in enumerate(tickets):
        px, info = srv.wait(t)
        assert px is not None
        batch_sizes.append(info["batch_size"])
        _check(px, alone[i])
        want, _ = oracle_lib.render(reqs[i])
        _check(px, want)
    srv.close()
    assert max(batch_sizes) > 1  # requests shared batches


def test_admission_refuses_oversized_and_poll(gpu_ctx):
    from skity_gb300 import _lib
    from skity_gb300.canvas import Server
    srv = Server(0, budget_bytes=8 << 20, workers=1)
    big = S.random_paths_scene(S.SEED_BASE + 700, 2048, 2048, 4, 3, 8)
    with pytest.raises(_lib.SkityCudaError) as e:
        srv.submit(big)
    assert e.value.code == -7
    small = S.random_paths_scene(S.SEED_BASE + 701, 64, 64, 4, 3, 8)
    t = srv.submit(small)
    px, info = srv.wait(t)
    assert px is not None and info["latency_ms"] >= info["queue_ms"] >= 0
    with pytest.raises(_lib.SkityCudaError):
        srv.wait(t)  # released
    srv.close()
