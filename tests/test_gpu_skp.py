"""The imported tiger picture (tests/golden/tiger_scene.bin.gz, made by
skity_gb300/skp.py from the reference's resources) rendered on the GPU
through the C ABI: bit-exact with the reference's own playback of the SKP
(pixel digest), alone and in a batch with other canvases."""
import hashlib

import pytest

from skity_gb300 import scene as S

pytestmark = pytest.mark.gpu


def test_tiger_matches_reference_playback(gpu_ctx):
    from test_skp import fixture
    stream, want = fixture()
    sc = S.Scene.from_bytes(stream)
    others = list(S.config3(n_canvases=6, scale=0.3))
    outs = gpu_ctx.render_streams([others[0], sc] + others[1:])
    assert hashlib.sha256(outs[1].tobytes()).hexdigest() == want["pixels_sha256"]
