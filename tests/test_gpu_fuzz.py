"""Parity sweep on the GPU: seeded scenes of every feature family
(tests/fuzz_scenes.py: canvas matrices, clip rects, path clips, layers,
blend modes, gradient kinds, colour filters, image shaders, mixed fills and
strokes) rendered in one batch through the C ABI, each against the oracle.
Bar: <= 1 LSB per channel and >= 99.9% exact (bit-exact expected)."""
import pytest

from fuzz_scenes import families

pytestmark = pytest.mark.gpu
TOL_LSB, MIN_EXACT = 1, 0.999


def test_feature_families_match_oracle(gpu_ctx, oracle_lib):
    cases = families(12)
    outs = gpu_ctx.render_streams([sc for _, sc in cases])
    bad = []
    for (name, sc), got in zip(cases, outs):
        ref, _ = oracle_lib.render(sc)
        c = oracle_lib.compare(got, ref)
        if not (c["max_abs_diff"] <= TOL_LSB and c["exact_frac"] >= MIN_EXACT) or c["bad_pixels"]:
            bad.append((name, sc.width, sc.height, c))
    assert not bad, bad
