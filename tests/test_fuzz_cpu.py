"""Parity sweep on the CPU: the device code's CPU build (tests/cpu_pipeline.cc)
against the oracle on seeded scenes of every feature family
(tests/fuzz_scenes.py), bit-exact."""
import pytest

from fuzz_scenes import families
from test_cpu_pipeline import cpu_render


@pytest.mark.parametrize("k", range(3))
def test_feature_families_bit_exact(cpu_pipeline, oracle_lib, k):
    for name, sc in families(3)[9 * k:9 * k + 9]:
        got, _ = cpu_render(cpu_pipeline, sc)
        ref, _ = oracle_lib.render(sc)
        c = oracle_lib.compare(got, ref)
        assert c["bad_pixels"] == 0, (name, sc.width, sc.height, c)
