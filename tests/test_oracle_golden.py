"""The oracle against the golden fixtures made by the reference's own
software backend (tests/golden/make_golden.py), and the fixtures against the
exact-pixel assertions of the reference's unit tests.  CPU only."""
import json
import os
import sys

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import golden_scenes as G  # noqa: E402

DIGESTS = json.load(open(os.path.join(GOLDEN, "digests.json")))
PIXELS = np.load(os.path.join(GOLDEN, "pixels.npz"))


@pytest.mark.parametrize("name", sorted(G.PIXEL_SCENES) + sorted(G.DIGEST_SCENES))
def test_scene_generator_is_stable(name):
    make = G.PIXEL_SCENES.get(name) or G.DIGEST_SCENES[name]
    assert G.scene_digest(make()) == DIGESTS[name]["scene_sha256"]


@pytest.mark.parametrize("name", sorted(G.PIXEL_SCENES))
def test_oracle_matches_golden_pixels(oracle_lib, name):
    got, _ = oracle_lib.render(G.PIXEL_SCENES[name]())
    want = PIXELS[name]
    assert got.shape == want.shape
    c = oracle_lib.compare(got, want)
    assert c["bad_pixels"] == 0, c


@pytest.mark.parametrize("name", sorted(G.DIGEST_SCENES))
def test_oracle_matches_golden_digests(oracle_lib, name):
    got, _ = oracle_lib.render(G.DIGEST_SCENES[name]())
    assert G.pixel_digest(got) == DIGESTS[name]["pixels_sha256"]


def test_golden_holds_reference_unit_test_answers():
    # sw_canvas_test.cc:83-84: GetPixel(12,20) == Color_WHITE, (7,20) == Color_RED
    st = PIXELS["stroke_then_fill"]
    assert tuple(st[20, 12]) == (255, 255, 255, 255)
    assert tuple(st[20, 7]) == (255, 0, 0, 255)
    # color_test.cc:44-51: Color4fToColor({-0.5, 1.5, 0.7, 0.2}) = ARGB(51, 0, 255, 178);
    # premultiplied with MulDiv255Round: (0, 51, 36, 51) as RGBA bytes
    ct = PIXELS["color_truncation"]
    assert (ct.reshape(-1, 4) == np.array([0, 51, 36, 51], np.uint8)).all()
