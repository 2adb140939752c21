"""SKP import (skity_gb300/skp.py) against the reference's own IO module:
the tiger picture of the reference's resources read by the importer,
rendered by the oracle, equals the reference's playback of the file
(oracle/_ref/ref_skp) pixel for pixel.  The committed fixtures (the
imported stream and the reference pixels' digest, tests/golden/
make_skp_golden.py) carry the check to machines without the checkout."""
import gzip
import hashlib
import json
import os

import numpy as np
import pytest

from skity_gb300 import scene as S
from skity_gb300 import skp

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def fixture():
    with gzip.open(os.path.join(GOLDEN, "tiger_scene.bin.gz"), "rb") as f:
        stream = f.read()
    want = json.load(open(os.path.join(GOLDEN, "skp_digests.json")))["tiger"]
    return stream, want


def test_fixture_renders_like_the_reference_playback(oracle_lib):
    stream, want = fixture()
    assert hashlib.sha256(stream).hexdigest() == want["stream_sha256"]
    sc = S.Scene.from_bytes(stream)
    assert (sc.width, sc.height) == (want["width"], want["height"]) and sc.n_draws == 305
    got, _ = oracle_lib.render(sc)
    assert hashlib.sha256(got.tobytes()).hexdigest() == want["pixels_sha256"]


def _skp(name):
    from oracle import oracle
    p = os.path.join(oracle.REFERENCE_SRC, "resources", "skp", name)
    if not os.path.exists(p):
        pytest.skip("reference checkout not present")
    return p


def test_importer_reproduces_fixture_and_reference(oracle_lib):
    path = _skp("tiger.skp")
    data = open(path, "rb").read()
    stream, want = fixture()
    assert hashlib.sha256(data).hexdigest() == want["skp_sha256"]
    assert skp.to_display_list(data).to_stream() == stream
    try:
        oracle_lib.build_reference()
    except RuntimeError as e:
        pytest.skip(f"reference build failed: {e}")
    ref = oracle_lib.render_reference_skp(path)
    assert hashlib.sha256(ref.tobytes()).hexdigest() == want["pixels_sha256"]


def test_pictures_with_text_are_refused():
    """A picture with typefaces (text) is refused by name, not drawn in part."""
    data = open(_skp("flutter_01.skp"), "rb").read()
    with pytest.raises(skp.SkpError, match="typefaces"):
        skp.load(data)


def test_malformed_pictures_are_refused():
    with pytest.raises(skp.SkpError):
        skp.load(b"not a picture at all")
    stream, _ = fixture()
    head = b"skiapict" + (109).to_bytes(4, "little") + np.zeros(4, np.float32).tobytes() + b"\1"
    with pytest.raises(skp.SkpError):
        skp.load(head)  # no tags: truncated
    with pytest.raises(skp.SkpError, match="version"):
        skp.load(b"skiapict" + (200).to_bytes(4, "little") + bytes(17))
