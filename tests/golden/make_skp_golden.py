"""Writes the SKP-import fixtures of tests/golden from the reference
checkout's resources/skp/tiger.skp: the scene stream the importer
(skity_gb300/skp.py) makes of it, and the SHA-256 of the pixels the
reference's own IO module plays it back to (oracle/_ref/ref_skp).  Needs the
reference checkout; run from the repo root:

    python tests/golden/make_skp_golden.py

Outputs: tests/golden/tiger_scene.bin.gz (the stream, gzip) and
tests/golden/skp_digests.json.
"""
from __future__ import annotations

import gzip
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402
from skity_gb300 import skp  # noqa: E402

TIGER = os.path.join(oracle.REFERENCE_SRC, "resources", "skp", "tiger.skp")


def main():
    if not oracle.build_reference():
        sys.exit("the reference checkout is needed to generate the SKP fixtures")
    data = open(TIGER, "rb").read()
    stream = skp.to_display_list(data).to_stream()
    px = oracle.render_reference_skp(TIGER)
    with gzip.open(os.path.join(HERE, "tiger_scene.bin.gz"), "wb", compresslevel=9) as f:
        f.write(stream)
    out = {"tiger": {"skp_sha256": hashlib.sha256(data).hexdigest(),
                     "stream_sha256": hashlib.sha256(stream).hexdigest(),
                     "pixels_sha256": hashlib.sha256(px.tobytes()).hexdigest(),
                     "width": int(px.shape[1]), "height": int(px.shape[0])}}
    with open(os.path.join(HERE, "skp_digests.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(out)


if __name__ == "__main__":
    main()
