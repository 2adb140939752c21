"""Writes the golden fixtures of tests/golden from the reference software
backend compiled from the reference's own sources (oracle/ref/Makefile ->
oracle/_ref/ref_render).  Needs the reference checkout; run from the repo
root:

    python tests/golden/make_golden.py

Outputs: tests/golden/pixels.npz (premultiplied RGBA8 of PIXEL_SCENES) and
tests/golden/digests.json (scene and pixel SHA-256 of every scene).
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import golden_scenes as G  # noqa: E402
from oracle import oracle  # noqa: E402


def main():
    if not oracle.build_reference():
        sys.exit("the reference checkout is needed to generate golden fixtures")
    pixels, digests = {}, {}
    for name, make in list(G.PIXEL_SCENES.items()) + list(G.DIGEST_SCENES.items()):
        sc = make()
        px = oracle.render_reference(sc)
        digests[name] = {"scene_sha256": G.scene_digest(sc), "pixels_sha256": G.pixel_digest(px),
                         "width": sc.width, "height": sc.height, "draws": sc.n_draws}
        if name in G.PIXEL_SCENES:
            pixels[name] = px
        print(name, sc.width, sc.height, sc.n_draws, digests[name]["pixels_sha256"][:16])
    np.savez_compressed(os.path.join(HERE, "pixels.npz"), **pixels)
    with open(os.path.join(HERE, "digests.json"), "w") as f:
        json.dump(digests, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
