"""Writes tests/golden/full_digests.json: SHA-256 digests of the oracle's
pixels for every canvas of the full-size seeded workloads -- the 512x512
scene (1,000 fills), the 2048x2048 scene (20,000 paths), the 256-canvas
batch and the 4096x4096 glyph-dense scene with blur -- so that GPU tests and
the bench can check a full-size render without re-running the oracle (which
takes minutes on the 2048x2048 scene).  A digest that does not match makes
the checker fall back to the oracle itself, which then reports the size of
the difference.

    python tests/golden/make_full_digests.py [threads]
"""
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def digest(px) -> str:
    return hashlib.sha256(px.tobytes()).hexdigest()


def main():
    from oracle import oracle
    from skity_gb300 import scene as S
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    oracle.build()
    out = {"generator": "oracle.render_mt over skity_gb300.scene.config1..config4 (default seeds)"}
    for name, scenes in [("config1", [S.config1()]), ("config4", [S.config4()]),
                         ("config3", S.config3()), ("config2", [S.config2()])]:
        t = time.time()
        out[name] = [digest(oracle.render_mt(sc, threads)[0]) for sc in scenes]
        print(name, len(scenes), f"{time.time() - t:.1f} s", flush=True)
    with open(os.path.join(HERE, "full_digests.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
