"""The canvas matrix of the C ABI canvas (translate / scale / rotate / skew /
concat / set_matrix, restated in skity_gb300/csrc/stroke.cuh) against the
reference's own Canvas computing it (oracle/_ref/ref_matrix, built from the
reference's sources): bit-identical Get9 values for seeded call sequences.
CPU only; skipped where the reference build is absent."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_MATRIX = os.path.join(ROOT, "oracle", "_ref", "ref_matrix")


@pytest.fixture(scope="module")
def ref_matrix(oracle_lib):
    try:
        oracle_lib.build_reference()
    except RuntimeError as e:
        pytest.skip(f"reference build failed: {e}")
    if not os.path.exists(REF_MATRIX):
        pytest.skip("reference checkout not present")
    return REF_MATRIX


NARGS = {0: 2, 1: 2, 2: 3, 3: 2, 4: 9, 5: 9}
LETTER = {0: "t", 1: "s", 2: "r", 3: "k", 4: "c", 5: "m"}


def _sequence(rng, n):
    ops, args = [], []
    for _ in range(n):
        op = int(rng.choice([0, 1, 2, 3, 4, 5], p=[0.25, 0.2, 0.25, 0.1, 0.15, 0.05]))
        if op == 0:
            a = rng.uniform(-200, 200, 2)
        elif op == 1:
            a = rng.uniform(-3, 3, 2)
        elif op == 2:
            a = np.concatenate([rng.uniform(-720, 720, 1), rng.uniform(-100, 300, 2)])
        elif op == 3:
            a = rng.uniform(-1, 1, 2)
        else:
            a = np.array([*rng.uniform(-2, 2, 2), rng.uniform(-90, 90), *rng.uniform(-2, 2, 2),
                          rng.uniform(-90, 90), 0.0, 0.0, 1.0])
        if rng.uniform() < 0.1 and op in (0, 1, 3):
            a = np.array([0.0, 0.0]) if op != 1 else np.array([1.0, 1.0])  # identity calls
        ops.append(op)
        args.append(np.asarray(a, np.float32))
    return ops, args


@pytest.mark.parametrize("seed", range(40))
def test_canvas_matrix_matches_reference(cpu_pipeline, ref_matrix, seed):
    rng = np.random.default_rng(1000 + seed)
    ops, args = _sequence(rng, int(rng.integers(1, 7)))
    flat = np.concatenate(args).astype(np.float32)
    cmd = [ref_matrix]
    for op, a in zip(ops, args):
        cmd += [LETTER[op]] + [float(v).hex() for v in a]
    want = [float.fromhex(v) for v in subprocess.check_output(cmd, text=True).split()]
    lib = cpu_pipeline
    lib.skc_canvas_matrix.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                      ctypes.c_void_p]
    o = np.asarray(ops, np.int32)
    out = np.zeros(9, np.float32)
    lib.skc_canvas_matrix(o.ctypes.data, len(ops), flat.ctypes.data, out.ctypes.data)
    assert np.asarray(want, np.float32).tobytes() == out.tobytes(), (ops, want, out.tolist())
