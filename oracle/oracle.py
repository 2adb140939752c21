"""Loader of the CPU oracle (oracle/sw_oracle.cc) and of the reference build
(oracle/_ref, present only where the reference sources were available).
Test infrastructure: see oracle/__init__.py."""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libskity_oracle.so")
REF_RENDER = os.path.join(HERE, "_ref", "ref_render")
REFERENCE_SRC = "/root/reference"


class Stats(ctypes.Structure):
    _fields_ = [("fragments", ctypes.c_uint64), ("spans", ctypes.c_uint64),
                ("edges", ctypes.c_uint64), ("tie_groups", ctypes.c_uint64),
                ("seconds", ctypes.c_double), ("draws", ctypes.c_uint64)]


def build() -> str:
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def build_reference() -> bool:
    """Compiles the reference's software backend from its own sources into
    oracle/_ref (only where the reference checkout exists)."""
    if not os.path.isdir(REFERENCE_SRC):
        return False
    r = subprocess.run(["make", "-s", "-j8", "-C", os.path.join(HERE, "ref"),
                        f"REF={REFERENCE_SRC}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout + r.stderr)
    return True


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
        _lib.sko_render.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_void_p, ctypes.POINTER(Stats)]
        _lib.sko_render.restype = ctypes.c_int
        _lib.sko_render_mt.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                       ctypes.POINTER(Stats)]
        _lib.sko_render_mt.restype = ctypes.c_int
        _lib.sko_cubic_quad_count.argtypes = [ctypes.POINTER(ctypes.c_float)]
        _lib.sko_quad_edge.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32)]
        _lib.sko_path_spans.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_uint32]
    return _lib


def render(scene, first: int = 0, count: int | None = None):
    """Pixels (h, w, 4) uint8 and Stats of replaying draws [first, first+count)."""
    b = scene.to_bytes()
    count = scene.n_draws if count is None else count
    out = np.zeros((scene.height, scene.width, 4), np.uint8)
    st = Stats()
    rc = lib().sko_render(b, len(b), first, count, out.ctypes.data, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    return out, st


def render_mt(scene, threads: int, first: int = 0, count: int | None = None):
    """render() on `threads` host threads (banded rows, identical pixels)."""
    b = scene.to_bytes()
    count = scene.n_draws if count is None else count
    out = np.zeros((scene.height, scene.width, 4), np.uint8)
    st = Stats()
    rc = lib().sko_render_mt(b, len(b), first, count, out.ctypes.data, threads, ctypes.byref(st))
    if rc != 0:
        raise RuntimeError(f"oracle render failed ({rc})")
    return out, st


def reference_available() -> bool:
    return os.path.exists(REF_RENDER)


def render_reference(scene, first: int = 0, count: int | None = None):
    """Pixels from the reference's own software backend (oracle/_ref)."""
    count = scene.n_draws if count is None else count
    with tempfile.TemporaryDirectory() as d:
        sp, op = os.path.join(d, "s.bin"), os.path.join(d, "o.rgba")
        with open(sp, "wb") as f:
            f.write(scene.to_bytes())
        r = subprocess.run([REF_RENDER, sp, op, str(first), str(count)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("ref_render failed: " + r.stderr)
        return np.fromfile(op, np.uint8).reshape(scene.height, scene.width, 4)


def compare(a: np.ndarray, b: np.ndarray) -> dict:
    """Parity statistics: max |delta| per channel, count and fraction of
    pixels that are not exactly equal."""
    d = np.abs(a.astype(np.int16) - b.astype(np.int16))
    bad = d.max(axis=-1) > 0
    return {"max_abs_diff": int(d.max()) if d.size else 0, "bad_pixels": int(bad.sum()),
            "exact_frac": float(1.0 - bad.mean()) if bad.size else 1.0}
