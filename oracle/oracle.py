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
# the reference checkout the pinning build compiles from
REFERENCE_SRC = os.environ.get("SKITY_REFERENCE", "/root/reference")


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
        _lib.sko_sample.argtypes = [ctypes.c_void_p] + [ctypes.c_uint32] * 6 + [ctypes.c_float] * 2
        _lib.sko_sample.restype = ctypes.c_uint32
        _lib.sko_render_mt.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                       ctypes.POINTER(Stats)]
        _lib.sko_render_mt.restype = ctypes.c_int
        _lib.sko_cubic_quad_count.argtypes = [ctypes.POINTER(ctypes.c_float)]
        _lib.sko_quad_edge.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32)]
        _lib.sko_path_spans.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_uint32]
        _lib.sko_fill_quads.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                        ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32)]
        _lib.ska_exact_coverage.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                            ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    return _lib


def sample(rgba, alpha_type, filter, tile_x, tile_y, u, v) -> int:
    """BitmapSampler::GetColor of an (h, w, 4) RGBA8 pixmap at unit
    coordinates (u, v), premultiplied as the pixmap brush does for
    unpremultiplied pixels: an ARGB colour."""
    px = np.ascontiguousarray(rgba, np.uint8)
    return int(lib().sko_sample(px.ctypes.data, px.shape[1], px.shape[0], alpha_type, filter,
                                tile_x, tile_y, u, v))


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


def fill_quads(scene, draw: int):
    """The QuadPath one draw's fill rasterises: (verbs u8, points (n, 2) f32)."""
    b = scene.to_bytes()
    L = lib()
    counts = (ctypes.c_uint32 * 2)()
    L.sko_fill_quads(b, len(b), draw, None, 0, None, 0, counts)
    verbs = np.zeros(max(counts[0], 1), np.uint8)
    pts = np.zeros((max(counts[1], 1), 2), np.float32)
    L.sko_fill_quads(b, len(b), draw, verbs.ctypes.data, counts[0], pts.ctypes.data, counts[1],
                     counts)
    return verbs[:counts[0]], pts[:counts[1]]


def exact_coverage(scene, draw: int, tol: float = 1e-4) -> np.ndarray:
    """FP64 exact-area coverage (height, width) in [0, 1] of one draw's fill
    (oracle/exact_area.cc)."""
    verbs, pts = fill_quads(scene, draw)
    cov = np.zeros((scene.height, scene.width), np.float64)
    pts = np.ascontiguousarray(pts, np.float32)
    rc = lib().ska_exact_coverage(verbs.ctypes.data, len(verbs), pts.ctypes.data, len(pts),
                                  int(scene.paints[draw]["fill_type"]) & 1, scene.width,
                                  scene.height, tol, cov.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"exact coverage failed ({rc})")
    return cov


def coverage_scenes(scene):
    """One single-draw scene per fill draw of `scene`: the draw's path and
    fill rule, an opaque white solid paint, on a transparent canvas -- the
    rendered alpha is the coverage the rasteriser gives the path."""
    from skity_gb300 import scene as S
    out = []
    for d in range(scene.n_draws):
        sub = scene.subset(d, 1)
        p = sub.paints[0]
        if p["style"] != S.FILL or p["blur_style"] != 0:
            continue
        p["fill_color"] = (1.0, 1.0, 1.0, 1.0)
        p["gradient"] = -1
        p["blend"] = S.BLEND_SRC_OVER
        sub.clear = (0.0, 0.0, 0.0, 0.0)
        out.append((d, sub))
    return out


def coverage_error(scene, alphas: list, tol: float = 1e-4) -> dict:
    """Max and mean |rendered coverage - exact area| in 1/255 units over the
    pixels either one touches, for the fill draws of `scene`; `alphas[i]` is
    the alpha channel (h, w) rendered for coverage_scenes(scene)[i]."""
    err_max, err_sum, n, edge = 0.0, 0.0, 0, 0
    for (d, _), a in zip(coverage_scenes(scene), alphas):
        ex = exact_coverage(scene, d, tol)
        got = np.asarray(a, np.float64) / 255.0
        m = (ex > 0) | (got > 0)
        e = np.abs(got - ex)[m] * 255.0
        if e.size:
            err_max = max(err_max, float(e.max()))
            err_sum += float(e.sum())
            n += int(e.size)
        edge += int(((ex > 0) & (ex < 1)).sum())
    return {"max_err_255": err_max, "mean_err_255": err_sum / max(n, 1), "pixels": n,
            "edge_pixels": edge, "tol_px": tol}


def reference_available() -> bool:
    return os.path.exists(REF_RENDER)


def render_reference_skp(skp_path: str):
    """An SKP file played back by the reference's own IO module onto its
    software canvas, cleared to opaque white (oracle/_ref/ref_skp)."""
    exe = os.path.join(os.path.dirname(REF_RENDER), "ref_skp")
    with tempfile.TemporaryDirectory() as d:
        op = os.path.join(d, "o.rgba")
        r = subprocess.run([exe, skp_path, op], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("ref_skp failed: " + r.stderr)
        w, h = (int(v) for v in r.stdout.split())
        return np.fromfile(op, np.uint8).reshape(h, w, 4)


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
