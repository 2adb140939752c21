"""Scenes whose reference pixels are committed as golden fixtures.

Each entry builds a scene deterministically (seeded generator or explicit
draws).  ``PIXEL_SCENES`` are small enough that their reference pixels are
stored whole (pixels.npz); ``DIGEST_SCENES`` are stored as SHA-256 digests
of the pixels (digests.json).  The fixtures are written by make_golden.py
from the reference software backend compiled from its own sources.
"""
from __future__ import annotations

import numpy as np

from skity_gb300 import scene as S


def stroke_then_fill():
    """test/ut/render/sw_canvas_test.cc:66-86: a 48x48 transparent bitmap, a
    rect (10,10,24,24) drawn kStrokeThenFill with width 10, red stroke and
    white fill; (12,20) must be white and (7,20) red."""
    b = S.SceneBuilder(48, 48, clear=None)
    p = S.default_paint()
    p["style"] = S.STROKE_THEN_FILL
    p["stroke_width"] = 10.0
    p["stroke_color"] = (1.0, 0.0, 0.0, 1.0)
    p["fill_color"] = (1.0, 1.0, 1.0, 1.0)
    b.draw_path([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE],
                [(10, 10), (34, 10), (34, 34), (10, 34)], p)
    return b.build()


def color_truncation():
    """test/ut/graphic/color_test.cc:44-51: Color4fToColor clamps and
    truncates ({-0.5, 1.5, 0.7, 0.2} -> ARGB(51, 0, 255, 178)); drawn with
    kSrc over the whole canvas, the bitmap holds the premultiplied colour."""
    b = S.SceneBuilder(8, 8, clear=(0.0, 0.0, 0.0, 0.0))
    p = S.default_paint()
    p["blend"] = S.BLEND_SRC
    p["fill_color"] = (-0.5, 1.5, 0.7, 0.2)
    b.draw_path([S.MOVE, S.LINE, S.LINE, S.LINE, S.CLOSE], [(0, 0), (8, 0), (8, 8), (0, 8)], p)
    return b.build()


def edge_cases():
    """Degenerate and clipped inputs: a lone move, a horizontal line, a huge
    triangle clipped on every side, an unclosed contour, a quad/cubic mix,
    a self-crossing even-odd star, a width-0 hairline stroke, and a conic
    stroked-and-filled with round caps."""
    b = S.SceneBuilder(64, 48)
    p = S.default_paint()
    p["fill_color"] = (0.2, 0.4, 0.6, 0.8)
    b.draw_path([S.MOVE], [(1, 1)], p)
    b.draw_path([S.MOVE, S.LINE, S.CLOSE], [(2, 2), (30, 2)], p)
    b.draw_path([S.MOVE, S.LINE, S.LINE, S.CLOSE], [(-50, -50), (200, 10), (10, 300)], p)
    b.draw_path([S.MOVE, S.LINE, S.LINE], [(5, 5), (40, 5.5), (20, 40)], p)
    b.draw_path([S.MOVE, S.QUAD, S.CUBIC, S.CLOSE],
                [(3, 40), (30, -20), (60, 40), (10, 10), (50, 10), (3, 40)], p)
    q = p.copy(); q["fill_type"] = S.EVEN_ODD
    b.draw_path([S.MOVE, S.LINE, S.LINE, S.LINE, S.LINE, S.CLOSE],
                [(10, 10), (50, 40), (50, 10), (10, 40), (30, 0)], q)
    s = p.copy(); s["style"] = S.STROKE; s["stroke_width"] = 0.0
    b.draw_path([S.MOVE, S.LINE], [(1, 30), (60, 31)], s)
    s2 = p.copy(); s2["style"] = S.STROKE_AND_FILL; s2["stroke_width"] = 3; s2["cap"] = S.ROUND
    b.draw_path([S.MOVE, S.CONIC, S.CLOSE], [(10, 20), (30, 0), (50, 20)], s2, weights=[0.5])
    return b.build()


def fills_128():
    """Config-1 style fills (3-32 verbs, lines/quads/cubics, nonzero) on a
    128x128 white canvas."""
    return S.random_paths_scene(S.SEED_BASE + 201, 128, 128, 60, 3, 32)


def mix_160():
    """Config-2 style mix on 160x160: coordinates beyond the canvas, 30%
    even-odd, 50% linear/radial gradients, 20% strokes with every cap and
    join."""
    return S.random_paths_scene(S.SEED_BASE + 202, 160, 160, 60, 3, 64,
                                coord_lo=(-16.0, -16.0), coord_hi=(176.0, 176.0),
                                evenodd_frac=0.3, gradient_frac=0.5, stroke_frac=0.2)


def strokes_160():
    """Every path stroked (width 1-8, all caps x joins), half even-odd."""
    return S.random_paths_scene(S.SEED_BASE + 203, 160, 120, 40, 2, 12,
                                coord_lo=(-8.0, -8.0), coord_hi=(168.0, 128.0),
                                evenodd_frac=0.5, stroke_frac=1.0)


def blur_160():
    """Config-4 style outlines (1-3 contours, even-odd), half with a kNormal
    blur mask filter."""
    return S.config4(seed=S.SEED_BASE + 204, n_outlines=60, width=160, height=160,
                     blur_frac=0.5)


PIXEL_SCENES = {
    "stroke_then_fill": stroke_then_fill,
    "color_truncation": color_truncation,
    "edge_cases": edge_cases,
    "fills_128": fills_128,
    "mix_160": mix_160,
    "strokes_160": strokes_160,
    "blur_160": blur_160,
}

DIGEST_SCENES = {
    "config1_512_1000": lambda: S.config1(),
    "config2_1024_300": lambda: S.config2(n_paths=300, width=1024, height=1024),
    "config4_1024_1500": lambda: S.config4(n_outlines=1500, width=1024, height=1024,
                                           blur_frac=0.2),
}


def pixel_digest(px: np.ndarray) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(px, np.uint8).tobytes()).hexdigest()


def scene_digest(sc) -> str:
    import hashlib
    return hashlib.sha256(sc.to_bytes()).hexdigest()
