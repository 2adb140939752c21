"""Seeded families of small scenes for the parity sweeps
(tests/test_fuzz_cpu.py on the CPU build of the device code,
tests/test_gpu_fuzz.py on the GPU): each family is one of the pinned
scene generators of tests/test_oracle_pin.py run over many seeds and canvas
sizes, so feature combinations the hand-picked seeds miss are reached."""
from skity_gb300 import scene as S

import test_oracle_pin as P
from test_image_shader import image_scene


def _size(seed, lo, hi):
    return lo + (seed * 37) % (hi - lo), lo + (seed * 53) % (hi - lo)


def families(n: int):
    """(name, scene) pairs: n seeds of each family."""
    out = []
    for k in range(n):
        seed = S.SEED_BASE + 5000 + 17 * k
        w, h = _size(k, 48, 200)
        out.append(("matrices", P.matrix_scene(seed, w, h, shaded=k % 2 == 0)))
        out.append(("clips", P.clipped_scene(seed + 1, w, h)))
        out.append(("path_clips", P.path_clips_scene(seed + 2, w, h, n_ops=40)))
        out.append(("layers", S.layered_scene(seed + 3, w, h, 40, 1 + k % 3,
                                              blends=(S.BLEND_SRC_OVER, 24, 5, 14))))
        out.append(("blend_modes", P.blend_modes_scene(seed + 4, w, h)))
        out.append(("gradients", P.sweep_conical_scene(seed + 5, w, h)))
        out.append(("color_filters", P.color_filters_scene(seed + 6, w, h)))
        out.append(("images", image_scene(seed + 7, w, h)))
        out.append(("fills", S.random_paths_scene(seed + 8, w, h, 30, 1, 40,
                                                  coord_lo=(-30.0, -30.0),
                                                  coord_hi=(w + 30.0, h + 30.0),
                                                  evenodd_frac=0.5, gradient_frac=0.4,
                                                  stroke_frac=0.4)))
    return out
