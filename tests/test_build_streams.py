"""The threaded stream build (BuildStreams: runs of canvases parsed on host
threads, then appended with their indices and offsets moved) builds the
same batch, byte for byte, as one thread adding the canvases in order --
over scenes with every kind of record a stream holds: gradients of each
kind, strokes, colour filters, blur temp canvases, layers, path clips and
images."""
import ctypes

import pytest

from skity_gb300 import scene as S


def _streams():
    from test_image_shader import image_scene
    from test_oracle_pin import (blend_modes_scene, blur_styles_scene, clip_path_cases_scene,
                                 clipped_scene, color_filters_scene, path_clips_scene,
                                 sweep_conical_scene, translated_scene)
    scenes = list(S.config3(n_canvases=24, scale=0.2))
    scenes += [translated_scene(), clipped_scene(), blend_modes_scene(), sweep_conical_scene(),
               blur_styles_scene(), color_filters_scene(), path_clips_scene(),
               clip_path_cases_scene(), image_scene(),
               S.layered_scene(S.SEED_BASE + 420, 96, 80, 60, 3),
               S.config4(n_outlines=400, width=256, height=256, blur_frac=0.3),
               S.config2(n_paths=300, width=256, height=256)]
    # the feature scenes spread between the plain canvases, so runs mix both
    mixed = []
    for i, sc in enumerate(scenes[24:]):
        mixed += scenes[2 * i:2 * i + 2] + [sc]
    return [sc.to_bytes() for sc in mixed]


@pytest.mark.parametrize("threads", [2, 3, 8, 16])
def test_threaded_build_matches_one_thread(cpu_pipeline, threads):
    lib = cpu_pipeline
    lib.skc_build_streams_compare.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_uint]
    bufs = _streams()
    n = len(bufs)
    cbufs = [ctypes.create_string_buffer(b, len(b)) for b in bufs]
    ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(c) for c in cbufs])
    lens = (ctypes.c_size_t * n)(*[len(b) for b in bufs])
    assert lib.skc_build_streams_compare(n, ptrs, lens, threads) == 0


def test_threaded_build_reports_first_bad_stream(cpu_pipeline):
    """A malformed stream fails the build with the status the one-thread
    loop returns for the first bad stream in order."""
    lib = cpu_pipeline
    lib.skc_build_streams_compare.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_uint]
    bufs = [sc.to_bytes() for sc in S.config3(n_canvases=16, scale=0.1)]
    bufs[9] = bufs[9][:len(bufs[9]) // 2]  # truncated
    n = len(bufs)
    cbufs = [ctypes.create_string_buffer(b, len(b)) for b in bufs]
    ptrs = (ctypes.c_void_p * n)(*[ctypes.addressof(c) for c in cbufs])
    lens = (ctypes.c_size_t * n)(*[len(b) for b in bufs])
    assert lib.skc_build_streams_compare(n, ptrs, lens, 4) == -2  # INVALID_ARGUMENT
