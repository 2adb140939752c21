"""ctypes binding of the C ABI in include/skity_cuda.h.

The library must be built (skity_gb300.build.build()) and a CUDA device
present; there is no CPU fallback: loading fails loudly otherwise.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

SUCCESS = 0
NOT_READY = 1
ERRORS = {
    1: "not ready", -10: "cancelled",
    -1: "invalid handle", -2: "invalid argument", -3: "initialization failed",
    -4: "out of host memory", -5: "not supported", -6: "device error",
    -7: "out of device memory", -8: "device timeout",
    -9: "input exceeds the fixed scratch of skity_cuda_draw_path_static",
}


class SkityCudaError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: {ERRORS.get(code, code)} ({code})")
        self.code = code


class Path_(ctypes.Structure):
    _fields_ = [("verbs", ctypes.c_void_p), ("verb_count", ctypes.c_uint32),
                ("points", ctypes.c_void_p), ("point_count", ctypes.c_uint32),
                ("conic_weights", ctypes.c_void_p), ("conic_weight_count", ctypes.c_uint32),
                ("fill_type", ctypes.c_uint32)]


class Gradient_(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("tile_mode", ctypes.c_uint32),
                ("stop_count", ctypes.c_uint32), ("has_offsets", ctypes.c_uint32),
                ("p0", ctypes.c_float * 2), ("p1", ctypes.c_float * 2),
                ("radius", ctypes.c_float * 2), ("colors", ctypes.c_void_p),
                ("offsets", ctypes.c_void_p)]


class ColorFilter_(ctypes.Structure):
    _fields_ = [("type", ctypes.c_uint32), ("blend_mode", ctypes.c_uint32),
                ("color", ctypes.c_uint32), ("matrix", ctypes.c_float * 20)]


class Image_(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("alpha_type", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("pixels", ctypes.c_void_p)]


class ImageShader_(ctypes.Structure):
    _fields_ = [("image", ctypes.POINTER(Image_)), ("filter", ctypes.c_uint32),
                ("tile_x", ctypes.c_uint32), ("tile_y", ctypes.c_uint32),
                ("local_matrix", ctypes.c_float * 6)]


class Paint_(ctypes.Structure):
    _fields_ = [("style", ctypes.c_uint32), ("cap", ctypes.c_uint32), ("join", ctypes.c_uint32),
                ("blend_mode", ctypes.c_uint32), ("fill_color", ctypes.c_float * 4),
                ("stroke_color", ctypes.c_float * 4), ("stroke_width", ctypes.c_float),
                ("miter_limit", ctypes.c_float), ("shader", ctypes.POINTER(Gradient_)),
                ("blur_style", ctypes.c_uint32), ("blur_radius", ctypes.c_float),
                ("color_filter", ctypes.POINTER(ColorFilter_)),
                ("image_shader", ctypes.POINTER(ImageShader_))]


class ContextInfo_(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("device_memory_budget", ctypes.c_uint64)]


class Stats_(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("total_ms", ctypes.c_double),
                ("draws", ctypes.c_uint64), ("passes", ctypes.c_uint64),
                ("edges", ctypes.c_uint64), ("spans", ctypes.c_uint64),
                ("pixels", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("retries", ctypes.c_uint64), ("geometry_ms", ctypes.c_double),
                ("sweep_count_ms", ctypes.c_double), ("sweep_emit_ms", ctypes.c_double),
                ("composite_ms", ctypes.c_double), ("blur_ms", ctypes.c_double),
                ("fragments", ctypes.c_uint64), ("graph_replays", ctypes.c_uint64),
                ("fragments_by_brush", ctypes.c_uint64 * 4), ("plan_ms", ctypes.c_double),
                ("host_syncs", ctypes.c_uint64), ("parse_ms", ctypes.c_double),
                ("upload_ms", ctypes.c_double), ("readback_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["fragments_by_brush"] = list(self.fragments_by_brush)
        return d


class ServerInfo_(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("memory_budget", ctypes.c_uint64), ("workers", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32)]


class RequestInfo_(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("batch_size", ctypes.c_uint32), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32)]


class RasterConfig_(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("tile_width", ctypes.c_uint32),
                ("ctas_per_sm", ctypes.c_uint32), ("band_rows", ctypes.c_uint32),
                ("sweep_warps", ctypes.c_uint32)]


# every entry point declared in include/skity_cuda.h: name -> (restype, argtypes)
_vp = ctypes.c_void_p
SIGNATURES = {
    "skity_cuda_version": (ctypes.c_char_p, []),
    "skity_cuda_context_create": (ctypes.c_int32, [ctypes.POINTER(ContextInfo_), ctypes.POINTER(_vp)]),
    "skity_cuda_context_destroy": (None, [_vp]),
    "skity_cuda_context_get_stats": (ctypes.c_int32, [_vp, ctypes.POINTER(Stats_)]),
    "skity_cuda_canvas_create": (ctypes.c_int32, [_vp, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                                  ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "skity_cuda_canvas_destroy": (None, [_vp]),
    "skity_cuda_canvas_clear": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "skity_cuda_canvas_draw_path": (ctypes.c_int32, [_vp, ctypes.POINTER(Path_), ctypes.POINTER(Paint_)]),
    "skity_cuda_canvas_flush": (ctypes.c_int32, [_vp]),
    "skity_cuda_canvas_save": (ctypes.c_int32, [_vp]),
    "skity_cuda_canvas_restore": (ctypes.c_int32, [_vp]),
    "skity_cuda_canvas_translate": (ctypes.c_int32, [_vp, ctypes.c_float, ctypes.c_float]),
    "skity_cuda_canvas_scale": (ctypes.c_int32, [_vp, ctypes.c_float, ctypes.c_float]),
    "skity_cuda_canvas_rotate": (ctypes.c_int32, [_vp, ctypes.c_float, ctypes.c_float,
                                                  ctypes.c_float]),
    "skity_cuda_canvas_skew": (ctypes.c_int32, [_vp, ctypes.c_float, ctypes.c_float]),
    "skity_cuda_canvas_concat": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "skity_cuda_canvas_set_matrix": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "skity_cuda_canvas_get_matrix": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "skity_cuda_canvas_concat44": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "skity_cuda_canvas_set_matrix44": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float)]),
    "skity_cuda_canvas_clip_rect": (ctypes.c_int32, [_vp, ctypes.c_float, ctypes.c_float,
                                                     ctypes.c_float, ctypes.c_float]),
    "skity_cuda_canvas_clip_path": (ctypes.c_int32, [_vp, ctypes.POINTER(Path_), ctypes.c_uint32]),
    "skity_cuda_canvas_draw_image_rect": (ctypes.c_int32, [_vp, ctypes.POINTER(Image_),
                                                           ctypes.POINTER(ctypes.c_float),
                                                           ctypes.POINTER(ctypes.c_float),
                                                           ctypes.c_uint32, ctypes.POINTER(Paint_)]),
    "skity_cuda_render_streams": (ctypes.c_int32, [_vp, ctypes.c_uint32, ctypes.POINTER(_vp),
                                                   ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_vp)]),
    "skity_cuda_batch_create": (ctypes.c_int32, [_vp, ctypes.c_uint32, ctypes.POINTER(_vp),
                                                 ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_vp)]),
    "skity_cuda_batch_render": (ctypes.c_int32, [_vp]),
    "skity_cuda_batch_render_per_draw": (ctypes.c_int32, [_vp]),
    "skity_cuda_canvas_save_layer": (ctypes.c_int32, [_vp, ctypes.POINTER(ctypes.c_float),
                                                      ctypes.POINTER(Paint_)]),
    "skity_cuda_recorder_begin": (ctypes.c_int32, [ctypes.c_uint32, ctypes.c_uint32,
                                                   ctypes.POINTER(_vp)]),
    "skity_cuda_recorder_finish": (ctypes.c_int32, [_vp, ctypes.POINTER(_vp)]),
    "skity_cuda_display_list_destroy": (None, [_vp]),
    "skity_cuda_display_list_op_count": (ctypes.c_uint32, [_vp]),
    "skity_cuda_display_list_draw": (ctypes.c_int32, [_vp, _vp]),
    "skity_cuda_display_list_to_stream": (ctypes.c_int32, [_vp, _vp,
                                                           ctypes.POINTER(ctypes.c_size_t)]),
    "skity_cuda_batch_read": (ctypes.c_int32, [_vp, ctypes.c_uint32, _vp]),
    "skity_cuda_batch_destroy": (None, [_vp]),
    "skity_cuda_context_set_config": (ctypes.c_int32, [_vp, ctypes.POINTER(RasterConfig_)]),
    "skity_cuda_batch_set_config": (ctypes.c_int32, [_vp, ctypes.POINTER(RasterConfig_)]),
    "skity_cuda_batch_get_config": (ctypes.c_int32, [_vp, ctypes.POINTER(RasterConfig_)]),
    "skity_cuda_server_create": (ctypes.c_int32, [ctypes.POINTER(ServerInfo_), ctypes.POINTER(_vp)]),
    "skity_cuda_server_submit": (ctypes.c_int32, [_vp, _vp, ctypes.c_size_t,
                                                  ctypes.POINTER(ctypes.c_uint64)]),
    "skity_cuda_server_wait": (ctypes.c_int32, [_vp, ctypes.c_uint64, ctypes.c_uint32, _vp,
                                                ctypes.POINTER(RequestInfo_)]),
    "skity_cuda_server_destroy": (None, [_vp]),
    "skity_cuda_draw_path_static": (ctypes.c_int32, [ctypes.c_int32, _vp, ctypes.c_uint32,
                                                     ctypes.c_uint32, ctypes.c_size_t,
                                                     ctypes.POINTER(Path_), ctypes.POINTER(Paint_),
                                                     _vp]),
}

_LIB = None


def library_path() -> str:
    return _build.LIB


def load(path: str | None = None) -> ctypes.CDLL:
    """Loads libskity_cuda.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or _build.LIB
    if not os.path.exists(p):
        raise RuntimeError(f"skity_gb300 CUDA library not built ({p}); run skity_gb300.build.build()")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(code: int, what: str) -> None:
    if code != SUCCESS:
        raise SkityCudaError(code, what)
