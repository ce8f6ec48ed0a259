"""ctypes bindings of libpanostitch.so (the C ABI in include/panostitch.h).

The shared library is built in-tree by ``panostitcher_gb300.build``.  There
is no fallback: if the library is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
# PS_LIBRARY=checked selects the bounds-checked build (libpanostitch_checked.so,
# every kernel access checked against its buffer; see ps_debug_bounds_violations).
LIB_PATH = os.path.join(HERE, "libpanostitch_checked.so" if os.environ.get("PS_LIBRARY") == "checked"
                        else "libpanostitch.so")

PS_OK, PS_EINVAL, PS_ENOMEM, PS_ECUDA, PS_ETIMEOUT, PS_ESTATE = 0, 1, 2, 3, 4, 5
PS_MAX_LEVELS, PS_MAX_CAMS, PS_MAX_IN_FLIGHT = 16, 64, 8
PS_FMT_BGR24, PS_FMT_BGR32 = 24, 32
PS_FMT_YUV420P, PS_FMT_NV12 = 420, 12
PS_SEAMS_NEAREST_AXIS, PS_SEAMS_DISTANCE = 0, 1
PS_MEM_HOST, PS_MEM_DEVICE = 0, 1
(EXPORT_XMAP, EXPORT_YMAP, EXPORT_COVERAGE, EXPORT_SEAM, EXPORT_WEIGHT, EXPORT_ALPHA, EXPORT_LINEAR_WEIGHT,
 EXPORT_LEVEL0) = range(8)

_STATUS_NAMES = {PS_EINVAL: "PS_EINVAL", PS_ENOMEM: "PS_ENOMEM", PS_ECUDA: "PS_ECUDA",
                 PS_ETIMEOUT: "PS_ETIMEOUT", PS_ESTATE: "PS_ESTATE"}


class PsError(RuntimeError):
    """A non-zero status from the C ABI, with ps_last_error()'s text."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class PhotoParam(C.Structure):
    """ps_photo_param == PhotoParam (source/Warp/ZReproject.h:17-50)."""

    _fields_ = [(n, C.c_int) for n in ("image_type", "crop_mode", "crop_x", "crop_y", "crop_width",
                                       "crop_height", "circle_x", "circle_y", "circle_r")] + \
               [(n, C.c_double) for n in ("hfov", "vfov", "alpha", "beta", "gamma", "shift_x", "shift_y",
                                          "shear_x", "shear_y", "yaw", "pitch", "roll")]

    @classmethod
    def from_dict(cls, d: dict) -> "PhotoParam":
        p = cls()
        for k, v in d.items():
            setattr(p, k, v)
        return p


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("pitch", C.c_longlong), ("width", C.c_int), ("height", C.c_int),
                ("format", C.c_int), ("location", C.c_int)]


class PlanarImage(C.Structure):
    """ps_planar_image: Y / U / V (YUV420P) or Y / UV (NV12) planes."""

    _fields_ = [("planes", C.c_void_p * 3), ("pitches", C.c_longlong * 3), ("width", C.c_int),
                ("height", C.c_int), ("format", C.c_int), ("location", C.c_int)]


class LaunchShape(C.Structure):
    """ps_launch_shape: the launch choices that can change after prepare."""

    _fields_ = [("tail_max_items", C.c_int), ("tail_cluster", C.c_int), ("tail_half_tiles", C.c_int),
                ("ctas_per_sm", C.c_int * 3), ("small_blend_max_items", C.c_int), ("remap_defer_ties", C.c_int)]


class TuneReport(C.Structure):
    _fields_ = [("ms_per_frame_default", C.c_double), ("ms_per_frame_chosen", C.c_double), ("trials", C.c_int),
                ("cached", C.c_int)]


_lib = None
_lock = threading.Lock()

# (name, restype, argtypes)
_SIGS = [
    ("ps_last_error", C.c_char_p, []),
    ("ps_version", C.c_char_p, []),
    ("ps_render_create", C.c_int, [C.POINTER(C.c_void_p)]),
    ("ps_render_destroy", None, [C.c_void_p]),
    ("ps_render_prepare", C.c_int, [C.c_void_p, C.POINTER(PhotoParam), C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ps_render_prepare_with_seams", C.c_int, [C.c_void_p, C.POINTER(PhotoParam), C.c_int, C.c_int, C.c_int,
                                               C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p),
                                               C.c_void_p]),
    ("ps_render_render", C.c_int, [C.c_void_p, C.POINTER(Image), C.c_int, C.c_void_p, C.c_int,
                                   C.POINTER(Image), C.c_void_p]),
    ("ps_render_render_yuv", C.c_int, [C.c_void_p, C.POINTER(Image), C.c_int, C.c_void_p, C.c_int,
                                       C.POINTER(PlanarImage), C.c_void_p]),
    ("ps_render_prepare_file", C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_void_p]),
    ("ps_load_photo_params", C.c_int, [C.c_char_p, C.POINTER(PhotoParam), C.c_int, C.POINTER(C.c_int)]),
    ("ps_render_set_seam_rule", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_render_set_custom_masks", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int, C.c_void_p]),
    ("ps_blender_set_custom_masks", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int, C.c_void_p]),
    ("ps_render_set_frames_in_flight", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_render_get_frames_in_flight", C.c_int, [C.c_void_p]),
    ("ps_render_set_memory_budget", C.c_int, [C.c_void_p, C.c_longlong]),
    ("ps_render_is_low_memory", C.c_int, [C.c_void_p]),
    ("ps_render_set_map_free", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_debug_bounds_violations", C.c_longlong, [C.c_int]),
    ("ps_render_is_map_free", C.c_int, [C.c_void_p]),
    ("ps_render_render_planar", C.c_int, [C.c_void_p, C.POINTER(PlanarImage), C.c_int, C.c_void_p, C.c_int,
                                          C.POINTER(Image), C.POINTER(PlanarImage), C.c_void_p]),
    ("ps_render_set_graph", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_render_check", C.c_int, [C.c_void_p]),
    ("ps_render_set_wait_probe", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_blender_check", C.c_int, [C.c_void_p]),
    ("ps_blender_begin", C.c_int, [C.c_void_p, C.c_void_p]),
    ("ps_blender_tile", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_void_p]),
    ("ps_blender_end", C.c_int, [C.c_void_p, C.POINTER(Image), C.c_void_p]),
    ("ps_blender_get_unique_masks", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int]),
    ("ps_blender_used_memory", C.c_longlong, [C.c_void_p]),
    ("ps_blender_estimate_memory", C.c_longlong, [C.c_int, C.c_int, C.c_int, C.c_int]),
    ("ps_render_get_unique_masks", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int]),
    ("ps_render_estimate_memory", C.c_longlong, [C.POINTER(PhotoParam), C.c_int, C.c_int, C.c_int, C.c_int,
                                                 C.c_int, C.c_int, C.c_int]),
    ("ps_blender_set_wait_probe", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_render_clear", None, [C.c_void_p]),
    ("ps_render_get_num_images", C.c_int, [C.c_void_p]),
    ("ps_render_get_num_levels", C.c_int, [C.c_void_p]),
    ("ps_render_is_full_mask", C.c_int, [C.c_void_p]),
    ("ps_render_resident_bytes", C.c_longlong, [C.c_void_p]),
    ("ps_render_get_input_buffer", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_void_p),
                                             C.POINTER(C.c_longlong)]),
    ("ps_render_export", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_longlong]),
    ("ps_render_export_collapsed", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong, C.c_void_p]),
    ("ps_render_profile", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_render_profile_read", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_longlong),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("ps_render_launches_per_frame", C.c_int, [C.c_void_p]),
    ("ps_render_algorithmic_bytes", C.c_double, [C.c_void_p, C.c_int, C.c_int]),
    ("ps_render_set_launch_shape", C.c_int, [C.c_void_p, C.POINTER(LaunchShape)]),
    ("ps_render_get_launch_shape", C.c_int, [C.c_void_p, C.POINTER(LaunchShape)]),
    ("ps_render_autotune", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(LaunchShape),
                                     C.POINTER(TuneReport)]),
    ("ps_render_batch", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.POINTER(Image)),
                                  C.POINTER(C.c_void_p), C.POINTER(Image), C.c_void_p]),
    ("ps_generate_reproject_map_and_mask", C.c_int, [C.POINTER(PhotoParam), C.c_int, C.c_int, C.c_int, C.c_int,
                                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("ps_reproject_to_16s", C.c_int, [C.POINTER(Image), C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_int,
                                      C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]),
    ("ps_get_lut", C.c_int, [C.c_double, C.c_void_p]),
    ("ps_non_intersecting_masks", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("ps_distance_transform_l1", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("ps_cvt_bgr32_to_yuv", C.c_int, [C.POINTER(Image), C.POINTER(PlanarImage), C.c_void_p]),
    ("ps_cvt_yuv_to_bgr32", C.c_int, [C.POINTER(PlanarImage), C.POINTER(Image), C.c_void_p]),
    ("ps_nearest_axis_seams_no_alloc", C.c_int, [C.POINTER(PhotoParam), C.c_int, C.c_int, C.c_int, C.c_int,
                                                 C.c_int, C.c_void_p, C.c_void_p]),
    ("ps_blender_create", C.c_int, [C.POINTER(C.c_void_p)]),
    ("ps_blender_destroy", None, [C.c_void_p]),
    ("ps_blender_prepare", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                     C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ps_blender_blend", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_longlong), C.c_int,
                                   C.POINTER(Image), C.c_void_p]),
    ("ps_blender_get_num_levels", C.c_int, [C.c_void_p]),
    ("ps_server_create", C.c_int, [C.c_longlong, C.c_int, C.POINTER(C.c_void_p)]),
    ("ps_server_destroy", None, [C.c_void_p]),
    ("ps_server_admit", C.c_int, [C.c_void_p, C.POINTER(PhotoParam), C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_int, C.c_int, C.POINTER(C.c_int)]),
    ("ps_server_remove", C.c_int, [C.c_void_p, C.c_int]),
    ("ps_server_resident_bytes", C.c_longlong, [C.c_void_p]),
    ("ps_server_run_trace", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.POINTER(Image)),
                                      C.POINTER(C.c_void_p), C.POINTER(Image), C.c_void_p, C.c_void_p]),
]


def lib():
    """Load libpanostitch.so (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: run panostitcher_gb300.build.build() first "
                                   "(there is no CPU fallback)")
            L = C.CDLL(LIB_PATH)
            for name, res, args in _SIGS:
                f = getattr(L, name, None)
                if f is None:
                    continue
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def check(status: int) -> None:
    if status != PS_OK:
        raise PsError(status, lib().ps_last_error().decode(errors="replace"))


def exported_symbols():
    """Names of the C ABI functions this module binds."""
    return [s[0] for s in _SIGS]
