"""CPU oracle for the panorama stitch path -- TEST INFRASTRUCTURE ONLY.

This package is the checker: ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` call it to produce
the reference answer and the CPU timing.  The product package
(``panostitcher_gb300``) never imports it.

The C library (``ps_oracle.c``) restates, in plain C, the reference's
CudaAccel integer semantics (``source/CudaAccel/CudaPyramid2.cu``,
``source/CudaAccel/CudaMultibandBlend.cpp``), its double-precision bilinear
remap (``source/Warp/ZReproject.cpp:101-130``) and its PanoTools geometry
(``source/Warp/Remap.cpp``).  It is pinned against the reference's own
code: ``oracle/ref.py`` builds the reference's geometry, remap, pyramid and
YUV sources unchanged into ``oracle/_ref/`` (where the reference tree is
present), ``tests/test_ref_pin.py`` compares the two bit for bit, and the
fixtures of ``tests/golden/`` are that build's outputs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpsoracle.so")
_lib = None
_lock = threading.Lock()


class OrcParam(C.Structure):
    """PhotoParam (source/Warp/ZReproject.h:17-50), same field order."""

    _fields_ = [(n, C.c_int) for n in ("imageType", "cropMode", "cropX", "cropY", "cropWidth",
                                       "cropHeight", "circleX", "circleY", "circleR")] + \
               [(n, C.c_double) for n in ("hfov", "vfov", "alpha", "beta", "gamma", "shiftX",
                                          "shiftY", "shearX", "shearY", "yaw", "pitch", "roll")]


_PARAM_KEYS = {
    "image_type": "imageType", "crop_mode": "cropMode", "crop_x": "cropX", "crop_y": "cropY",
    "crop_width": "cropWidth", "crop_height": "cropHeight", "circle_x": "circleX",
    "circle_y": "circleY", "circle_r": "circleR", "shift_x": "shiftX", "shift_y": "shiftY",
    "shear_x": "shearX", "shear_y": "shearY",
}


def make_param(p: dict) -> OrcParam:
    """Build an OrcParam from a dict with snake_case PhotoParam keys."""
    out = OrcParam()
    for k, v in p.items():
        setattr(out, _PARAM_KEYS.get(k, k), v)
    return out


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f))
                                              for f in ("ps_oracle.c", "ps_oracle_cpu.c", "ps_oracle.h", "Makefile")):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            P = C.POINTER
            vp = C.c_void_p
            L.orc_reproject_map.argtypes = [P(OrcParam), C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp]
            L.orc_nearest_axis_seams.argtypes = [P(OrcParam), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]
            L.orc_reproject_map_rows.argtypes = [P(OrcParam), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                 vp, vp, vp, vp]
            L.orc_nearest_axis_seams_rows.argtypes = [P(OrcParam), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                                      C.c_int, C.c_int, vp, vp]
            L.orc_get_lut.argtypes = [C.c_double, vp]
            L.orc_reproject_bilinear_16s.argtypes = [vp, C.c_int, C.c_int, C.c_longlong, C.c_int, vp, vp, vp,
                                                     C.c_int, C.c_int, vp]
            L.orc_num_levels.argtypes = [C.c_int] * 4
            L.orc_num_levels.restype = C.c_int
            for name in ("orc_pyr_down_16sc1_to_32sc1", "orc_pyr_down_16sc1_to_16sc1",
                         "orc_pyr_up_16sc4", "orc_pyr_up_32sc4"):
                getattr(L, name).argtypes = [vp, C.c_int, C.c_int, vp, C.c_int, C.c_int]
            L.orc_pyr_down_16sc4_masked.argtypes = [vp, C.c_int, C.c_int, vp, vp, C.c_int, C.c_int]
            L.orc_mb_prepare.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
            L.orc_mb_prepare.restype = vp
            L.orc_mb_free.argtypes = [vp]
            L.orc_mb_set_custom_masks.argtypes = [vp, vp]
            L.orc_mb_set_custom_masks.restype = C.c_int
            L.orc_mb_num_levels.argtypes = [vp]
            L.orc_mb_num_levels.restype = C.c_int
            L.orc_mb_full_mask.argtypes = [vp]
            L.orc_mb_full_mask.restype = C.c_int
            L.orc_mb_get_alpha.argtypes = [vp, C.c_int, C.c_int, vp]
            L.orc_mb_get_weight.argtypes = [vp, C.c_int, C.c_int, vp]
            L.orc_mb_blend.argtypes = [vp, vp, vp, vp, vp]
            L.orc_mb_blend_mt.argtypes = [vp, vp, vp, C.c_int]
            L.orc_render.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int]
            L.orc_cpu_mb_prepare.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
            L.orc_cpu_mb_prepare.restype = vp
            L.orc_cpu_mb_free.argtypes = [vp]
            L.orc_cpu_mb_num_levels.argtypes = [vp]
            L.orc_cpu_mb_num_levels.restype = C.c_int
            L.orc_cpu_mb_full_mask.argtypes = [vp]
            L.orc_cpu_mb_full_mask.restype = C.c_int
            L.orc_cpu_mb_get_weight.argtypes = [vp, C.c_int, C.c_int, vp]
            L.orc_cpu_mb_get_alpha.argtypes = [vp, C.c_int, C.c_int, vp]
            L.orc_cpu_mb_blend.argtypes = [vp, vp, vp, vp, C.c_int]
            L.orc_cpu_render.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int]
            L.orc_linear_weights.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp]
            L.orc_linear_render.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int,
                                            vp]
            L.orc_distance_transform_l1.argtypes = [vp, C.c_int, C.c_int, vp]
            L.orc_non_intersecting_masks.argtypes = [vp, C.c_int, C.c_int, C.c_int, vp]
            L.orc_bgr32_to_yuv.argtypes = [vp, C.c_longlong, C.c_int, C.c_int, C.c_int, vp, C.c_longlong, vp,
                                           C.c_longlong, vp, C.c_longlong]
            L.orc_yuv_to_bgr32.argtypes = [vp, C.c_longlong, vp, C.c_longlong, vp, C.c_longlong, C.c_int, C.c_int,
                                           C.c_int, vp, C.c_longlong]
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def _ptr_array(arrs):
    return (C.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


# ---------------------------------------------------------------- geometry
def _row_bands(H: int, threads: int):
    k = max(1, min(threads, H))
    return [(H * i // k, H * (i + 1) // k) for i in range(k)]


def _run_bands(fn, H: int, threads: int):
    bands = _row_bands(H, threads)
    if len(bands) == 1:
        fn(*bands[0])
        return
    from concurrent.futures import ThreadPoolExecutor  # ctypes calls release the GIL
    with ThreadPoolExecutor(max_workers=len(bands)) as ex:
        list(ex.map(lambda b: fn(*b), bands))


def reproject_map(param: dict, cam_size, canvas_size, with_double: bool = False, threads: int = 1):
    """getReprojectMap32FAndMask: float x/y maps (-1 sentinel) and 0/255 mask (row bands on `threads`)."""
    cw, ch = cam_size
    W, H = canvas_size
    xm = np.empty((H, W), np.float32)
    ym = np.empty((H, W), np.float32)
    mk = np.empty((H, W), np.uint8)
    m64 = np.empty((H, W, 2), np.float64) if with_double else None
    p = make_param(param)
    L = lib()
    _run_bands(lambda r0, r1: L.orc_reproject_map_rows(C.byref(p), cw, ch, W, H, r0, r1,
                                                       _ptr(m64) if with_double else None, _ptr(xm), _ptr(ym),
                                                       _ptr(mk)), H, threads)
    return (xm, ym, mk, m64) if with_double else (xm, ym, mk)


def nearest_axis_seams(params, cam_size, canvas_size, coverage: np.ndarray, threads: int = 1) -> np.ndarray:
    n = len(params)
    W, H = canvas_size
    arr = (OrcParam * n)(*[make_param(p) for p in params])
    cov = np.ascontiguousarray(coverage, dtype=np.uint8)
    seams = np.empty((n, H, W), np.uint8)
    L = lib()
    _run_bands(lambda r0, r1: L.orc_nearest_axis_seams_rows(arr, n, cam_size[0], cam_size[1], W, H, r0, r1,
                                                            _ptr(cov), _ptr(seams)), H, threads)
    return seams


def get_lut(k: float) -> np.ndarray:
    out = np.empty(256, np.uint8)
    lib().orc_get_lut(float(k), _ptr(out))
    return out


# ------------------------------------------------------------------- reference seams
DT_FAR = 1 << 28


def distance_transform_l1(mask: np.ndarray) -> np.ndarray:
    """L1 distance of every pixel to the nearest zero pixel (int32; DT_FAR + d without zeros)."""
    m = np.ascontiguousarray(mask, np.uint8)
    H, W = m.shape
    out = np.empty((H, W), np.int32)
    lib().orc_distance_transform_l1(_ptr(m), W, H, _ptr(out))
    return out


def non_intersecting_masks(masks: np.ndarray) -> np.ndarray:
    """getNonIntersectingMasks: (n, H, W) coverage -> (n, H, W) 0/255 unique masks."""
    m = np.ascontiguousarray(masks, np.uint8)
    n, H, W = m.shape
    out = np.empty_like(m)
    lib().orc_non_intersecting_masks(_ptr(m), n, W, H, _ptr(out))
    return out


# ------------------------------------------------------------------- linear blend
def linear_weights(coverage: np.ndarray, seams: np.ndarray, radius: int) -> np.ndarray:
    """getWeightsLinearBlend32F over given masks: (n, H, W) float32 weights."""
    cov = np.ascontiguousarray(coverage, np.uint8)
    sm = np.ascontiguousarray(seams, np.uint8)
    n, H, W = cov.shape
    out = np.empty((n, H, W), np.float32)
    lib().orc_linear_weights(_ptr(cov), _ptr(sm), n, W, H, int(radius), _ptr(out))
    return out


def linear_render(srcs, luts, xmaps, ymaps, weights: np.ndarray) -> np.ndarray:
    """The linear-blend render (BGR32 (H, W, 4))."""
    srcs = [np.ascontiguousarray(s, np.uint8) for s in srcs]
    n = len(srcs)
    sh, sw, chn = srcs[0].shape
    H, W = xmaps[0].shape
    xs = [np.ascontiguousarray(m, np.float32) for m in xmaps]
    ys = [np.ascontiguousarray(m, np.float32) for m in ymaps]
    w = np.ascontiguousarray(weights, np.float32)
    lt = None if luts is None else np.ascontiguousarray(luts, np.uint8)
    dst = np.empty((H, W, 4), np.uint8)
    lib().orc_linear_render(_ptr_array(srcs), sw, sh, chn, None if lt is None else _ptr(lt), _ptr_array(xs),
                            _ptr_array(ys), _ptr(w), n, W, H, _ptr(dst))
    return dst


# ------------------------------------------------------------------- encoder handoff
FMT_YUV420P = 420
FMT_NV12 = 12


def bgr32_to_yuv(bgr: np.ndarray, fmt: int = FMT_YUV420P):
    """BGR32 HxWx4 -> (Y, U, V) planes (YUV420P) or (Y, UV) planes (NV12)."""
    bgr = np.ascontiguousarray(bgr, np.uint8)
    H, W, chn = bgr.shape
    if chn != 4 or H % 2 or W % 2:
        raise ValueError("BGR32 image with even width and height expected")
    y = np.empty((H, W), np.uint8)
    if fmt == FMT_NV12:
        uv = np.empty((H // 2, W), np.uint8)
        lib().orc_bgr32_to_yuv(_ptr(bgr), W * 4, W, H, fmt, _ptr(y), W, _ptr(uv), W, None, 0)
        return y, uv
    u = np.empty((H // 2, W // 2), np.uint8)
    v = np.empty((H // 2, W // 2), np.uint8)
    lib().orc_bgr32_to_yuv(_ptr(bgr), W * 4, W, H, FMT_YUV420P, _ptr(y), W, _ptr(u), W // 2, _ptr(v), W // 2)
    return y, u, v


def yuv_to_bgr32(planes, fmt: int = FMT_YUV420P) -> np.ndarray:
    """(Y, U, V) planes (YUV420P) or (Y, UV) planes (NV12) -> BGR32 HxWx4 (fourth byte 0)."""
    planes = [np.ascontiguousarray(p, np.uint8) for p in planes]
    H, W = planes[0].shape
    if H % 2 or W % 2:
        raise ValueError("even width and height expected")
    out = np.empty((H, W, 4), np.uint8)
    if fmt == FMT_NV12:
        y, uv = planes
        assert uv.shape == (H // 2, W)
        lib().orc_yuv_to_bgr32(_ptr(y), W, _ptr(uv), W, None, 0, W, H, fmt, _ptr(out), W * 4)
    else:
        y, u, v = planes
        assert u.shape == (H // 2, W // 2) and v.shape == (H // 2, W // 2)
        lib().orc_yuv_to_bgr32(_ptr(y), W, _ptr(u), W // 2, _ptr(v), W // 2, W, H, FMT_YUV420P, _ptr(out), W * 4)
    return out


# ------------------------------------------------------------------- remap
def reproject_16s(src: np.ndarray, xmap: np.ndarray, ymap: np.ndarray, lut: np.ndarray | None = None):
    """LUT (3x256 B,G,R) on the source, then double bilinear -> int16 HxWx4."""
    src = np.ascontiguousarray(src)
    sh, sw, chn = src.shape
    H, W = xmap.shape
    out = np.empty((H, W, 4), np.int16)
    lt = None if lut is None else np.ascontiguousarray(lut, np.uint8).reshape(3, 256)
    lib().orc_reproject_bilinear_16s(_ptr(src), sw, sh, sw * chn, chn, None if lt is None else _ptr(lt),
                                     _ptr(np.ascontiguousarray(xmap, np.float32)),
                                     _ptr(np.ascontiguousarray(ymap, np.float32)), W, H, _ptr(out))
    return out


# ---------------------------------------------------------------- pyramids
def num_levels(width, height, max_levels, min_length=2):
    return lib().orc_num_levels(width, height, max_levels, min_length)


def down_size(w, h):
    return (w + 1) // 2, (h + 1) // 2


def pyr_down_16sc1_to_32sc1(src: np.ndarray) -> np.ndarray:
    sh, sw = src.shape
    dw, dh = down_size(sw, sh)
    out = np.empty((dh, dw), np.int32)
    lib().orc_pyr_down_16sc1_to_32sc1(_ptr(np.ascontiguousarray(src, np.int16)), sw, sh, _ptr(out), dw, dh)
    return out


def pyr_down_16sc1_to_16sc1(src: np.ndarray) -> np.ndarray:
    sh, sw = src.shape
    dw, dh = down_size(sw, sh)
    out = np.empty((dh, dw), np.int16)
    lib().orc_pyr_down_16sc1_to_16sc1(_ptr(np.ascontiguousarray(src, np.int16)), sw, sh, _ptr(out), dw, dh)
    return out


def pyr_down_16sc4_masked(src: np.ndarray, scale: np.ndarray) -> np.ndarray:
    sh, sw, _ = src.shape
    dh, dw = scale.shape
    out = np.empty((dh, dw, 4), np.int16)
    lib().orc_pyr_down_16sc4_masked(_ptr(np.ascontiguousarray(src, np.int16)), sw, sh,
                                    _ptr(np.ascontiguousarray(scale, np.int32)), _ptr(out), dw, dh)
    return out


def pyr_up_16sc4(src: np.ndarray, dst_size) -> np.ndarray:
    sh, sw, _ = src.shape
    dw, dh = dst_size
    out = np.empty((dh, dw, 4), np.int16)
    lib().orc_pyr_up_16sc4(_ptr(np.ascontiguousarray(src, np.int16)), sw, sh, _ptr(out), dw, dh)
    return out


def pyr_up_32sc4(src: np.ndarray, dst_size) -> np.ndarray:
    sh, sw, _ = src.shape
    dw, dh = dst_size
    out = np.empty((dh, dw, 4), np.int32)
    lib().orc_pyr_up_32sc4(_ptr(np.ascontiguousarray(src, np.int32)), sw, sh, _ptr(out), dw, dh)
    return out


def level_sizes(w, h, levels):
    sizes = [(w, h)]
    for _ in range(levels):
        w, h = down_size(w, h)
        sizes.append((w, h))
    return sizes


# ------------------------------------------------------------------- blend
class Blender:
    """CudaTilingMultibandBlendFast restated: prepare(masks) + blend(images)."""

    def __init__(self, masks: np.ndarray, seams: np.ndarray, max_levels: int, min_length: int = 2):
        masks = np.ascontiguousarray(masks, np.uint8)
        seams = np.ascontiguousarray(seams, np.uint8)
        self.n, self.H, self.W = masks.shape
        self._masks, self._seams = masks, seams
        self._h = lib().orc_mb_prepare(_ptr(masks), _ptr(seams), self.n, self.W, self.H, max_levels, min_length)
        if not self._h:
            raise ValueError("oracle prepare failed")
        self.levels = lib().orc_mb_num_levels(self._h)
        self.full_mask = bool(lib().orc_mb_full_mask(self._h))
        self.sizes = level_sizes(self.W, self.H, self.levels)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_mb_free(h)
            self._h = None

    def set_custom_masks(self, masks) -> None:
        """blend(images, masks, blendImage) (CudaMultibandBlend.cpp:825-893): later blends weight the
        cameras by these (n, H, W) masks, normalise by the weight sums and zero the pixels outside the
        masks' union; None restores the prepared unique masks."""
        if masks is None:
            lib().orc_mb_set_custom_masks(self._h, None)
        else:
            m = np.ascontiguousarray(masks, np.uint8)
            if m.shape != (self.n, self.H, self.W):
                raise ValueError(f"custom masks of shape {(self.n, self.H, self.W)} expected")
            lib().orc_mb_set_custom_masks(self._h, _ptr(m))
        self.full_mask = bool(lib().orc_mb_full_mask(self._h))

    def alpha(self, cam: int, level: int) -> np.ndarray:
        w, h = self.sizes[level]
        out = np.empty((h, w), np.int32)
        lib().orc_mb_get_alpha(self._h, cam, level, _ptr(out))
        return out

    def weight(self, cam: int, level: int) -> np.ndarray:
        w, h = self.sizes[level]
        out = np.empty((h, w), np.int16)
        lib().orc_mb_get_weight(self._h, cam, level, _ptr(out))
        return out

    def _split(self, flat: np.ndarray):
        out, off = [], 0
        for (w, h) in self.sizes:
            out.append(flat[off:off + w * h].reshape(h, w, 4))
            off += w * h
        return out

    def blend(self, images, pyramids: bool = False, nthreads: int = 1):
        imgs = [np.ascontiguousarray(im, np.int16) for im in images]
        assert len(imgs) == self.n
        dst = np.empty((self.H, self.W, 4), np.uint8)
        if pyramids:
            tot = sum(w * h for (w, h) in self.sizes)
            norm = np.empty((tot, 4), np.int32)
            coll = np.empty((tot, 4), np.int32)
            lib().orc_mb_blend(self._h, _ptr_array(imgs), _ptr(dst), _ptr(norm), _ptr(coll))
            return dst, self._split(norm), self._split(coll)
        if nthreads > 1:
            lib().orc_mb_blend_mt(self._h, _ptr_array(imgs), _ptr(dst), nthreads)
        else:
            lib().orc_mb_blend(self._h, _ptr_array(imgs), _ptr(dst), None, None)
        return dst

    def render(self, srcs, luts, xmaps, ymaps, nthreads: int = 1) -> np.ndarray:
        """LUT -> bilinear remap -> blend, the CPUPanoramaRender dataflow."""
        srcs = [np.ascontiguousarray(s, np.uint8) for s in srcs]
        sh, sw, chn = srcs[0].shape
        xm = [np.ascontiguousarray(x, np.float32) for x in xmaps]
        ym = [np.ascontiguousarray(y, np.float32) for y in ymaps]
        lt = None if luts is None else np.ascontiguousarray(luts, np.uint8).reshape(self.n, 3, 256)
        dst = np.empty((self.H, self.W, 4), np.uint8)
        lib().orc_render(self._h, _ptr_array(srcs), sw, sh, chn, None if lt is None else _ptr(lt),
                         _ptr_array(xm), _ptr_array(ym), _ptr(dst), nthreads)
        return dst


class CpuBlender:
    """TilingMultibandBlendFast restated (the reference's CPU twin of the blend,
    source/Blend/MultiBandBlend.cpp:906-1031): prepare(masks) + blend(images).

    Its arithmetic differs from the CudaAccel semantics that Blender restates
    and the product computes (x255 masked pyrDown, R >> 8 full-mask
    normalisation, saturating Laplacian, OpenCV borders); it serves the
    secondary difference histogram and the timed reference CPU path."""

    def __init__(self, masks: np.ndarray, seams: np.ndarray, max_levels: int, min_length: int = 2):
        masks = np.ascontiguousarray(masks, np.uint8)
        seams = np.ascontiguousarray(seams, np.uint8)
        self.n, self.H, self.W = masks.shape
        self._h = lib().orc_cpu_mb_prepare(_ptr(masks), _ptr(seams), self.n, self.W, self.H, max_levels,
                                           min_length)
        if not self._h:
            raise ValueError("oracle prepare failed")
        self.levels = lib().orc_cpu_mb_num_levels(self._h)
        self.full_mask = bool(lib().orc_cpu_mb_full_mask(self._h))
        self.sizes = level_sizes(self.W, self.H, self.levels)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_cpu_mb_free(h)
            self._h = None

    def weight(self, cam: int, level: int) -> np.ndarray:
        w, h = self.sizes[level]
        out = np.empty((h, w), np.int16)
        lib().orc_cpu_mb_get_weight(self._h, cam, level, _ptr(out))
        return out

    def alpha(self, cam: int, level: int) -> np.ndarray:
        w, h = self.sizes[level]
        out = np.empty((h, w), np.int32)
        lib().orc_cpu_mb_get_alpha(self._h, cam, level, _ptr(out))
        return out

    def blend(self, images, pyramids: bool = False, nthreads: int = 1):
        """BGR32 (H, W, 4) blend of n (H, W, 4) int16 level-0 images; with ``pyramids`` also the
        collapsed int32x3 result pyramid, level by level."""
        imgs = [np.ascontiguousarray(im, np.int16) for im in images]
        assert len(imgs) == self.n
        dst = np.empty((self.H, self.W, 4), np.uint8)
        if not pyramids:
            lib().orc_cpu_mb_blend(self._h, _ptr_array(imgs), _ptr(dst), None, nthreads)
            return dst
        tot = sum(w * h for (w, h) in self.sizes)
        coll = np.empty((tot, 3), np.int32)
        lib().orc_cpu_mb_blend(self._h, _ptr_array(imgs), _ptr(dst), _ptr(coll), nthreads)
        out, off = [], 0
        for (w, h) in self.sizes:
            out.append(coll[off:off + w * h].reshape(h, w, 3))
            off += w * h
        return dst, out

    def render(self, srcs, luts, xmaps, ymaps, nthreads: int = 1) -> np.ndarray:
        """CPUPanoramaRender::render: LUT -> bilinear remap to int16 -> this blend."""
        srcs = [np.ascontiguousarray(s, np.uint8) for s in srcs]
        sh, sw, chn = srcs[0].shape
        xm = [np.ascontiguousarray(x, np.float32) for x in xmaps]
        ym = [np.ascontiguousarray(y, np.float32) for y in ymaps]
        lt = None if luts is None else np.ascontiguousarray(luts, np.uint8).reshape(self.n, 3, 256)
        dst = np.empty((self.H, self.W, 4), np.uint8)
        lib().orc_cpu_render(self._h, _ptr_array(srcs), sw, sh, chn, None if lt is None else _ptr(lt),
                             _ptr_array(xm), _ptr_array(ym), _ptr(dst), nthreads)
        return dst
