"""The reference's own code, built here as the oracle's pin -- TEST INFRASTRUCTURE ONLY.

``oracle/Makefile``'s ``ref`` target compiles, unchanged and from where they
lie in the reference tree, the reference's geometry and CPU remap
(``source/Warp/Remap.cpp``, ``source/Warp/ZReproject.cpp``), its integer
pyramid kernels with their host wrappers (``source/CudaAccel/CudaPyramid2.cu``,
``CudaUtil.cuh``), its YUV conversions (``source/CudaAccel/ImageProc.cu``) and
its CPU multiband blend (``source/Blend/MultiBandBlend.cpp`` with
``Pyramid.cpp``) into ``oracle/_ref/libpsref.so``.  OpenCV is replaced by ``oracle/ref/cv_shim``
and the CUDA runtime by ``oracle/ref/cuda_emu``, which runs the kernels on host
cores.  ``oracle/ref/ref_driver.cpp`` chains them as the reference's callers do.

The library exists only where the reference tree does; ``available()``
says whether it was built.  ``tests/test_ref_pin.py`` compares the oracle
with it directly, and ``tests/golden/make_golden.py`` writes its outputs as
committed fixtures, so that the pin also holds where the reference tree is
absent (``tests/test_golden.py``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from . import OrcParam, make_param

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_ref", "libpsref.so")
_REF_SRC = os.environ.get("PS_REFERENCE_SOURCE", "/root/reference/source")
_lib = None
_lock = threading.Lock()

FMT_YUV420P = 420
FMT_NV12 = 12


def source_present() -> bool:
    return os.path.isfile(os.path.join(_REF_SRC, "CudaAccel", "CudaPyramid2.cu"))


def build(force: bool = False) -> str | None:
    """Build oracle/_ref/libpsref.so when the reference tree is present; return its path or None."""
    if not source_present():
        return _LIB_PATH if os.path.exists(_LIB_PATH) else None
    cmd = ["make", "-s", "-C", _HERE, "ref", f"REF_SRC={_REF_SRC}"]
    if force:
        cmd.insert(3, "-B")
    subprocess.run(cmd, check=True)
    return _LIB_PATH


def available() -> bool:
    try:
        return lib() is not None
    except OSError:
        return False


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            if path is None or not os.path.exists(path):
                return None
            L = C.CDLL(path)
            vp, i = C.c_void_p, C.c_int
            L.psref_num_threads.argtypes = [i]
            L.psref_num_threads.restype = i
            L.psref_reproject_map.argtypes = [C.POINTER(OrcParam), i, i, i, i, vp, vp]
            L.psref_reproject_16s.argtypes = [vp, i, i, i, vp, i, i, vp]
            L.psref_mb_blend.argtypes = [i, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
            L.psref_cpu_mb_blend.argtypes = [i, i, i, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
            L.psref_bgr32_to_yuv.argtypes = [vp, i, i, i, vp, vp, vp]
            L.psref_yuv_to_bgr32.argtypes = [vp, vp, vp, i, i, i, vp]
            for name in ("psref_reproject_map", "psref_reproject_16s", "psref_mb_blend", "psref_cpu_mb_blend",
                         "psref_bgr32_to_yuv", "psref_yuv_to_bgr32"):
                getattr(L, name).restype = i
            _lib = L
    return _lib


def _need():
    L = lib()
    if L is None:
        raise RuntimeError("the reference build (oracle/_ref) is not available here")
    return L


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"reference {what} failed (a CV_Assert or an exception)")


def num_threads(n: int = 0) -> int:
    return _need().psref_num_threads(int(n))


def reproject_map(param: dict, cam_size, canvas_size):
    """getReprojectMapAndMask: (H, W, 2) float64 dst->src map (-1 outside) and (H, W) 0/255 mask."""
    W, H = canvas_size
    m = np.empty((H, W, 2), np.float64)
    k = np.empty((H, W), np.uint8)
    p = make_param(param)
    _check(_need().psref_reproject_map(C.byref(p), cam_size[0], cam_size[1], W, H, _ptr(m), _ptr(k)),
           "getReprojectMapAndMask")
    return m, k


def reproject_16s(src: np.ndarray, map64: np.ndarray) -> np.ndarray:
    """reprojectParallelTo16S: bilinear int16 samples (H, W, C) of an (h, w, C) byte image."""
    src = np.ascontiguousarray(src, np.uint8)
    sh, sw, chn = src.shape
    m = np.ascontiguousarray(map64, np.float64)
    H, W, _ = m.shape
    out = np.empty((H, W, chn), np.int16)
    _check(_need().psref_reproject_16s(_ptr(src), sw, sh, chn, _ptr(m), W, H, _ptr(out)), "reprojectParallelTo16S")
    return out


def _level_sizes(W, H, levels):
    sizes = [(W, H)]
    for _ in range(levels):
        W, H = (W + 1) // 2, (H + 1) // 2
        sizes.append((W, H))
    return sizes


def _split(flat, sizes, ch):
    out, off = [], 0
    for (w, h) in sizes:
        n = w * h
        out.append(flat[off:off + n].reshape((h, w, ch) if ch > 1 else (h, w)))
        off += n
    return out


def mb_blend(masks: np.ndarray, seams: np.ndarray, images, levels: int, pyramids: bool = False):
    """CudaTilingMultibandBlendFast::prepare + blend through the reference's pyramid wrappers.

    masks / seams: (n, H, W) coverage and unique masks; images: n (H, W, 4)
    int16 level-0 images.  Returns the BGR32 (H, W, 4) blend, and with
    ``pyramids`` also a dict of the normalised and collapsed int32x4 result
    pyramids and the per-camera weight (int16) and alpha (int32) pyramids.
    """
    masks = np.ascontiguousarray(masks, np.uint8)
    seams = np.ascontiguousarray(seams, np.uint8)
    n, H, W = masks.shape
    imgs = np.ascontiguousarray(np.stack([np.asarray(im, np.int16) for im in images]))
    assert imgs.shape == (n, H, W, 4)
    sizes = _level_sizes(W, H, levels)
    tot = sum(w * h for (w, h) in sizes)
    out = np.empty((H, W, 4), np.uint8)
    if not pyramids:
        _check(_need().psref_mb_blend(n, W, H, levels, _ptr(masks), _ptr(seams), _ptr(imgs), _ptr(out),
                                      None, None, None, None), "multiband blend")
        return out
    coll = np.empty((tot, 4), np.int32)
    norm = np.empty((tot, 4), np.int32)
    wts = np.empty((n, tot), np.int16)
    als = np.empty((n, tot), np.int32)
    _check(_need().psref_mb_blend(n, W, H, levels, _ptr(masks), _ptr(seams), _ptr(imgs), _ptr(out),
                                  _ptr(coll), _ptr(norm), _ptr(wts), _ptr(als)), "multiband blend")
    return out, {
        "norm": _split(norm, sizes, 4),
        "coll": _split(coll, sizes, 4),
        "weight": [_split(wts[i], sizes, 1) for i in range(n)],
        "alpha": [_split(als[i], sizes, 1) for i in range(n)],
    }


def cpu_mb_blend(masks: np.ndarray, seams: np.ndarray, images, max_levels: int, min_length: int = 2):
    """The reference's TilingMultibandBlendFast: prepare(masks, max_levels, min_length) + blend(images).

    masks / seams: (n, H, W) coverage and unique masks; images: n (H, W, 4)
    int16 level-0 images (B, G, R used).  Returns the BGR32 (H, W, 4) blend
    and a dict of the collapsed int32x3 result pyramid and the per-camera
    weight (int16) and alpha (int32) pyramids.
    """
    masks = np.ascontiguousarray(masks, np.uint8)
    seams = np.ascontiguousarray(seams, np.uint8)
    n, H, W = masks.shape
    imgs = np.ascontiguousarray(np.stack([np.asarray(im, np.int16) for im in images]))
    assert imgs.shape == (n, H, W, 4)
    from . import num_levels
    sizes = _level_sizes(W, H, num_levels(W, H, max_levels, min_length))
    tot = sum(w * h for (w, h) in sizes)
    out = np.empty((H, W, 4), np.uint8)
    coll = np.empty((tot, 3), np.int32)
    wts = np.empty((n, tot), np.int16)
    als = np.empty((n, tot), np.int32)
    levels = C.c_int(-1)
    _check(_need().psref_cpu_mb_blend(n, W, H, max_levels, min_length, _ptr(masks), _ptr(seams), _ptr(imgs),
                                      _ptr(out), _ptr(coll), _ptr(wts), _ptr(als), C.byref(levels)),
           "TilingMultibandBlendFast")
    assert levels.value == len(sizes) - 1
    return out, {
        "coll": _split(coll, sizes, 3),
        "weight": [_split(wts[i], sizes, 1) for i in range(n)],
        "alpha": [_split(als[i], sizes, 1) for i in range(n)],
    }


def bgr32_to_yuv(bgr: np.ndarray, fmt: int = FMT_YUV420P):
    bgr = np.ascontiguousarray(bgr, np.uint8)
    H, W, _ = bgr.shape
    y = np.empty((H, W), np.uint8)
    if fmt == FMT_NV12:
        uv = np.empty((H // 2, W), np.uint8)
        _check(_need().psref_bgr32_to_yuv(_ptr(bgr), W, H, fmt, _ptr(y), _ptr(uv), None), "cvtBGR32ToNV12")
        return y, uv
    u = np.empty((H // 2, W // 2), np.uint8)
    v = np.empty((H // 2, W // 2), np.uint8)
    _check(_need().psref_bgr32_to_yuv(_ptr(bgr), W, H, fmt, _ptr(y), _ptr(u), _ptr(v)), "cvtBGR32ToYUV420P")
    return y, u, v


def yuv_to_bgr32(planes, fmt: int = FMT_YUV420P) -> np.ndarray:
    planes = [np.ascontiguousarray(p, np.uint8) for p in planes]
    H, W = planes[0].shape
    out = np.empty((H, W, 4), np.uint8)
    if fmt == FMT_NV12:
        y, uv = planes
        _check(_need().psref_yuv_to_bgr32(_ptr(y), _ptr(uv), None, W, H, fmt, _ptr(out)), "cvtNV12ToBGR32")
    else:
        y, u, v = planes
        _check(_need().psref_yuv_to_bgr32(_ptr(y), _ptr(u), _ptr(v), W, H, fmt, _ptr(out)), "cvtYUV420PToBGR32")
    return out
