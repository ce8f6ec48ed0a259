"""Host-side mirror of the reference's render interface over the C ABI.

``CudaPanoramaRender2`` keeps the method names, argument meaning and
bool-returning error behaviour of the reference class
(source/Task/RicohUtil.h:193-220): ``prepare`` / ``render`` return False and
record the reason in ``last_error`` (the reference logs it with lprintf).
Pass ``check=True`` to raise ``PsError`` instead.

Images are numpy uint8 arrays (host memory) or CUDA tensors with a
``data_ptr()`` (device memory), shaped (H, W, 3) for BGR24 or (H, W, 4) for
BGR32.  All work runs in libpanostitch.so; nothing here computes pixels.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib as L
from ._lib import PhotoParam, Image, PlanarImage, PsError, check, lib


def _require(ok: bool, what: str) -> None:
    """Argument checks that stay on under python -O (ValueError, like the other shape errors here)."""
    if not ok:
        raise ValueError(what)


def _is_device(a) -> bool:
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def as_image(a) -> Image:
    """ps_image view of a numpy array (host) or a CUDA tensor (device)."""
    if _is_device(a):
        _require(a.dim() == 3 and a.shape[2] in (3, 4) and a.stride(2) == 1 and a.stride(1) == a.shape[2]
                 and a.element_size() == 1, "a device image is a uint8 (H, W, 3 or 4) tensor with dense rows")
        return Image(a.data_ptr(), a.stride(0) * a.element_size(), a.shape[1], a.shape[0],
                     L.PS_FMT_BGR32 if a.shape[2] == 4 else L.PS_FMT_BGR24, L.PS_MEM_DEVICE)
    _require(isinstance(a, np.ndarray) and a.dtype == np.uint8 and a.ndim == 3 and a.shape[2] in (3, 4)
             and a.strides[2] == 1 and a.strides[1] == a.shape[2],
             "a host image is a uint8 (H, W, 3 or 4) numpy array with dense rows")
    return Image(a.ctypes.data, a.strides[0], a.shape[1], a.shape[0],
                 L.PS_FMT_BGR32 if a.shape[2] == 4 else L.PS_FMT_BGR24, L.PS_MEM_HOST)


def as_planar(planes: Sequence, fmt: int) -> PlanarImage:
    """ps_planar_image view of (Y, U, V) or (Y, UV) 2-D uint8 planes, all numpy
    (host) or all CUDA tensors (device); the luma plane sets the size."""
    want = 2 if fmt == L.PS_FMT_NV12 else 3
    if len(planes) != want:
        raise ValueError(f"{want} planes expected for format {fmt}")
    dev = _is_device(planes[0])
    ptrs, pitches = [], []
    for p in planes:
        if _is_device(p) != dev:
            raise ValueError("planes must all be host arrays or all CUDA tensors")
        if dev:
            _require(p.dim() == 2 and p.stride(1) == 1 and p.element_size() == 1,
                     "a device plane is a 2-D uint8 tensor with dense rows")
            ptrs.append(p.data_ptr())
            pitches.append(p.stride(0))
        else:
            _require(isinstance(p, np.ndarray) and p.dtype == np.uint8 and p.ndim == 2 and p.strides[1] == 1,
                     "a host plane is a 2-D uint8 numpy array with dense rows")
            ptrs.append(p.ctypes.data)
            pitches.append(p.strides[0])
    while len(ptrs) < 3:
        ptrs.append(None)
        pitches.append(0)
    im = PlanarImage()
    im.planes[:] = ptrs
    im.pitches[:] = pitches
    im.height, im.width = int(planes[0].shape[0]), int(planes[0].shape[1])
    im.format = fmt
    im.location = L.PS_MEM_DEVICE if dev else L.PS_MEM_HOST
    return im


def _stream_handle(stream):
    if stream is None:
        return None
    return getattr(stream, "cuda_stream", stream)


def _params(params: Sequence[dict]):
    arr = (PhotoParam * len(params))(*[PhotoParam.from_dict(p) for p in params])
    return arr


def _luts_arg(luts, n):
    if luts is None:
        return None, 0, None
    a = np.ascontiguousarray(luts, dtype=np.uint8)
    if a.size % 768:
        return a, -1, None
    return a, a.size // 768, a.ctypes.data


def _mask_ptrs(masks):
    """Host uint8 masks -> (kept arrays, void* array, count); None -> (None, None, 0)."""
    if masks is None:
        return None, None, 0
    ms = [np.ascontiguousarray(m, np.uint8) for m in masks]
    return ms, (C.c_void_p * len(ms))(*[m.ctypes.data for m in ms]), len(ms)


class CudaPanoramaRender2:
    """CudaPanoramaRender2 (source/Task/RicohUtil.h:193-220) over libpanostitch."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().ps_render_create(C.byref(h)))
        self._h = h
        self.last_error = ""

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().ps_render_destroy(h)
            except Exception:
                pass
            self._h = None

    def _status(self, status: int, check_: bool) -> bool:
        if status == L.PS_OK:
            return True
        self.last_error = lib().ps_last_error().decode(errors="replace")
        if check_:
            raise PsError(status, self.last_error)
        return False

    # -- reference methods -------------------------------------------------
    def prepare(self, params: Sequence[dict], high_quality_blend: int, blend_param: int, src_size, dst_size,
                seams=None, stream=None, check: bool = False) -> bool:
        """prepare(params, highQualityBlend, blendParam, srcSize, dstSize); sizes are (w, h)."""
        arr = _params(params)
        self._size = tuple(dst_size)
        if seams is None:
            st = lib().ps_render_prepare(self._h, arr, len(params), high_quality_blend, blend_param,
                                         src_size[0], src_size[1], dst_size[0], dst_size[1],
                                         _stream_handle(stream))
        else:
            ms = [np.ascontiguousarray(m, np.uint8) for m in seams]
            ptrs = (C.c_void_p * len(ms))(*[m.ctypes.data for m in ms])
            st = lib().ps_render_prepare_with_seams(self._h, arr, len(params), high_quality_blend, blend_param,
                                                    src_size[0], src_size[1], dst_size[0], dst_size[1], ptrs,
                                                    _stream_handle(stream))
        return self._status(st, check)

    def prepare_file(self, path: str, high_quality_blend: int, blend_param: int, src_size, dst_size, stream=None,
                     check: bool = False) -> bool:
        """prepare(path, highQualityBlend, blendParam, srcSize, dstSize) with a PTGui .pts camera file."""
        self._size = tuple(dst_size)
        st = lib().ps_render_prepare_file(self._h, path.encode(), high_quality_blend, blend_param, src_size[0],
                                          src_size[1], dst_size[0], dst_size[1], _stream_handle(stream))
        return self._status(st, check)

    def set_frames_in_flight(self, n: int) -> None:
        """Sets of per-frame state the next prepare allocates (1..PS_MAX_IN_FLIGHT)."""
        check(lib().ps_render_set_frames_in_flight(self._h, n))

    @property
    def frames_in_flight(self) -> int:
        return lib().ps_render_get_frames_in_flight(self._h)

    def set_memory_budget(self, nbytes: int) -> None:
        """Device bytes the next prepare may take (0: the free memory only); fewer frames in flight fit."""
        check(lib().ps_render_set_memory_budget(self._h, int(nbytes)))

    def set_map_free(self, enable: bool) -> None:
        """Next multiband prepare keeps no maps: fp32 coordinates per pixel (level 0 within +-1)."""
        check(lib().ps_render_set_map_free(self._h, int(bool(enable))))

    @property
    def map_free(self) -> bool:
        return bool(lib().ps_render_is_map_free(self._h))

    def level0(self, cam: int) -> np.ndarray:
        """Level 0 of the last render for one camera (uint8 (H, W, 4)): the remap's output."""
        W, H = self._size
        return self.export(L.EXPORT_LEVEL0, cam, 0, (H, W, 4), np.uint8)

    @property
    def low_memory(self) -> bool:
        """The last prepare took fewer frames in flight than asked for (the reference's low-memory path)."""
        return bool(lib().ps_render_is_low_memory(self._h))

    @staticmethod
    def estimate_memory(params: Sequence[dict], blend_param: int, src_size, dst_size, frames_in_flight: int = 8):
        """Device bytes a render of this rig would hold (upper bound, no allocation)."""
        arr, n = _params(params), len(params)
        v = lib().ps_render_estimate_memory(arr, n, blend_param, src_size[0], src_size[1], dst_size[0], dst_size[1],
                                            frames_in_flight)
        if v < 0:
            raise PsError(L.PS_EINVAL, lib().ps_last_error().decode(errors="replace"))
        return v

    def get_unique_masks(self) -> list:
        """The seam masks (uint8 (H, W), 0 / 255), one per camera."""
        n = self.getNumImages()
        W, H = self._size
        out = [np.empty((H, W), np.uint8) for _ in range(n)]
        check(lib().ps_render_get_unique_masks(self._h, (C.c_void_p * n)(*[o.ctypes.data for o in out]), n))
        return out

    def set_seam_rule(self, rule: int) -> None:
        """PS_SEAMS_NEAREST_AXIS (default) or PS_SEAMS_DISTANCE (getNonIntersectingMasks); next prepare."""
        check(lib().ps_render_set_seam_rule(self._h, rule))

    def set_custom_masks(self, masks=None, stream=None, check: bool = False) -> bool:
        """Weight the following frames by one host uint8 (H, W) mask per camera, as
        CudaTilingMultibandBlendFast::blend(images, masks, blendImage) does; None returns to the unique
        masks."""
        keep, ptrs, n = _mask_ptrs(masks)
        return self._status(lib().ps_render_set_custom_masks(self._h, ptrs, n, _stream_handle(stream)), check)

    def render(self, src: Sequence, dst, luts=None, stream=None, check: bool = False) -> bool:
        """render(src, dst, luts): src frames -> dst canvas (both host or device)."""
        imgs = (Image * len(src))(*[as_image(s) for s in src])
        keep, nl, lp = _luts_arg(luts, len(src))
        d = as_image(dst)
        st = lib().ps_render_render(self._h, imgs, len(src), lp, nl, C.byref(d), _stream_handle(stream))
        del keep
        return self._status(st, check)

    def render_yuv(self, src: Sequence, planes: Sequence, luts=None, fmt: int = L.PS_FMT_YUV420P, stream=None,
                   check: bool = False) -> bool:
        """render + cvtBGR32ToYUV420P / cvtBGR32ToNV12 + download in one call: planes
        are (Y, U, V) or (Y, UV), host arrays or CUDA tensors."""
        imgs = (Image * len(src))(*[as_image(s) for s in src])
        keep, nl, lp = _luts_arg(luts, len(src))
        d = as_planar(planes, fmt)
        st = lib().ps_render_render_yuv(self._h, imgs, len(src), lp, nl, C.byref(d), _stream_handle(stream))
        del keep
        return self._status(st, check)

    def render_planar(self, src: Sequence, dst=None, luts=None, src_fmt: int = L.PS_FMT_NV12, ydst=None,
                      ydst_fmt: int = L.PS_FMT_NV12, stream=None, check: bool = False) -> bool:
        """render from decoder frames: src holds one (Y, U, V) or (Y, UV) plane list
        per camera (src_fmt, or a (planes, fmt) pair per camera), host arrays or
        CUDA tensors; out to the BGR canvas dst or to the planes ydst."""
        frames = []
        for s in src:
            if isinstance(s, tuple) and len(s) == 2 and isinstance(s[1], int):
                frames.append(as_planar(s[0], s[1]))
            else:
                frames.append(as_planar(s, src_fmt))
        arr = (PlanarImage * len(frames))(*frames)
        keep, nl, lp = _luts_arg(luts, len(src))
        d = C.byref(as_image(dst)) if dst is not None else None
        y = C.byref(as_planar(ydst, ydst_fmt)) if ydst is not None else None
        st = lib().ps_render_render_planar(self._h, arr, len(frames), lp, nl, d, y, _stream_handle(stream))
        del keep
        return self._status(st, check)

    def check_status(self, check: bool = True) -> bool:
        """Waits for the frames in flight and reports a bounded kernel wait that ran out since the last
        check (PS_ETIMEOUT: those frames may be wrong)."""
        return self._status(lib().ps_render_check(self._h), check)

    def set_wait_probe(self, polls: int) -> None:
        """Failure-path test hook: every blend launch makes one wait of `polls` polls that runs out."""
        check(lib().ps_render_set_wait_probe(self._h, int(polls)))

    def clear(self) -> None:
        lib().ps_render_clear(self._h)

    def getNumImages(self) -> int:
        return lib().ps_render_get_num_images(self._h)

    # -- extras ----------------------------------------------------------------
    @property
    def num_levels(self) -> int:
        return lib().ps_render_get_num_levels(self._h)

    @property
    def full_mask(self) -> bool:
        return bool(lib().ps_render_is_full_mask(self._h))

    @property
    def resident_bytes(self) -> int:
        return lib().ps_render_resident_bytes(self._h)

    def set_graph(self, enabled: bool) -> None:
        check(lib().ps_render_set_graph(self._h, int(bool(enabled))))

    def profile(self, enabled: bool) -> None:
        check(lib().ps_render_profile(self._h, int(bool(enabled))))

    KERNELS = {0: "k_remap", 1: "k_pyrdown", 2: "k_blend", 3: "k_tail", 4: "k_linear", 5: "k_yuv_to_bgr32",
               6: "k_blend_small", 7: "k_remap_fix"}

    def profile_read(self, kind: int, level: int = -1):
        """(launches, total_ms, algorithmic_bytes) of finished profiled launches."""
        n, ms, b = C.c_longlong(), C.c_double(), C.c_double()
        check(lib().ps_render_profile_read(self._h, kind, level, C.byref(n), C.byref(ms), C.byref(b)))
        return n.value, ms.value, b.value

    @property
    def launches_per_frame(self) -> int:
        return lib().ps_render_launches_per_frame(self._h)

    def algorithmic_bytes(self, bytes_in_per_px: int = 4, bytes_out_per_px: int = 4) -> float:
        return lib().ps_render_algorithmic_bytes(self._h, bytes_in_per_px, bytes_out_per_px)

    SHAPE_DEFAULT = {"tail_max_items": 16, "tail_cluster": 0, "tail_half_tiles": 1, "ctas_per_sm": (0, 0, 0),
                     "small_blend_max_items": 0, "remap_defer_ties": 1}

    @staticmethod
    def _shape_dict(s: "L.LaunchShape") -> dict:
        return {"tail_max_items": s.tail_max_items, "tail_cluster": s.tail_cluster,
                "tail_half_tiles": s.tail_half_tiles, "ctas_per_sm": tuple(s.ctas_per_sm),
                "small_blend_max_items": s.small_blend_max_items, "remap_defer_ties": s.remap_defer_ties}

    def launch_shape(self) -> dict:
        """The render's launch shape (ps_launch_shape fields)."""
        s = L.LaunchShape()
        check(lib().ps_render_get_launch_shape(self._h, C.byref(s)))
        return self._shape_dict(s)

    def set_launch_shape(self, **fields) -> None:
        """Change some fields of the launch shape (the others keep their value)."""
        cur = self.launch_shape()
        unknown = set(fields) - set(cur)
        if unknown:
            raise ValueError(f"unknown launch-shape fields {sorted(unknown)}")
        cur.update(fields)
        s = L.LaunchShape(cur["tail_max_items"], cur["tail_cluster"], cur["tail_half_tiles"],
                          (C.c_int * 3)(*cur["ctas_per_sm"]), cur["small_blend_max_items"], cur["remap_defer_ties"])
        check(lib().ps_render_set_launch_shape(self._h, C.byref(s)))

    def autotune(self, frames_per_trial: int = 0, in_flight: int = 0, force: bool = False) -> dict:
        """Time launch shapes on this rig and keep the fastest (ps_render_autotune)."""
        s, rep = L.LaunchShape(), L.TuneReport()
        check(lib().ps_render_autotune(self._h, frames_per_trial, in_flight, int(bool(force)), C.byref(s),
                                       C.byref(rep)))
        return {"shape": self._shape_dict(s), "ms_per_frame_default": rep.ms_per_frame_default,
                "ms_per_frame_chosen": rep.ms_per_frame_chosen, "trials": rep.trials, "cached": bool(rep.cached)}

    def input_buffer(self, cam: int):
        p, pitch = C.c_void_p(), C.c_longlong()
        check(lib().ps_render_get_input_buffer(self._h, cam, C.byref(p), C.byref(pitch)))
        return p.value, pitch.value

    def export(self, what: int, cam: int, level: int, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype)
        check(lib().ps_render_export(self._h, what, cam, level, out.ctypes.data, out.nbytes))
        return out

    def maps(self, cam: int, dst_size):
        W, H = dst_size
        return (self.export(L.EXPORT_XMAP, cam, 0, (H, W), np.float32),
                self.export(L.EXPORT_YMAP, cam, 0, (H, W), np.float32))

    def coverage(self, cam: int, dst_size) -> np.ndarray:
        return self.export(L.EXPORT_COVERAGE, cam, 0, (dst_size[1], dst_size[0]), np.uint8)

    def linear_weight(self, cam: int, dst_size) -> np.ndarray:
        """Linear-blend mode: the camera's float weight per canvas pixel."""
        return self.export(L.EXPORT_LINEAR_WEIGHT, cam, 0, (dst_size[1], dst_size[0]), np.float32)

    def seam(self, cam: int, dst_size) -> np.ndarray:
        return self.export(L.EXPORT_SEAM, cam, 0, (dst_size[1], dst_size[0]), np.uint8)

    def collapsed(self, level: int, size) -> np.ndarray:
        w, h = size
        out = np.empty((h, w, 4), np.int16)
        check(lib().ps_render_export_collapsed(self._h, level, out.ctypes.data, out.nbytes, None))
        return out


class CudaRicohPanoramaRender:
    """CudaRicohPanoramaRender (source/Task/RicohUtil.cpp:1363-1406): a dual
    fisheye camera delivering both lenses in one frame.  The rig has two
    cameras whose crops select the halves of the frame; render takes the one
    frame and stitches it as both cameras' source."""

    def __init__(self):
        self._r = CudaPanoramaRender2()
        self.last_error = ""

    def _fail(self, code: int, msg: str, check_: bool) -> bool:
        self.last_error = msg
        if check_:
            raise PsError(code, msg)
        return False

    def _checked(self, ok: bool, check_: bool) -> bool:
        if not ok:
            return self._fail(L.PS_EINVAL, self._r.last_error, check_)
        n = self._r.getNumImages()
        if n != 2:  # RicohUtil.cpp:1368-1373
            self._r.clear()
            return self._fail(L.PS_EINVAL, f"num images = {n}, requires 2", check_)
        return True

    def prepare(self, params: Sequence[dict], high_quality_blend: int, blend_param: int, src_size, dst_size,
                stream=None, check: bool = False) -> bool:
        return self._checked(self._r.prepare(params, high_quality_blend, blend_param, src_size, dst_size,
                                             stream=stream), check)

    def prepare_file(self, path: str, high_quality_blend: int, blend_param: int, src_size, dst_size, stream=None,
                     check: bool = False) -> bool:
        return self._checked(self._r.prepare_file(path, high_quality_blend, blend_param, src_size, dst_size,
                                                  stream=stream), check)

    def render(self, src: Sequence, dst, luts=None, stream=None, check: bool = False) -> bool:
        """render(src, dst, luts) with src the one dual-fisheye frame."""
        if self._r.getNumImages() != 2:
            return self._fail(L.PS_ESTATE, "have not prepared or prepare failed before", check)
        if len(src) != 1:
            return self._fail(L.PS_EINVAL, f"src size = {len(src)}, requires 1", check)
        ok = self._r.render([src[0], src[0]], dst, luts, stream=stream)
        if not ok:
            return self._fail(L.PS_EINVAL, self._r.last_error, check)
        return True

    def clear(self) -> None:
        self._r.clear()

    def getNumImages(self) -> int:
        return 1 if self._r.getNumImages() == 2 else 0

    @property
    def render2(self) -> CudaPanoramaRender2:
        """The two-camera render underneath (for exports and measurement hooks)."""
        return self._r


def render_batch(renders: Sequence[CudaPanoramaRender2], srcs: Sequence[Sequence], dsts: Sequence,
                 luts: Sequence | None = None, stream=None) -> None:
    """One launch sequence for several rigs (one frame each)."""
    k = len(renders)
    hs = (C.c_void_p * k)(*[r._h.value for r in renders])
    arrays = [(Image * len(s))(*[as_image(x) for x in s]) for s in srcs]
    sp = (C.POINTER(Image) * k)(*[C.cast(a, C.POINTER(Image)) for a in arrays])
    keep = []
    lp = None
    if luts is not None:
        ptrs = []
        for lt in luts:
            if lt is None:
                ptrs.append(None)
            else:
                a = np.ascontiguousarray(lt, np.uint8)
                keep.append(a)
                ptrs.append(a.ctypes.data)
        lp = (C.c_void_p * k)(*ptrs)
    ds = (Image * k)(*[as_image(d) for d in dsts])
    check(lib().ps_render_batch(hs, k, sp, lp, ds, _stream_handle(stream)))


class CudaTilingMultibandBlendFast:
    """CudaTilingMultibandBlendFast (source/CudaAccel/CudaInterface.h:45-82)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().ps_blender_create(C.byref(h)))
        self._h = h
        self.last_error = ""

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().ps_blender_destroy(h)
            except Exception:
                pass
            self._h = None

    def prepare(self, masks, seams=None, max_levels: int = 16, min_length: int = 2, stream=None) -> bool:
        """prepare(masks, maxLevels, minLength); seams None derives them as the reference does."""
        ms = [np.ascontiguousarray(m, np.uint8) for m in masks]
        ss = None if seams is None else [np.ascontiguousarray(s, np.uint8) for s in seams]
        H, W = ms[0].shape
        mp = (C.c_void_p * len(ms))(*[m.ctypes.data for m in ms])
        sp = None if ss is None else (C.c_void_p * len(ss))(*[s.ctypes.data for s in ss])
        st = lib().ps_blender_prepare(self._h, mp, sp, len(ms), W, H, max_levels, min_length,
                                      _stream_handle(stream))
        self._n = len(ms)
        if st != L.PS_OK:
            self.last_error = lib().ps_last_error().decode(errors="replace")
            return False
        return True

    def blend(self, images, dst, stream=None, check_: bool = True) -> bool:
        """images: CUDA int16 (H, W, 4) or uint8 (H, W, 4) tensors."""
        fmt = 16 if images[0].element_size() == 2 else 8
        ptrs = (C.c_void_p * len(images))(*[t.data_ptr() for t in images])
        pitches = (C.c_longlong * len(images))(*[t.stride(0) * t.element_size() for t in images])
        d = as_image(dst)
        st = lib().ps_blender_blend(self._h, ptrs, pitches, fmt, C.byref(d), _stream_handle(stream))
        if st != L.PS_OK:
            self.last_error = lib().ps_last_error().decode(errors="replace")
            if check_:
                raise PsError(st, self.last_error)
            return False
        return True

    def set_custom_masks(self, masks=None, stream=None) -> bool:
        """blend(images, masks, blendImage): later blends weight the cameras by these host uint8 (H, W)
        masks; None returns to the unique masks."""
        keep, ptrs, n = _mask_ptrs(masks)
        st = lib().ps_blender_set_custom_masks(self._h, ptrs, n, _stream_handle(stream))
        if st != L.PS_OK:
            self.last_error = lib().ps_last_error().decode(errors="replace")
            return False
        return True

    @property
    def num_levels(self) -> int:
        return lib().ps_blender_get_num_levels(self._h)

    def begin(self, stream=None) -> None:
        """begin(): a blend fed one camera at a time."""
        check(lib().ps_blender_begin(self._h, _stream_handle(stream)))

    def tile(self, image, index: int, stream=None) -> None:
        """tile(image, index): camera `index`'s CUDA int16 (H, W, 4) or uint8 (H, W, 4) level-0 image."""
        fmt = 16 if image.element_size() == 2 else 8
        check(lib().ps_blender_tile(self._h, image.data_ptr(), image.stride(0) * image.element_size(), fmt, index,
                                    _stream_handle(stream)))

    def end(self, dst, stream=None) -> None:
        """end(blendImage): blends the tiled cameras into dst."""
        d = as_image(dst)
        check(lib().ps_blender_end(self._h, C.byref(d), _stream_handle(stream)))

    def get_unique_masks(self, size) -> list:
        """getUniqueMasks: the seam masks (uint8 (H, W), 0 / 255); size = (W, H)."""
        W, H = size
        n = self._n
        out = [np.empty((H, W), np.uint8) for _ in range(n)]
        check(lib().ps_blender_get_unique_masks(self._h, (C.c_void_p * n)(*[o.ctypes.data for o in out]), n))
        return out

    def calc_used_memory_size(self) -> int:
        """calcUsedMemorySize: device bytes the blender holds."""
        return lib().ps_blender_used_memory(self._h)

    @staticmethod
    def estimate_memory_size(width: int, height: int, num_images: int, max_levels: int = 16) -> int:
        """estimateMemorySize: device bytes a blender of this size would hold at most."""
        return lib().ps_blender_estimate_memory(width, height, num_images, max_levels)

    def check_status(self) -> int:
        """PS_OK, or PS_ETIMEOUT when a bounded kernel wait ran out since the last check."""
        st = lib().ps_blender_check(self._h)
        if st != L.PS_OK:
            self.last_error = lib().ps_last_error().decode(errors="replace")
        return st

    def set_wait_probe(self, polls: int) -> None:
        """Failure-path test hook: every blend launch makes one wait of `polls` polls that runs out."""
        check(lib().ps_blender_set_wait_probe(self._h, int(polls)))


def generate_reproject_map_and_mask(param: dict, src_size, dst_size, xmap, ymap, mask, stream=None) -> None:
    """cudaGenerateReprojectMapAndMask into CUDA tensors (float32, float32, uint8; (H, W))."""
    p = PhotoParam.from_dict(param)
    check(lib().ps_generate_reproject_map_and_mask(C.byref(p), src_size[0], src_size[1], dst_size[0],
                                                   dst_size[1], xmap.data_ptr(), ymap.data_ptr(),
                                                   mask.data_ptr(), _stream_handle(stream)))


def reproject_to_16s(src, xmap, ymap, dst, lut=None, stream=None) -> None:
    """cudaTransform + cudaReprojectTo16S: CUDA tensors in, int16 (H, W, 4) out."""
    s = as_image(src)
    H, W = xmap.shape
    check(lib().ps_reproject_to_16s(C.byref(s), xmap.data_ptr(), ymap.data_ptr(), xmap.stride(0) * 4, W, H,
                                    None if lut is None else lut.data_ptr(), dst.data_ptr(),
                                    dst.stride(0) * dst.element_size(), _stream_handle(stream)))


def non_intersecting_masks(masks, out, stream=None) -> None:
    """getNonIntersectingMasks: (n, H, W) uint8 CUDA tensor -> (n, H, W) 0/255 CUDA tensor."""
    n, H, W = masks.shape
    _require(masks.is_contiguous() and out.is_contiguous() and tuple(out.shape) == (n, H, W),
             "masks and out are contiguous (n, H, W) tensors")
    check(lib().ps_non_intersecting_masks(masks.data_ptr(), n, W, H, out.data_ptr(), _stream_handle(stream)))


def distance_transform_l1(mask, dist, stream=None) -> None:
    """cv::distanceTransform(mask, dist, CV_DIST_L1, 3): uint8 (H, W) -> int32 (H, W) CUDA tensors."""
    H, W = mask.shape
    _require(mask.is_contiguous() and dist.is_contiguous() and tuple(dist.shape) == (H, W),
             "mask and dist are contiguous (H, W) tensors")
    check(lib().ps_distance_transform_l1(mask.data_ptr(), W, H, dist.data_ptr(), _stream_handle(stream)))


def cvt_bgr32_to_yuv(src, planes: Sequence, fmt: int = L.PS_FMT_YUV420P, stream=None) -> None:
    """cvtBGR32ToYUV420P / cvtBGR32ToNV12 (ImageProc.cu:120-160): a BGR32 CUDA tensor
    to (Y, U, V) or (Y, UV) CUDA tensor planes."""
    s = as_image(src)
    d = as_planar(planes, fmt)
    check(lib().ps_cvt_bgr32_to_yuv(C.byref(s), C.byref(d), _stream_handle(stream)))


def cvt_yuv_to_bgr32(planes: Sequence, dst, fmt: int = L.PS_FMT_YUV420P, stream=None) -> None:
    """cvtYUV420PToBGR32 / cvtNV12ToBGR32 (ImageProc.cu:165-259): (Y, U, V) or (Y, UV)
    CUDA tensor planes to a BGR32 CUDA tensor (fourth byte 0)."""
    s = as_planar(planes, fmt)
    d = as_image(dst)
    check(lib().ps_cvt_yuv_to_bgr32(C.byref(s), C.byref(d), _stream_handle(stream)))


def load_photo_params(path: str) -> list:
    """loadPhotoParams for a PTGui .pts file: a list of parameter dicts."""
    n = C.c_int(0)
    check(lib().ps_load_photo_params(path.encode(), None, 0, C.byref(n)))
    arr = (PhotoParam * max(1, n.value))()
    check(lib().ps_load_photo_params(path.encode(), arr, n.value, C.byref(n)))
    return [{k: getattr(arr[i], k) for k, _ in PhotoParam._fields_} for i in range(n.value)]


def get_lut(k: float) -> np.ndarray:
    """getLUT (source/Blend/ExposureColorOptimize.cpp:1217-1223)."""
    out = np.empty(256, np.uint8)
    check(lib().ps_get_lut(float(k), out.ctypes.data))
    return out
