"""The C ABI library: builds, loads, exports every declared entry point, and
rejects bad arguments before touching the GPU (CPU only)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(ps_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(built_lib):
    decl = declared_functions()
    assert len(decl) >= 25
    missing = [n for n in sorted(decl) if not hasattr(built_lib, n)]
    assert not missing, missing
    # the Python bindings cover the whole ABI
    assert decl <= set(L.exported_symbols())


def test_checked_build_exports_the_same_abi(built_lib):
    path = os.path.join(ROOT, "panostitcher_gb300", "libpanostitch_checked.so")
    checked = C.CDLL(path)
    missing = [n for n in sorted(declared_functions()) if not hasattr(checked, n)]
    assert not missing, missing
    built_lib.ps_debug_bounds_violations.restype = C.c_longlong
    assert built_lib.ps_debug_bounds_violations(0) == -1  # the normal build checks nothing


def test_version_and_empty_error(built_lib):
    assert b"sm_103a" in built_lib.ps_version()


def test_get_lut_host_path(built_lib):
    assert np.array_equal(P.get_lut(1.0), np.arange(256))
    assert np.array_equal(P.get_lut(1.17), S.lut_from_gain(1.17))
    with pytest.raises(P.PsError) as e:
        P.get_lut(0.0)
    assert e.value.code == L.PS_EINVAL


def _prepare_err(**kw):
    r = P.CudaPanoramaRender2()
    cfg = S.rig("c1")
    args = dict(params=cfg.cams, high_quality_blend=1, blend_param=5, src_size=cfg.src_size,
                dst_size=cfg.dst_size)
    args.update(kw)
    ok = r.prepare(args["params"], args["high_quality_blend"], args["blend_param"], args["src_size"],
                   args["dst_size"])
    assert not ok
    assert r.getNumImages() == 0
    return r.last_error


def test_prepare_preconditions_like_reference(built_lib):
    # dstSize must be even with width == 2 * height (source/Task/RicohUtil.cpp:1098-1103)
    assert "not qualified" in _prepare_err(dst_size=(2048, 1000))
    assert "not qualified" in _prepare_err(dst_size=(2047, 1024 - 0))
    # blendParam > 0 (:1105-1109)
    assert "positive" in _prepare_err(blend_param=0)
    assert "camera" in _prepare_err(params=[])
    assert "image_type" in _prepare_err(params=[S.photo_param(7, 90.0)])
    # linear-blend mode: the Gaussian radius is bounded
    assert "radius" in _prepare_err(high_quality_blend=0, blend_param=5000)
    assert "srcSize" in _prepare_err(src_size=(0, 10))


def test_render_before_prepare_fails(built_lib):
    r = P.CudaPanoramaRender2()
    dst = np.zeros((8, 16, 4), np.uint8)
    assert not r.render([np.zeros((4, 4, 4), np.uint8)], dst)
    assert "prepare" in r.last_error
    with pytest.raises(P.PsError) as e:
        r.render([np.zeros((4, 4, 4), np.uint8)], dst, check=True)
    assert e.value.code == L.PS_ESTATE


def test_blender_prepare_validation(built_lib):
    b = P.CudaTilingMultibandBlendFast()
    h = C.c_void_p()
    assert built_lib.ps_blender_prepare(b._h, None, None, 0, 8, 8, 3, 2, None) == L.PS_EINVAL
    assert built_lib.ps_blender_blend(b._h, None, None, 16, None, None) == L.PS_ESTATE
    assert b.num_levels == 0


def test_null_handles_are_rejected(built_lib):
    assert built_lib.ps_render_create(None) == L.PS_EINVAL
    assert built_lib.ps_render_get_num_images(None) == 0
    built_lib.ps_render_destroy(None)
    built_lib.ps_blender_destroy(None)
    assert built_lib.ps_render_batch(None, 0, None, None, None, None) == L.PS_EINVAL


def test_yuv_entry_points_validate_before_the_gpu(built_lib):
    r = P.CudaPanoramaRender2()
    y = np.zeros((64, 128), np.uint8)
    u = np.zeros((32, 64), np.uint8)
    v = np.zeros((32, 64), np.uint8)
    frames = [np.zeros((8, 8, 4), np.uint8)]
    assert not r.render_yuv(frames, [y, u, v])
    assert "prepare" in r.last_error
    im = P.as_image(np.zeros((4, 6, 4), np.uint8))
    pl = P.as_planar([np.zeros((4, 6), np.uint8), np.zeros((2, 6), np.uint8)], P.PS_FMT_NV12)
    assert built_lib.ps_cvt_bgr32_to_yuv(C.byref(im), C.byref(pl), None) == L.PS_EINVAL  # host source
    pl.format = 77
    im.location = L.PS_MEM_DEVICE
    assert built_lib.ps_cvt_bgr32_to_yuv(C.byref(im), C.byref(pl), None) == L.PS_EINVAL  # unknown format
    assert "format" in built_lib.ps_last_error().decode()
    pl.format = P.PS_FMT_NV12
    pl.height = 5
    assert built_lib.ps_cvt_bgr32_to_yuv(C.byref(im), C.byref(pl), None) == L.PS_EINVAL  # size mismatch


def test_launch_shape_validation_before_the_gpu(built_lib):
    r = P.CudaPanoramaRender2()
    assert r.launch_shape() == P.CudaPanoramaRender2.SHAPE_DEFAULT
    for bad in ({"tail_cluster": 5}, {"tail_half_tiles": 2}, {"tail_max_items": -1}, {"ctas_per_sm": (0, -1, 0)},
                {"ctas_per_sm": (0, 0, 65)}, {"small_blend_max_items": -3}, {"remap_defer_ties": 2}):
        with pytest.raises(P.PsError) as e:
            r.set_launch_shape(**bad)
        assert e.value.code == L.PS_EINVAL
    assert r.launch_shape() == P.CudaPanoramaRender2.SHAPE_DEFAULT  # rejected shapes leave it unchanged
    # before prepare the shape is only stored (it applies at prepare)
    r.set_launch_shape(tail_max_items=0, tail_cluster=8, tail_half_tiles=0, ctas_per_sm=(1, 2, 3),
                       small_blend_max_items=256, remap_defer_ties=0)
    assert r.launch_shape() == {"tail_max_items": 0, "tail_cluster": 8, "tail_half_tiles": 0,
                                "ctas_per_sm": (1, 2, 3), "small_blend_max_items": 256, "remap_defer_ties": 0}
    with pytest.raises(ValueError):
        r.set_launch_shape(tile=64)
    with pytest.raises(P.PsError) as e:
        r.autotune()
    assert e.value.code == L.PS_ESTATE
    assert built_lib.ps_render_set_launch_shape(None, None) == L.PS_EINVAL
    assert built_lib.ps_render_autotune(None, 0, 0, 0, None, None) == L.PS_EINVAL


def test_frames_in_flight_validation_before_the_gpu(built_lib):
    r = P.CudaPanoramaRender2()
    assert r.frames_in_flight == 0  # not prepared
    for bad in (0, -1, L.PS_MAX_IN_FLIGHT + 1):
        with pytest.raises(P.PsError) as e:
            r.set_frames_in_flight(bad)
        assert e.value.code == L.PS_EINVAL
    r.set_frames_in_flight(1)
    r.set_frames_in_flight(L.PS_MAX_IN_FLIGHT)
    assert built_lib.ps_render_set_frames_in_flight(None, 2) == L.PS_EINVAL
    assert built_lib.ps_render_get_frames_in_flight(None) == 0


def test_intersecting_seams_rejected_before_the_gpu(built_lib):
    """Explicit seams must not intersect (as getNonIntersectingMasks' never do); both prepares check it on
    the host before any device work and name the first shared pixel."""
    cfg = S.rig("c1")
    W, H = cfg.dst_size
    seams = np.zeros((cfg.num_cams, H, W), np.uint8)
    seams[0][:, : W // 2] = 255
    seams[1][:, W // 2 - 1:] = 255  # column W/2 - 1 is both cameras'
    r = P.CudaPanoramaRender2()
    assert not r.prepare(cfg.cams, 1, 5, cfg.src_size, cfg.dst_size, seams=list(seams))
    assert f"seam masks 0 and 1 intersect at ({W // 2 - 1}, 0)" in r.last_error and r.getNumImages() == 0
    b = P.CudaTilingMultibandBlendFast()
    cov = np.full((2, 16, 32), 255, np.uint8)
    small = np.zeros_like(cov)
    small[0][:, :20] = 255
    small[1][:, 19:] = 255
    assert not b.prepare(list(cov), list(small), 3)
    assert "intersect at (19, 0)" in b.last_error and b.num_levels == 0
    # disjoint seams pass the check (on a host without a GPU the prepare then fails further on)
    small[1][:, 19] = 0
    ok = b.prepare(list(cov), list(small), 3)
    assert ok or "intersect" not in b.last_error


def test_custom_masks_need_a_prepared_multiband_rig(built_lib):
    assert built_lib.ps_render_set_custom_masks(None, None, 0, None) == L.PS_EINVAL
    assert built_lib.ps_blender_set_custom_masks(None, None, 0, None) == L.PS_EINVAL
    r = P.CudaPanoramaRender2()
    m = np.zeros((8, 16), np.uint8)
    assert not r.set_custom_masks([m, m])
    assert "prepare" in r.last_error
    b = P.CudaTilingMultibandBlendFast()
    assert not b.set_custom_masks(None)
    assert "prepare" in b.last_error
