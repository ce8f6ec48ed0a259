"""Camera parameter files: the PTGui .pts reader of loadPhotoParams
(source/Warp/PhotoParam.cpp:681-771), and prepare(path, ...)."""
import os

import numpy as np
import pytest

import panostitcher_gb300 as P

PTS = """# ptGui project file
#-imgfile 1920 1080 "cam0.jpg"
o f0 y0 r0 p0 v100 a0.01 b-0.02 c0.03 d1.5 e-2.5 g0 t0
#-imgfile 1920 1080 "cam0.jpg"
o f0 y10.5 r1 p-2 v100 a0 b0 c0 d0 e0 g0 t0 C10,1910,20,1060
#-imgfile 1280 960 "cam1.jpg"
o f3 y180 r0 p5 v100 a0 b0 c0 d0 e0 g0 t0
o f2 y90 r0 p0 C0,100,0,100,5
"""


def _write(tmp_path, text, name="rig.pts"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_pts_global_and_cameras(built_lib, tmp_path):
    params = P.load_photo_params(_write(tmp_path, PTS))
    # the first complete "o" line is the global one; the crop with five values is rejected
    assert len(params) == 2
    a, b = params
    assert a["image_type"] == 0 and (a["yaw"], a["pitch"], a["roll"]) == (10.5, -2.0, 1.0)
    assert (a["crop_x"], a["crop_y"], a["crop_width"], a["crop_height"]) == (10, 20, 1900, 1040)
    assert b["image_type"] == 1 and b["yaw"] == 180 and b["pitch"] == 5  # PanoTools 3 = full-frame fisheye
    for p in params:  # global values copied to every camera
        assert (p["hfov"], p["alpha"], p["beta"], p["gamma"]) == (100, 0.01, -0.02, 0.03)
        assert (p["shift_x"], p["shift_y"], p["shear_x"], p["shear_y"]) == (1.5, -2.5, 0, 0)


def test_pts_without_header_or_global_has_no_cameras(built_lib, tmp_path):
    assert P.load_photo_params(_write(tmp_path, PTS.replace("ptGui project file", "something else"))) == []
    no_global = "# ptGui project file\no f0 y0 r0 p0\n"
    assert P.load_photo_params(_write(tmp_path, no_global, "b.pts")) == []


def test_other_files_are_rejected(built_lib, tmp_path):
    with pytest.raises(P.PsError) as e:
        P.load_photo_params(_write(tmp_path, "<Root/>", "rig.xml"))
    assert "ticpp" in str(e.value)
    with pytest.raises(P.PsError):
        P.load_photo_params(_write(tmp_path, PTS, "noextension"))
    with pytest.raises(P.PsError):
        P.load_photo_params(str(tmp_path / "missing.pts"))
    r = P.CudaPanoramaRender2()
    assert not r.prepare_file(_write(tmp_path, PTS.replace("ptGui", "x"), "c.pts"), 1, 8, (1920, 1080), (2048, 1024))
    assert "load photo params failed" in r.last_error


@pytest.mark.gpu
def test_prepare_file_equals_prepare(cuda, tmp_path):
    path = _write(tmp_path, PTS)
    params = P.load_photo_params(path)
    a, b = P.CudaPanoramaRender2(), P.CudaPanoramaRender2()
    assert a.prepare_file(path, 1, 6, (1920, 1080), (512, 256), check=True)
    assert b.prepare(params, 1, 6, (1920, 1080), (512, 256), check=True)
    for i in range(len(params)):
        for what in (0, 1, 3):
            ea = a.export(what, i, 0, (256, 512), np.float32 if what < 2 else np.uint8)
            eb = b.export(what, i, 0, (256, 512), np.float32 if what < 2 else np.uint8)
            assert np.array_equal(ea, eb)
