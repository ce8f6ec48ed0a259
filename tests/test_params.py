"""Camera parameter files: the PTGui .pts and XML readers of loadPhotoParams
(source/Warp/PhotoParam.cpp:17-506, 681-771), and prepare(path, ...)."""
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


# The per-camera layout (loadPhotoParamFromXML2): every field on each camera element.
XML_PER_CAMERA = """<?xml version="1.0" encoding="utf-8"?>
<!-- two cameras -->
<Root>
  <POSITION>
    <IMAGETYPE>0</IMAGETYPE><CROPMODE>0</CROPMODE><HFOV>100</HFOV><VFOV>0</VFOV>
    <Alpha>0.01</Alpha><Beta>-0.02</Beta><Gamma>0.03</Gamma><ShiftX>1.5</ShiftX><ShiftY>-2.5</ShiftY>
    <ShearX>0</ShearX><ShearY>0</ShearY>
    <CROPLEFT>10</CROPLEFT><CROPRIGHT>1910</CROPRIGHT><CROPTOP>20</CROPTOP><CROPBOTTOM>1060</CROPBOTTOM>
    <CircleX>0</CircleX><CircleY>0</CircleY><CircleR>0</CircleR>
    <YAW>10.5</YAW><PITCH>-2</PITCH><ROLL>1</ROLL>
  </POSITION>
  <POSITION note="attributes are ignored">
    <IMAGETYPE>1</IMAGETYPE><CROPMODE>0</CROPMODE><HFOV>100</HFOV><VFOV>0</VFOV>
    <Alpha>0.01</Alpha><Beta>-0.02</Beta><Gamma>0.03</Gamma><ShiftX>1.5</ShiftX><ShiftY>-2.5</ShiftY>
    <ShearX>0</ShearX><ShearY>0</ShearY>
    <CROPLEFT>0</CROPLEFT><CROPRIGHT>0</CROPRIGHT><CROPTOP>0</CROPTOP><CROPBOTTOM>0</CROPBOTTOM>
    <CircleX>640</CircleX><CircleY>480</CircleY><CircleR>470</CircleR>
    <YAW>180</YAW><PITCH>5</PITCH><ROLL>0</ROLL>
  </POSITION>
</Root>
"""

# The GlobalInfo layout (loadPhotoParamFromXML1): lens and crop once, the pose per camera element.
XML_GLOBAL = """<Root>
  <GlobalInfo>
    <IMAGETYPE>0</IMAGETYPE><CROPMODE>0</CROPMODE><HFOV>100</HFOV><VFOV>0</VFOV>
    <CROPLEFT>10</CROPLEFT><CROPRIGHT>1910</CROPRIGHT><CROPTOP>20</CROPTOP><CROPBOTTOM>1060</CROPBOTTOM>
    <Alpha>0.01</Alpha><Beta>-0.02</Beta><Gamma>0.03</Gamma><ShiftX>1.5</ShiftX><ShiftY>-2.5</ShiftY>
    <ShearX>0</ShearX><ShearY>0</ShearY>
  </GlobalInfo>
  <VIDEO><YAW>10.5</YAW><PITCH>-2</PITCH><ROLL>1</ROLL></VIDEO>
  <VIDEO><YAW> 190 </YAW><PITCH>0</PITCH><ROLL>0</ROLL></VIDEO>
</Root>
"""


def test_xml_per_camera_layout_equals_pts(built_lib, tmp_path):
    xml = P.load_photo_params(_write(tmp_path, XML_PER_CAMERA, "rig.xml"))
    pts = P.load_photo_params(_write(tmp_path, PTS))
    assert len(xml) == 2
    # the first camera is the .pts file's first camera, field for field
    assert xml[0] == pts[0]
    b = xml[1]
    assert b["image_type"] == 1 and (b["yaw"], b["pitch"]) == (180, 5)
    assert (b["circle_x"], b["circle_y"], b["circle_r"]) == (640, 480, 470)


def test_xml_global_info_layout(built_lib, tmp_path):
    cams = P.load_photo_params(_write(tmp_path, XML_GLOBAL, "rig.cfg"))  # any extension but .pts is XML
    assert len(cams) == 2
    pts = P.load_photo_params(_write(tmp_path, PTS))
    assert cams[0] == pts[0]
    assert cams[1]["yaw"] == 190 and cams[1]["crop_width"] == 1900
    for c in cams:
        assert (c["hfov"], c["shift_x"], c["alpha"]) == (100, 1.5, 0.01)


def test_xml_layouts_fall_back_and_fail(built_lib, tmp_path):
    # a camera element without IMAGETYPE: not the per-camera layout, and no GlobalInfo either
    broken = XML_PER_CAMERA.replace("<IMAGETYPE>1</IMAGETYPE>", "")
    assert P.load_photo_params(_write(tmp_path, broken, "a.xml")) == []
    # not a number, unclosed elements, no Root: no cameras
    assert P.load_photo_params(_write(tmp_path, XML_GLOBAL.replace(">100<", ">x<"), "b.xml")) == []
    assert P.load_photo_params(_write(tmp_path, "<Root><POSITION>", "c.xml")) == []
    assert P.load_photo_params(_write(tmp_path, "<Other/>", "d.xml")) == []
    r = P.CudaPanoramaRender2()
    assert not r.prepare_file(_write(tmp_path, "<Root/>", "e.xml"), 1, 8, (1920, 1080), (2048, 1024))
    assert "load photo params failed" in r.last_error


def test_other_files_are_rejected(built_lib, tmp_path):
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


@pytest.mark.gpu
def test_prepare_xml_file_equals_prepare(cuda, tmp_path):
    path = _write(tmp_path, XML_PER_CAMERA, "rig.xml")
    params = P.load_photo_params(path)
    a, b = P.CudaPanoramaRender2(), P.CudaPanoramaRender2()
    assert a.prepare_file(path, 1, 6, (1920, 1080), (512, 256), check=True)
    assert b.prepare(params, 1, 6, (1920, 1080), (512, 256), check=True)
    for i in range(len(params)):
        for what in (0, 1, 3):
            ea = a.export(what, i, 0, (256, 512), np.float32 if what < 2 else np.uint8)
            eb = b.export(what, i, 0, (256, 512), np.float32 if what < 2 else np.uint8)
            assert np.array_equal(ea, eb)
