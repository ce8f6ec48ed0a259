"""The dual-fisheye render (GPU): CudaRicohPanoramaRender
(source/Task/RicohUtil.cpp:1363-1406) stitches one frame holding two circular
fisheyes, each camera's crop one half.  Checks the circular-fisheye crop
geometry against the oracle, the render against the oracle's render of the
same frame given to both cameras (a full-coverage rig, so the full-mask
normalisation), the one-upload path for a host frame given twice, and the
reference's argument checks."""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[4, 2], ids=lambda f: f"ricoh/{f}")
def rig(request, cuda, oracle_lib):
    cfg = S.scaled_rig(S.rig("ricoh"), request.param)
    p = Prepared(cfg)
    return cfg, p


def test_circular_fisheye_crops_match_oracle(rig):
    cfg, p = rig
    assert p.r.full_mask  # the two halves cover the whole canvas
    npx = cfg.canvas_pixels
    for i, cam in enumerate(cfg.cams):
        xm, ym, mk = O.reproject_map(cam, cfg.src_size, cfg.dst_size)
        assert int(np.count_nonzero((mk > 0) != (p.cov[i] > 0))) <= max(4, npx // 100000)
        both = (mk > 0) & (p.cov[i] > 0)
        assert np.abs(p.maps[i][0][both] - xm[both]).max() <= 1e-3
        assert np.abs(p.maps[i][1][both] - ym[both]).max() <= 1e-3
        half = cfg.src_size[0] // 2  # camera i samples only its half of the frame
        assert (xm[both] >= i * half).all() and (xm[both] < (i + 1) * half).all()


def test_ricoh_render_equals_oracle(rig):
    import torch
    cfg, p = rig
    W, H = cfg.dst_size
    r = P.CudaRicohPanoramaRender()
    assert r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    assert r.getNumImages() == 1
    for k in (0, 1):
        frame = p.frames.frame(k)[0]  # one dual-fisheye frame
        ref = p.oracle_render([frame, frame], p.luts)[..., :3]
        out = np.zeros((H, W, 4), np.uint8)
        assert r.render([frame], out, p.luts, check=True)
        dev = torch.from_numpy(frame).cuda()
        dout = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
        assert r.render([dev], dout, p.luts, check=True)
        torch.cuda.synchronize()
        assert np.array_equal(out[..., :3], ref), diff_histogram(out[..., :3], ref)
        assert np.array_equal(dout.cpu().numpy()[..., :3], ref)


def test_host_frame_given_twice_goes_up_once(rig):
    import torch
    cfg, p = rig
    W, H = cfg.dst_size
    frame = p.frames.frame(2)[0]
    ref = p.oracle_render([frame, frame], p.luts)[..., :3]
    outs = [np.zeros((H, W, 4), np.uint8) for _ in range(3)]
    for o in outs:  # in flight together, each call with one frame for both cameras
        assert p.r.render([frame, frame], o, p.luts, check=True)
    # decoder frames: the same NV12 planes for both cameras
    planes = list(O.bgr32_to_yuv(frame, O.FMT_NV12))
    conv = O.yuv_to_bgr32(planes, O.FMT_NV12)
    pref = p.oracle_render([conv, conv], p.luts)[..., :3]
    pout = np.zeros((H, W, 4), np.uint8)
    assert p.r.render_planar([planes, planes], pout, p.luts, src_fmt=P.PS_FMT_NV12, check=True)
    torch.cuda.synchronize()
    for o in outs:
        assert np.array_equal(o[..., :3], ref), diff_histogram(o[..., :3], ref)
    assert np.array_equal(pout[..., :3], pref), diff_histogram(pout[..., :3], pref)


def test_ricoh_argument_checks(cuda):
    cfg = S.scaled_rig(S.rig("ricoh"), 4)
    W, H = cfg.dst_size
    r = P.CudaRicohPanoramaRender()
    frame = np.zeros((cfg.src_size[1], cfg.src_size[0], 4), np.uint8)
    out = np.zeros((H, W, 4), np.uint8)
    assert not r.render([frame], out)  # not prepared
    assert "prepare" in r.last_error
    three = cfg.cams + [S.photo_param(3, 200.0, 90.0, crop_x=0, crop_y=0, crop_width=cfg.src_size[1],
                                      crop_height=cfg.src_size[1])]
    assert not r.prepare(three, 1, cfg.levels, cfg.src_size, cfg.dst_size)  # RicohUtil.cpp:1368-1373
    assert "requires 2" in r.last_error and r.getNumImages() == 0
    assert r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size)
    assert not r.render([frame, frame], out)  # RicohUtil.cpp:1387-1391
    assert "requires 1" in r.last_error
    with pytest.raises(P.PsError):
        r.render([], out, check=True)
    assert r.render([frame], out, check=True)
