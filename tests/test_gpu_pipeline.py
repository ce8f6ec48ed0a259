"""Renders in flight together (GPU).

A render keeps eight sets of per-frame state, so consecutive calls with host
buffers, and calls issued on several streams, overlap on the GPU.  Every frame
must still come out exactly as the oracle stitches it alone.
"""
import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu

FRAMES = 6


@pytest.fixture(scope="module")
def prepared(cuda, oracle_lib):
    p = Prepared(S.scaled_rig(S.rig("c2"), 8))
    frames = [p.frames.frame(k) for k in range(FRAMES)]
    refs = [p.oracle_render(f, p.luts)[..., :3] for f in frames]
    return p, frames, refs


def test_host_buffers_back_to_back(prepared):
    import torch
    p, frames, refs = prepared
    W, H = p.cfg.dst_size
    outs = [np.zeros((H, W, 4), np.uint8) for _ in frames]
    for f, o in zip(frames, outs):  # no synchronisation between the calls
        assert p.r.render(f, o, p.luts, check=True)
    torch.cuda.synchronize()
    for k, (o, ref) in enumerate(zip(outs, refs)):
        assert np.array_equal(o[..., :3], ref), (k, diff_histogram(o[..., :3], ref))


def test_device_buffers_on_two_streams(prepared):
    import torch
    p, frames, refs = prepared
    W, H = p.cfg.dst_size
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    dev_frames = [[torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in f] for f in frames]
    outs = [torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda") for _ in frames]
    torch.cuda.synchronize()
    for k in range(FRAMES):
        assert p.r.render(dev_frames[k], outs[k], p.luts, stream=streams[k % 2], check=True)
    torch.cuda.synchronize()
    for k, (o, ref) in enumerate(zip(outs, refs)):
        got = o.cpu().numpy()[..., :3]
        assert np.array_equal(got, ref), (k, diff_histogram(got, ref))


def test_yuv_and_bgr_interleaved(prepared):
    import oracle as O
    import torch
    p, frames, refs = prepared
    W, H = p.cfg.dst_size
    bgr = [np.zeros((H, W, 4), np.uint8) for _ in range(3)]
    nv12 = [[np.zeros((H, W), np.uint8), np.zeros((H // 2, W), np.uint8)] for _ in range(3)]
    for k in range(3):
        assert p.r.render(frames[2 * k], bgr[k], p.luts, check=True)
        assert p.r.render_yuv(frames[2 * k + 1], nv12[k], p.luts, P.PS_FMT_NV12, check=True)
    torch.cuda.synchronize()
    for k in range(3):
        assert np.array_equal(bgr[k][..., :3], refs[2 * k])
        full = np.zeros((H, W, 4), np.uint8)
        full[..., :3] = refs[2 * k + 1]
        for got, want in zip(nv12[k], O.bgr32_to_yuv(full, O.FMT_NV12)):
            assert np.array_equal(got, want)


@pytest.mark.parametrize("slots", [1, 3])
def test_fewer_frames_in_flight(cuda, oracle_lib, slots):
    torch = cuda
    cfg = S.scaled_rig(S.rig("c2"), 8)
    full = Prepared(cfg)
    r = P.CudaPanoramaRender2()
    r.set_frames_in_flight(slots)
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    assert r.frames_in_flight == slots and full.r.frames_in_flight == P.PS_MAX_IN_FLIGHT
    assert r.resident_bytes < full.r.resident_bytes  # fewer sets of per-frame state
    W, H = cfg.dst_size
    frames = [full.frames.frame(k) for k in range(5)]
    outs = [np.zeros((H, W, 4), np.uint8) for _ in frames]
    for f, o in zip(frames, outs):  # more calls than slots, no synchronisation
        assert r.render(f, o, full.luts, check=True)
    torch.cuda.synchronize()
    for f, o in zip(frames, outs):
        ref = full.oracle_render(f, full.luts)[..., :3]
        assert np.array_equal(o[..., :3], ref), diff_histogram(o[..., :3], ref)


def test_prepare_again_with_frames_in_flight(cuda, oracle_lib):
    """A new prepare (and clear) while frames are still in flight waits for
    them before freeing their state: the frames finish with the old rig, the
    next frames use the new one."""
    torch = cuda
    a = Prepared(S.scaled_rig(S.rig("c2"), 8))
    b_cfg = S.scaled_rig(S.rig("c3c"), 8)
    b = Prepared(b_cfg)
    fa = [a.frames.frame(k) for k in range(3)]
    refs_a = [a.oracle_render(f, a.luts)[..., :3] for f in fa]
    fb = b.frames.frame(0)
    ref_b = b.oracle_render(fb, b.luts)[..., :3]
    r = P.CudaPanoramaRender2()
    assert r.prepare(a.cfg.cams, 1, a.cfg.levels, a.cfg.src_size, a.cfg.dst_size, check=True)
    Wa, Ha = a.cfg.dst_size
    st = torch.cuda.Stream()
    dev = [[torch.from_numpy(np.ascontiguousarray(c)).cuda() for c in f] for f in fa]
    outs = [torch.zeros((Ha, Wa, 4), dtype=torch.uint8, device="cuda") for _ in fa]
    host_out = np.zeros((Ha, Wa, 4), np.uint8)
    torch.cuda.synchronize()
    for k in range(3):
        assert r.render(dev[k], outs[k], a.luts, stream=st, check=True)
    assert r.render(fa[0], host_out, a.luts, check=True)  # a host frame in flight too
    # no synchronisation: prepare the other rig at once
    assert r.prepare(b_cfg.cams, 1, b_cfg.levels, b_cfg.src_size, b_cfg.dst_size, check=True)
    Wb, Hb = b_cfg.dst_size
    ob = np.zeros((Hb, Wb, 4), np.uint8)
    assert r.render(fb, ob, b.luts, check=True)
    torch.cuda.synchronize()
    for k in range(3):
        got = outs[k].cpu().numpy()[..., :3]
        assert np.array_equal(got, refs_a[k]), (k, diff_histogram(got, refs_a[k]))
    assert np.array_equal(host_out[..., :3], refs_a[0])
    assert np.array_equal(ob[..., :3], ref_b), diff_histogram(ob[..., :3], ref_b)
    r.clear()
    assert r.getNumImages() == 0
