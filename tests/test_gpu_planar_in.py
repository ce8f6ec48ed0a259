"""Parity of the decoder handoff, YUV420P / NV12 -> BGR32 (GPU).

The standalone conversion (ps_cvt_yuv_to_bgr32) must equal the oracle's
conversion byte for byte, and a render from decoder frames
(ps_render_render_planar) must equal the oracle's render of the oracle's
conversion of the same frames: host and device planes, both formats, mixed
per camera, BGR or planar output, and several renders in flight.
"""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu

FMTS = [P.PS_FMT_YUV420P, P.PS_FMT_NV12]


def _ofmt(fmt):
    return O.FMT_NV12 if fmt == P.PS_FMT_NV12 else O.FMT_YUV420P


def _random_planes(rng, W, H, fmt):
    y = rng.integers(0, 256, (H, W), dtype=np.uint8)
    if fmt == P.PS_FMT_NV12:
        return [y, rng.integers(0, 256, (H // 2, W), dtype=np.uint8)]
    return [y, rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8),
            rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8)]


def _device_padded(torch, a, pad):
    t = torch.zeros((a.shape[0], a.shape[1] + pad), dtype=torch.uint8, device="cuda")[:, :a.shape[1]]
    t.copy_(torch.from_numpy(a))
    return t


def _host_padded(a, pad):
    h = np.full((a.shape[0], a.shape[1] + pad), 3, np.uint8)[:, :a.shape[1]]
    h[...] = a
    return h


# ppad 0 with W % 8 == 0 and an aligned destination takes the 8-pixel vector
# path; other pads and widths the per-block path (odd dpad: 4-byte stores)
@pytest.mark.parametrize("fmt", FMTS)
@pytest.mark.parametrize("W,H,ppad,dpad", [(2, 2, 0, 0), (64, 8, 5, 1), (130, 66, 5, 3), (1000, 502, 5, 0),
                                           (1000, 502, 0, 0), (64, 8, 0, 0), (136, 70, 8, 4)])
def test_cvt_matches_oracle(cuda, oracle_lib, fmt, W, H, ppad, dpad):
    torch = cuda
    rng = np.random.default_rng(W + 3 * H + fmt + ppad)
    planes = _random_planes(rng, W, H, fmt)
    dev = [_device_padded(torch, p, ppad) for p in planes]
    dst = torch.full((H, W + dpad, 4), 9, dtype=torch.uint8, device="cuda")[:, :W]
    P.cvt_yuv_to_bgr32(dev, dst, fmt)
    torch.cuda.synchronize()
    got = dst.cpu().numpy()
    ref = O.yuv_to_bgr32(planes, _ofmt(fmt))
    assert np.array_equal(got, ref), diff_histogram(got, ref)


@pytest.fixture(scope="module")
def rig(cuda, oracle_lib):
    p = Prepared(S.scaled_rig(S.rig("c2"), 4))  # 480x270 sources: decoder frames are even-sized
    return p


def _decoder_frames(p, k, fmts):
    """Camera frames of frame k as decoder planes (fmts per camera), and the
    BGR32 frames the oracle converts them to."""
    bgr = p.frames.frame(k)
    planes = [list(O.bgr32_to_yuv(b, _ofmt(f))) for b, f in zip(bgr, fmts)]
    conv = [O.yuv_to_bgr32(pl, _ofmt(f)) for pl, f in zip(planes, fmts)]
    return planes, conv


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("fmt", FMTS)
def test_render_planar_equals_oracle(cuda, rig, fmt, where):
    torch = cuda
    p = rig
    W, H = p.cfg.dst_size
    n = p.cfg.num_cams
    for k in (0, 1):
        planes, conv = _decoder_frames(p, k, [fmt] * n)
        ref = p.oracle_render(conv, p.luts)[..., :3]
        if where == "device":
            src = [[_device_padded(torch, a, 7) for a in pl] for pl in planes]
        else:
            src = [[_host_padded(a, 2) for a in pl] for pl in planes]
        out = np.zeros((H, W, 4), np.uint8)
        assert p.r.render_planar(src, out, p.luts, src_fmt=fmt, check=True)
        torch.cuda.synchronize()
        assert np.array_equal(out[..., :3], ref), diff_histogram(out[..., :3], ref)


def test_render_planar_mixed_formats_and_planar_output(cuda, rig):
    torch = cuda
    p = rig
    W, H = p.cfg.dst_size
    n = p.cfg.num_cams
    fmts = [FMTS[i % 2] for i in range(n)]
    planes, conv = _decoder_frames(p, 2, fmts)
    ref = p.oracle_render(conv, p.luts)
    # cameras alternate formats; every other camera's planes on the device
    src = []
    for i, (pl, f) in enumerate(zip(planes, fmts)):
        src.append(([_device_padded(torch, a, 1) for a in pl] if i % 2 else pl, f))
    for ofmt in FMTS:
        full = np.zeros((H, W, 4), np.uint8)
        full[..., :3] = ref[..., :3]
        want = O.bgr32_to_yuv(full, _ofmt(ofmt))
        got = [np.zeros_like(w) for w in want]
        assert p.r.render_planar(src, luts=p.luts, ydst=got, ydst_fmt=ofmt, check=True)
        torch.cuda.synchronize()
        for g, w in zip(got, want):
            assert np.array_equal(g, w), diff_histogram(g, w)


def test_render_planar_in_flight_with_bgr_renders(cuda, rig):
    torch = cuda
    p = rig
    W, H = p.cfg.dst_size
    n = p.cfg.num_cams
    jobs = []
    for k in range(6):
        planes, conv = _decoder_frames(p, k, [P.PS_FMT_NV12] * n)
        jobs.append((planes, conv, p.frames.frame(k)))
    outs = [np.zeros((H, W, 4), np.uint8) for _ in range(12)]
    for k, (planes, _, bgr) in enumerate(jobs):  # no synchronisation between the calls
        assert p.r.render_planar(planes, outs[2 * k], p.luts, src_fmt=P.PS_FMT_NV12, check=True)
        assert p.r.render(bgr, outs[2 * k + 1], p.luts, check=True)
    torch.cuda.synchronize()
    for k, (_, conv, bgr) in enumerate(jobs):
        assert np.array_equal(outs[2 * k][..., :3], p.oracle_render(conv, p.luts)[..., :3])
        assert np.array_equal(outs[2 * k + 1][..., :3], p.oracle_render(bgr, p.luts)[..., :3])


def test_render_planar_rejects_bad_inputs(cuda, rig):
    p = rig
    W, H = p.cfg.dst_size
    Ws, Hs = p.cfg.src_size
    n = p.cfg.num_cams
    good = [[np.zeros((Hs, Ws), np.uint8), np.zeros((Hs // 2, Ws), np.uint8)] for _ in range(n)]
    out = np.zeros((H, W, 4), np.uint8)
    assert not p.r.render_planar(good[:-1], out)  # one camera short
    assert "source frames" in p.r.last_error
    bad = [list(g) for g in good]
    bad[1] = [np.zeros((Hs, Ws - 2), np.uint8), np.zeros((Hs // 2, Ws - 2), np.uint8)]
    assert not p.r.render_planar(bad, out)  # wrong size
    assert not p.r.render_planar(good)  # neither dst nor ydst
    ydst = [np.zeros((H, W), np.uint8), np.zeros((H // 2, W), np.uint8)]
    assert not p.r.render_planar(good, out, ydst=ydst)  # both
    assert "exactly one" in p.r.last_error
    assert p.r.render_planar(good, out, check=True)  # the render still works
    # a rig whose sources are odd-sized takes no decoder frames
    odd = S.scaled_rig(S.rig("c2"), 8)
    r = P.CudaPanoramaRender2()
    r.prepare(odd.cams, 1, odd.levels, odd.src_size, odd.dst_size, check=True)
    w, h = odd.src_size
    assert h % 2
    frames = [[np.zeros((h, w), np.uint8), np.zeros((h // 2, w), np.uint8)] for _ in range(odd.num_cams)]
    assert not r.render_planar(frames, np.zeros((odd.dst_size[1], odd.dst_size[0], 4), np.uint8))
    assert "even" in r.last_error


def test_full_size_decoder_and_encoder_handoffs(cuda, oracle_lib):
    """The bench's planar leg at full size: 6 x 1920x1080 NV12 host frames in,
    4096x2048 NV12 host planes out, against the oracle's conversion, render
    and conversion of the same frames; and the same frames as BGR24 host
    images against the oracle's render of them."""
    import os
    torch = cuda
    p = Prepared(S.rig("c2"))
    W, H = p.cfg.dst_size
    n = p.cfg.num_cams
    planes, conv = _decoder_frames(p, 5, [P.PS_FMT_NV12] * n)
    ref = np.zeros((H, W, 4), np.uint8)
    ref[..., :3] = p.oracle_render(conv, p.luts, nthreads=os.cpu_count() or 4)[..., :3]
    want = O.bgr32_to_yuv(ref, O.FMT_NV12)
    got = [np.zeros_like(w) for w in want]
    assert p.r.render_planar(planes, luts=p.luts, ydst=got, ydst_fmt=P.PS_FMT_NV12, check=True)
    torch.cuda.synchronize()
    for g, w in zip(got, want):
        assert np.array_equal(g, w), diff_histogram(g, w)
    bgr24 = [np.ascontiguousarray(f[..., :3]) for f in p.frames.frame(6)]
    ref24 = p.oracle_render([np.concatenate([f, np.zeros_like(f[..., :1])], axis=2) for f in bgr24], p.luts,
                            nthreads=os.cpu_count() or 4)[..., :3]
    out = p.product_render(bgr24, p.luts)[..., :3]
    assert np.array_equal(out, ref24), diff_histogram(out, ref24)
