"""Parity of the encoder handoff, BGR32 -> YUV420P / NV12 (GPU).

The render's fused output (ps_render_render_yuv) must equal, byte for byte,
the oracle's conversion of the oracle's render, and the standalone
conversion (ps_cvt_bgr32_to_yuv) the oracle's conversion of the same image.
Canvases cover the three level-0 paths: the tail kernel (few tiles), the
level-0 blend kernel, and a height that leaves the last tile row partial.
"""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu

FMTS = [P.PS_FMT_YUV420P, P.PS_FMT_NV12]
RIGS = [("c1", 16), ("c2", 8), ("c2", 12)]


def _shapes(W, H, fmt):
    return [(H, W), (H // 2, W)] if fmt == P.PS_FMT_NV12 else [(H, W), (H // 2, W // 2), (H // 2, W // 2)]


def _host_planes(W, H, fmt, pad=0):
    """Padded host planes pre-filled with a marker, as views of width W."""
    return [np.full((h, w + pad), 7, np.uint8)[:, :w] for h, w in _shapes(W, H, fmt)]


def _device_planes(W, H, fmt, pad=0):
    import torch
    return [torch.full((h, w + pad), 7, dtype=torch.uint8, device="cuda")[:, :w] for h, w in _shapes(W, H, fmt)]


def _oracle_planes(bgr32, fmt):
    return O.bgr32_to_yuv(np.ascontiguousarray(bgr32), O.FMT_NV12 if fmt == P.PS_FMT_NV12 else O.FMT_YUV420P)


@pytest.mark.parametrize("fmt", FMTS)
@pytest.mark.parametrize("W,H", [(2, 2), (64, 8), (130, 66), (1000, 502)])
def test_cvt_matches_oracle(cuda, oracle_lib, fmt, W, H):
    import torch
    rng = np.random.default_rng(W * 7 + H + fmt)
    host = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    src = torch.zeros((H, W + 3, 4), dtype=torch.uint8, device="cuda")[:, :W]
    src.copy_(torch.from_numpy(host))
    planes = _device_planes(W, H, fmt, pad=5)
    P.cvt_bgr32_to_yuv(src, planes, fmt)
    torch.cuda.synchronize()
    for got, ref in zip(planes, _oracle_planes(host, fmt)):
        assert np.array_equal(got.cpu().numpy(), ref), diff_histogram(got.cpu().numpy(), ref)


@pytest.mark.parametrize("fmt", FMTS)
@pytest.mark.parametrize("name,factor", RIGS)
def test_render_yuv_equals_converted_render(cuda, oracle_lib, name, factor, fmt):
    import torch
    cfg = S.scaled_rig(S.rig(name), factor)
    W, H = cfg.dst_size
    p = Prepared(cfg)
    for f in (0, 1):
        frames = p.frames.frame(f)
        ref = _oracle_planes(p.oracle_render(frames, p.luts), fmt)
        host = _host_planes(W, H, fmt, pad=3)
        assert p.r.render_yuv(frames, host, p.luts, fmt, check=True)
        dev = _device_planes(W, H, fmt, pad=9)
        assert p.r.render_yuv(frames, dev, p.luts, fmt, check=True)
        torch.cuda.synchronize()
        for k, r in enumerate(ref):
            assert np.array_equal(host[k], r), (k, diff_histogram(host[k], r))
            d = dev[k].cpu().numpy()
            assert np.array_equal(d, r), (k, diff_histogram(d, r))
        # the BGR render of the same frame is untouched by the YUV path
        bgr = p.product_render(frames, p.luts)
        assert np.array_equal(bgr[..., :3], p.oracle_render(frames, p.luts)[..., :3])


def test_render_yuv_graph_off_and_no_luts(cuda, oracle_lib):
    import torch
    cfg = S.scaled_rig(S.rig("c2"), 8)
    W, H = cfg.dst_size
    p = Prepared(cfg, graph=False)
    frames = p.frames.frame(3)
    ref = _oracle_planes(p.oracle_render(frames, None), P.PS_FMT_NV12)
    dev = _device_planes(W, H, P.PS_FMT_NV12)
    assert p.r.render_yuv(frames, dev, None, P.PS_FMT_NV12, check=True)
    torch.cuda.synchronize()
    for d, r in zip(dev, ref):
        assert np.array_equal(d.cpu().numpy(), r)


def test_yuv_rejects_bad_inputs(cuda):
    import torch
    cfg = S.scaled_rig(S.rig("c1"), 16)
    W, H = cfg.dst_size
    r = P.CudaPanoramaRender2()
    frames = S.FrameSource(cfg).frame(0)
    # before prepare
    assert not r.render_yuv(frames, _host_planes(W, H, P.PS_FMT_YUV420P))
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    # wrong size
    assert not r.render_yuv(frames, _host_planes(W - 2, H, P.PS_FMT_YUV420P))
    assert "size" in r.last_error
    # pitch too small: a U plane narrower than W/2
    bad = _host_planes(W, H, P.PS_FMT_YUV420P)
    bad[1] = np.zeros((H // 2, W // 2 - 2), np.uint8)
    assert not r.render_yuv(frames, bad)
    # standalone conversion: odd sizes, non-BGR32, host memory
    src = torch.zeros((5, 6, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(P.PsError):
        P.cvt_bgr32_to_yuv(src, _device_planes(6, 5, P.PS_FMT_NV12)[:1] + [torch.zeros((2, 6), dtype=torch.uint8,
                                                                                        device="cuda")],
                           P.PS_FMT_NV12)
    with pytest.raises(P.PsError):
        P.cvt_bgr32_to_yuv(torch.zeros((4, 6, 3), dtype=torch.uint8, device="cuda"),
                           _device_planes(6, 4, P.PS_FMT_NV12), P.PS_FMT_NV12)
    with pytest.raises(P.PsError):
        P.cvt_bgr32_to_yuv(torch.zeros((4, 6, 4), dtype=torch.uint8, device="cuda"),
                           _host_planes(6, 4, P.PS_FMT_NV12), P.PS_FMT_NV12)
    # the render still works after the rejected calls
    good = _host_planes(W, H, P.PS_FMT_YUV420P)
    assert r.render_yuv(frames, good, None, check=True)
