"""Parity of the linear-blend render mode (highQualityBlend == 0; GPU).

The weights (Gaussian-feathered seam masks, getWeightsLinearBlend32F) must
equal the oracle's bit for bit given the same coverage and seams, and the
render (fp32 weighted accumulation of the warped frames, convertTo CV_8U)
must equal the oracle's render bit for bit given the same maps and weights.
"""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import diff_histogram

pytestmark = pytest.mark.gpu

CASES = [("c1", 8, 6, P.PS_SEAMS_NEAREST_AXIS), ("c2", 8, 10, P.PS_SEAMS_NEAREST_AXIS),
         ("c2", 12, 4, P.PS_SEAMS_DISTANCE), ("c3c", 8, 16, P.PS_SEAMS_DISTANCE)]


class Linear:
    def __init__(self, name, factor, radius, rule, graph=True):
        self.cfg = cfg = S.scaled_rig(S.rig(name), factor)
        self.r = P.CudaPanoramaRender2()
        self.r.set_seam_rule(rule)
        self.r.set_graph(graph)
        self.r.prepare(cfg.cams, 0, radius, cfg.src_size, cfg.dst_size, check=True)
        n = cfg.num_cams
        self.maps = [self.r.maps(i, cfg.dst_size) for i in range(n)]
        self.cov = np.stack([self.r.coverage(i, cfg.dst_size) for i in range(n)])
        self.seams = np.stack([self.r.seam(i, cfg.dst_size) for i in range(n)])
        self.w = np.stack([self.r.linear_weight(i, cfg.dst_size) for i in range(n)])
        self.radius = radius
        self.frames = S.FrameSource(cfg)
        self.luts = S.luts(cfg)

    def oracle(self, frames, luts):
        return O.linear_render(frames, luts, [m[0] for m in self.maps], [m[1] for m in self.maps], self.w)

    def product(self, frames, luts, channels=4):
        import torch
        W, H = self.cfg.dst_size
        dst = np.zeros((H, W, channels), np.uint8)
        self.r.render(frames, dst, luts, check=True)
        torch.cuda.synchronize()
        return dst


@pytest.mark.parametrize("name,factor,radius,rule", CASES)
def test_linear_weights_bit_exact(cuda, oracle_lib, name, factor, radius, rule):
    p = Linear(name, factor, radius, rule)
    ref = O.linear_weights(p.cov, p.seams, radius)
    assert np.array_equal(p.w.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("name,factor,radius,rule", CASES)
def test_linear_render_bit_exact(cuda, oracle_lib, name, factor, radius, rule):
    p = Linear(name, factor, radius, rule)
    for f in (0, 1):
        frames = p.frames.frame(f)
        got = p.product(frames, p.luts)
        ref = p.oracle(frames, p.luts)
        assert np.array_equal(got, ref), diff_histogram(got[..., :3], ref[..., :3])


def test_linear_io_variants(cuda, oracle_lib):
    import torch
    p = Linear("c2", 8, 8, P.PS_SEAMS_NEAREST_AXIS, graph=False)
    W, H = p.cfg.dst_size
    frames = p.frames.frame(2)
    ref = p.oracle(frames, None)
    assert np.array_equal(p.product(frames, None), ref)
    assert np.array_equal(p.product(frames, None, channels=3), ref[..., :3])
    dev_frames = [torch.from_numpy(np.ascontiguousarray(f)).cuda() for f in frames]
    dst = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    p.r.render(dev_frames, dst, None, check=True)
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy(), ref)


def test_linear_and_multiband_batch(cuda, oracle_lib):
    import torch
    lin = Linear("c1", 8, 5, P.PS_SEAMS_NEAREST_AXIS)
    cfg = S.scaled_rig(S.rig("c2"), 8)
    mb = P.CudaPanoramaRender2()
    mb.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    fl, fm = lin.frames.frame(0), S.FrameSource(cfg).frame(0)
    singles = []
    for r, c, fr, lt in ((lin.r, lin.cfg, fl, lin.luts), (mb, cfg, fm, S.luts(cfg))):
        d = torch.zeros((c.dst_size[1], c.dst_size[0], 4), dtype=torch.uint8, device="cuda")
        r.render([torch.from_numpy(f).cuda() for f in fr], d, lt, check=True)
        singles.append(d)
    dsts = [torch.zeros_like(d) for d in singles]
    P.render_batch([lin.r, mb], [[torch.from_numpy(f).cuda() for f in fl], [torch.from_numpy(f).cuda() for f in fm]],
                   dsts, [lin.luts, S.luts(cfg)])
    torch.cuda.synchronize()
    for a, b in zip(singles, dsts):
        assert torch.equal(a, b)


def test_linear_rejects(cuda):
    cfg = S.scaled_rig(S.rig("c1"), 8)
    r = P.CudaPanoramaRender2()
    assert not r.prepare(cfg.cams, 0, 1025, cfg.src_size, cfg.dst_size)
    assert "radius" in r.last_error
    r.prepare(cfg.cams, 0, 4, cfg.src_size, cfg.dst_size, check=True)
    W, H = cfg.dst_size
    planes = [np.zeros((H, W), np.uint8), np.zeros((H // 2, W // 2), np.uint8), np.zeros((H // 2, W // 2), np.uint8)]
    assert not r.render_yuv(S.FrameSource(cfg).frame(0), planes)
    assert "BGR" in r.last_error
