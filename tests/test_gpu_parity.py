"""Parity of the CUDA path with the oracle (GPU).

Bars: pyramids, weights, accumulators and the blended output are bit-exact
given identical warped inputs; the bilinear remap must be within +-1 LSB per
channel of the double-precision oracle (this implementation is designed to
be exact and the strict test checks that); maps within 1e-3 px of the
double-precision geometry.
"""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu

SMALL = [("c1", 8), ("c1", 4), ("c2", 8), ("c3c", 8), ("c3a", 16), ("c5", 16)]


def _cfg(name, factor):
    return S.scaled_rig(S.rig(name), factor)


@pytest.mark.parametrize("name,factor", [("c1", 4), ("c2", 8), ("c3d", 16)])
def test_maps_and_coverage_match_oracle(cuda, oracle_lib, name, factor):
    cfg = _cfg(name, factor)
    p = Prepared(cfg)
    npx = cfg.canvas_pixels
    for i, cam in enumerate(cfg.cams):
        xm, ym, mk = O.reproject_map(cam, cfg.src_size, cfg.dst_size)
        px, py = p.maps[i]
        cov_mismatch = int(np.count_nonzero((mk > 0) != (p.cov[i] > 0)))
        assert cov_mismatch <= max(4, npx // 100000), cov_mismatch
        both = (mk > 0) & (p.cov[i] > 0)
        assert np.abs(px[both] - xm[both]).max(initial=0) <= 1e-3
        assert np.abs(py[both] - ym[both]).max(initial=0) <= 1e-3


@pytest.mark.parametrize("name,factor", [("c1", 4), ("c2", 8)])
def test_nearest_axis_seams_match_oracle(cuda, oracle_lib, name, factor):
    cfg = _cfg(name, factor)
    p = Prepared(cfg)
    ref = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, p.cov)
    mism = int(np.count_nonzero(ref != p.seams))
    assert mism <= max(4, cfg.canvas_pixels // 100000), mism
    # invariants of getNonIntersectingMasks: subset of coverage, partition of the union
    assert ((p.seams > 0) <= (p.cov > 0)).all()
    assert ((p.seams > 0).sum(0) == (p.cov.max(0) > 0)).all()


@pytest.mark.parametrize("name,factor", [("c1", 4), ("c2", 8), ("c5", 16)])
def test_remap_within_one_lsb_and_exact(cuda, oracle_lib, name, factor):
    import torch
    cfg = _cfg(name, factor)
    p = Prepared(cfg)
    frames = p.frames.frame(3)
    W, H = cfg.dst_size
    hist_total = {}
    for i in range(cfg.num_cams):
        src = torch.from_numpy(frames[i]).cuda()
        xm = torch.from_numpy(p.maps[i][0]).cuda()
        ym = torch.from_numpy(p.maps[i][1]).cuda()
        lut = torch.from_numpy(p.luts[i].reshape(-1).copy()).cuda()
        out = torch.empty((H, W, 4), dtype=torch.int16, device="cuda")
        P.reproject_to_16s(src, xm, ym, out, lut)
        got = out.cpu().numpy()
        ref = O.reproject_16s(frames[i], p.maps[i][0], p.maps[i][1], p.luts[i])
        for k, v in diff_histogram(got[..., :3], ref[..., :3]).items():
            hist_total[k] = hist_total.get(k, 0) + v
        assert (got[..., 3] == 0).all()
    print("remap delta histogram", hist_total)
    assert max(abs(k) for k in hist_total) <= 1          # the +-1 LSB bar
    assert set(hist_total) == {0}, hist_total            # this implementation is exact


@pytest.mark.parametrize("name,factor", [("c1", 8), ("c2", 8)])
def test_weight_and_alpha_pyramids_bit_exact(cuda, oracle_lib, name, factor):
    cfg = _cfg(name, factor)
    p = Prepared(cfg)
    ob = p.ob
    assert p.r.num_levels == ob.levels
    assert p.r.full_mask == ob.full_mask
    for i in range(cfg.num_cams):
        for j in range(ob.levels + 1):
            w, h = ob.sizes[j]
            got_w = p.r.export(P._lib.EXPORT_WEIGHT, i, j, (h, w), np.int16)
            assert np.array_equal(got_w, ob.weight(i, j)), (i, j)
            if j:
                got_a = p.r.export(P._lib.EXPORT_ALPHA, i, j, (h, w), np.int32)
                assert np.array_equal(got_a, ob.alpha(i, j)), (i, j)


@pytest.mark.parametrize("name,factor", SMALL)
def test_render_bit_exact(cuda, oracle_lib, name, factor):
    cfg = _cfg(name, factor)
    p = Prepared(cfg)
    for f in (0, 1):
        frames = p.frames.frame(f)
        ref = p.oracle_render(frames, p.luts)
        got = p.product_render(frames, p.luts)
        assert np.array_equal(got[..., :3], ref[..., :3]), diff_histogram(got[..., :3], ref[..., :3])
        assert (got[..., 3] == 0).all()


@pytest.mark.parametrize("name,factor", [("c1", 8), ("c2", 8)])
def test_collapsed_pyramid_bit_exact(cuda, oracle_lib, name, factor):
    cfg = _cfg(name, factor)
    p = Prepared(cfg)
    frames = p.frames.frame(0)
    p.product_render(frames, p.luts)
    imgs = [O.reproject_16s(frames[i], p.maps[i][0], p.maps[i][1], p.luts[i]) for i in range(cfg.num_cams)]
    dst, norm, coll = p.ob.blend(imgs, pyramids=True)
    for j in range(1, p.ob.levels + 1):
        got = p.r.collapsed(j, p.ob.sizes[j]).astype(np.int32)
        assert np.array_equal(got[..., :3], coll[j][..., :3]), j


def test_render_without_luts_and_graph_off(cuda, oracle_lib):
    cfg = _cfg("c2", 8)
    p = Prepared(cfg, graph=False)
    frames = p.frames.frame(5)
    assert np.array_equal(p.product_render(frames, None)[..., :3], p.oracle_render(frames, None)[..., :3])


def test_device_io_bgr24_bgr32_agree(cuda, oracle_lib):
    import torch
    cfg = _cfg("c1", 8)
    p = Prepared(cfg)
    frames = p.frames.frame(2)
    ref = p.oracle_render(frames, p.luts)
    W, H = cfg.dst_size
    dev_src = [torch.from_numpy(f).cuda() for f in frames]
    dev_dst = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    p.r.render(dev_src, dev_dst, p.luts, check=True)
    torch.cuda.synchronize()
    assert np.array_equal(dev_dst.cpu().numpy()[..., :3], ref[..., :3])
    f24 = [np.ascontiguousarray(f[..., :3]) for f in frames]
    out24 = p.product_render(f24, p.luts, channels_out=3)
    assert np.array_equal(out24, ref[..., :3])
    dev24 = [torch.from_numpy(f).cuda() for f in f24]
    dst24 = torch.zeros((H, W, 3), dtype=torch.uint8, device="cuda")
    p.r.render(dev24, dst24, p.luts, check=True)
    torch.cuda.synchronize()
    assert np.array_equal(dst24.cpu().numpy(), ref[..., :3])


def test_alternating_source_formats(cuda, oracle_lib):
    """The remap is specialised for BGR32 sources; a state slot whose recorded launches were made for the
    other format records them again.  Twenty renders alternate the formats over the eight slots, and a batch
    mixes them (the remap then takes the format from each frame)."""
    import torch
    cfg = _cfg("c1", 8)
    p = Prepared(cfg)
    W, H = cfg.dst_size
    frames = [p.frames.frame(k) for k in (3, 4)]
    refs = [p.oracle_render(f, p.luts)[..., :3] for f in frames]
    dst = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    for k in range(20):
        f = frames[k % 2]
        src = [torch.from_numpy(np.ascontiguousarray(x if k % 3 else x[..., :3])).cuda() for x in f]
        p.r.render(src, dst, p.luts, check=True)
        torch.cuda.synchronize()
        assert np.array_equal(dst.cpu().numpy()[..., :3], refs[k % 2]), k
    q = Prepared(_cfg("c3c", 8))
    fq = q.frames.frame(1)
    dsts = [np.zeros((c.dst_size[1], c.dst_size[0], 4), np.uint8) for c in (cfg, q.cfg)]
    for _ in range(2):
        P.render_batch([p.r, q.r], [[np.ascontiguousarray(x[..., :3]) for x in frames[0]], fq], dsts,
                       [p.luts, q.luts])
        cuda.cuda.synchronize()
        assert np.array_equal(dsts[0][..., :3], refs[0])
        assert np.array_equal(dsts[1][..., :3], q.oracle_render(fq, q.luts)[..., :3])


def test_explicit_seams(cuda, oracle_lib):
    cfg = _cfg("c2", 8)
    base = Prepared(cfg)
    # move every seam pixel of camera 0 that camera 1 also covers to camera 1
    seams = base.seams.copy()
    move = (seams[0] > 0) & (base.cov[1] > 0)
    seams[0][move] = 0
    seams[1][move] = 255
    p = Prepared(cfg, seams=list(seams))
    assert np.array_equal(p.seams, seams)
    frames = p.frames.frame(0)
    assert np.array_equal(p.product_render(frames, p.luts)[..., :3], p.oracle_render(frames, p.luts)[..., :3])


def test_batch_equals_single(cuda, oracle_lib):
    cfgs = [_cfg("c1", 8), _cfg("c2", 8), _cfg("c3c", 8), _cfg("c3a", 16)]
    ps = [Prepared(c) for c in cfgs]
    frames = [p.frames.frame(7) for p in ps]
    singles = [p.product_render(f, p.luts) for p, f in zip(ps, frames)]
    dsts = [np.zeros((c.dst_size[1], c.dst_size[0], 4), np.uint8) for c in cfgs]
    for _ in range(2):  # second call replays the captured graph
        P.render_batch([p.r for p in ps], frames, dsts, [p.luts for p in ps])
        cuda.cuda.synchronize()
        for d, s in zip(dsts, singles):
            assert np.array_equal(d, s)


def _random_partition(rng, n, H, W):
    """n coverage masks (random rectangles, wrapping) and a seam partition."""
    cov = np.zeros((n, H, W), np.uint8)
    for i in range(n):
        y0, y1 = sorted(rng.integers(0, H + 1, 2))
        x0 = rng.integers(0, W)
        wdt = rng.integers(1, W + 1)
        cols = (x0 + np.arange(wdt)) % W
        cov[i][max(0, y0 - 1):max(y1, y0 + 1)][:, cols] = 255
    owner = np.full((H, W), -1)
    score = rng.random((n, H, W))
    score[cov == 0] = -1
    best = score.argmax(0)
    covered = cov.max(0) > 0
    seams = np.zeros_like(cov)
    for i in range(n):
        seams[i][(best == i) & covered] = 255
    return cov, seams


@pytest.mark.parametrize("W,H,levels", [(3, 2, 4), (5, 4, 4), (33, 17, 5), (94, 47, 6), (130, 67, 8),
                                        (257, 129, 16)])
def test_blender_odd_sizes_bit_exact(cuda, oracle_lib, W, H, levels):
    import torch
    rng = np.random.default_rng(W * 1000 + H)
    n = 3
    cov, seams = _random_partition(rng, n, H, W)
    ob = O.Blender(cov, seams, levels)
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(seams), levels), b.last_error
    assert b.num_levels == ob.levels
    imgs = []
    for i in range(n):
        im = rng.integers(0, 256, (H, W, 4)).astype(np.int16)
        im[..., 3] = 0
        im[cov[i] == 0] = 0
        imgs.append(im)
    ref = ob.blend(imgs)
    dev = [torch.from_numpy(im).cuda() for im in imgs]
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    b.blend(dev, out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy()[..., :3], ref[..., :3])


def test_blender_kat_single_camera_identity(cuda):
    import torch
    rng = np.random.default_rng(1)
    H, W = 96, 192
    mk = np.full((H, W), 255, np.uint8)
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare([mk], [mk], 6)
    img = rng.integers(0, 256, (H, W, 4)).astype(np.uint8)
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    b.blend([torch.from_numpy(img).cuda()], out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy()[..., :3], img[..., :3])


def test_blender_rejects_bad_inputs(cuda):
    import torch
    H, W = 16, 32
    mk = np.zeros((H, W), np.uint8)
    mk[:, :16] = 255
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare([mk], [mk], 3)
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    bad = torch.zeros((H, W, 4), dtype=torch.int16, device="cuda")
    bad[0, 0, 0] = 300
    with pytest.raises(P.PsError) as e:
        b.blend([bad], out)
    assert e.value.code == P._lib.PS_EINVAL
    outside = torch.zeros((H, W, 4), dtype=torch.int16, device="cuda")
    outside[0, 20, 1] = 5      # non-zero where the coverage mask is 0
    with pytest.raises(P.PsError):
        b.blend([outside], out)


@pytest.mark.parametrize("name", ["c1", "c2", "c3a", "c3c", "c3d", "ricoh", "c5"])
def test_render_full_size_bit_exact(cuda, oracle_lib, name):
    """Every benchmark rig at full size: every kernel path (bulk-copied interior
    tiles, border tiles, uniform tiles, the tail kernel) against the oracle,
    up to the largest ones (8 x 2704x2028 and 8 x 3840x2160 -> 7680x3840, 8 and
    10 levels)."""
    import os
    cfg = S.rig(name)
    p = Prepared(cfg)
    frames = p.frames.frame(9)
    ref = p.oracle_render(frames, p.luts, nthreads=os.cpu_count() or 4)
    got = p.product_render(frames, p.luts)
    assert np.array_equal(got[..., :3], ref[..., :3]), diff_histogram(got[..., :3], ref[..., :3])
