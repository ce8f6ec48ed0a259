"""Parity of the reference seam rule, getNonIntersectingMasks
(source/Blend/Mask.cpp:376-398), and of its exact L1 distance transform
(GPU).  The device computes the transform separably (row scans, column
sweeps); the oracle runs the two-pass 3x3 chamfer; both must agree exactly.
"""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu


def _blobs(rng, n, H, W):
    m = np.zeros((n, H, W), np.uint8)
    for i in range(n):
        for _ in range(rng.integers(1, 4)):
            y0, x0 = rng.integers(0, H), rng.integers(0, W)
            m[i, y0:y0 + rng.integers(1, H), x0:x0 + rng.integers(1, W)] = 255
    return m


@pytest.mark.parametrize("H,W", [(1, 1), (1, 37), (29, 1), (16, 16), (67, 130), (300, 601)])
def test_distance_transform_matches_oracle(cuda, oracle_lib, H, W):
    import torch
    rng = np.random.default_rng(H * 1000 + W)
    cases = [(rng.random((H, W)) < p).astype(np.uint8) * 255 for p in (0.5, 0.97, 1.0)]
    cases.append(np.zeros((H, W), np.uint8))
    for m in cases:
        dm = torch.from_numpy(m).cuda()
        dd = torch.empty((H, W), dtype=torch.int32, device="cuda")
        P.distance_transform_l1(dm, dd)
        got = np.minimum(dd.cpu().numpy(), O.DT_FAR)
        ref = np.minimum(O.distance_transform_l1(m), O.DT_FAR)
        assert np.array_equal(got, ref), diff_histogram(got, ref)


@pytest.mark.parametrize("n,H,W", [(1, 8, 8), (2, 40, 80), (4, 64, 128), (6, 101, 202), (9, 50, 300)])
def test_non_intersecting_masks_match_oracle(cuda, oracle_lib, n, H, W):
    import torch
    rng = np.random.default_rng(n * 7 + H)
    m = _blobs(rng, n, H, W)
    out = torch.empty((n, H, W), dtype=torch.uint8, device="cuda")
    P.non_intersecting_masks(torch.from_numpy(m).cuda(), out)
    got = out.cpu().numpy()
    ref = O.non_intersecting_masks(m)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("name,factor", [("c1", 8), ("c2", 8), ("c3c", 8)])
def test_render_with_distance_seams_bit_exact(cuda, oracle_lib, name, factor):
    cfg = S.scaled_rig(S.rig(name), factor)
    r = P.CudaPanoramaRender2()
    r.set_seam_rule(P.PS_SEAMS_DISTANCE)
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    n = cfg.num_cams
    cov = np.stack([r.coverage(i, cfg.dst_size) for i in range(n)])
    seams = np.stack([r.seam(i, cfg.dst_size) for i in range(n)])
    assert np.array_equal(seams, O.non_intersecting_masks(cov))
    # the whole render with those seams against the oracle
    p = Prepared(cfg, seams=list(seams))
    frames = p.frames.frame(0)
    assert np.array_equal(p.product_render(frames, p.luts)[..., :3], p.oracle_render(frames, p.luts)[..., :3])


def test_blender_derives_reference_seams(cuda, oracle_lib):
    import torch
    rng = np.random.default_rng(21)
    n, H, W = 3, 66, 130
    masks = _blobs(rng, n, H, W)
    masks[0, :, :] = np.where(rng.random((H, W)) < 0.9, 255, 0)
    seams = O.non_intersecting_masks(masks)
    imgs = [rng.integers(0, 256, (H, W, 4)).astype(np.int16) for _ in range(n)]
    for im, m in zip(imgs, masks):
        im[..., 3] = 0
        im[m == 0] = 0  # warped images are zero outside their coverage
    outs = []
    for s in (None, list(seams)):
        b = P.CudaTilingMultibandBlendFast()
        assert b.prepare(list(masks), s, 5), b.last_error
        dst = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
        b.blend([torch.from_numpy(im).cuda() for im in imgs], dst)
        torch.cuda.synchronize()
        outs.append(dst.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    ob = O.Blender(masks, seams, 5)
    ref = ob.blend(imgs)
    assert np.array_equal(outs[0][..., :3], ref[..., :3]), diff_histogram(outs[0][..., :3], ref[..., :3])


def test_seam_rule_rejects_unknown(cuda):
    r = P.CudaPanoramaRender2()
    with pytest.raises(P.PsError):
        r.set_seam_rule(7)
