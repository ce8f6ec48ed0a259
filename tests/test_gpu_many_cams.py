"""Many cameras per tile (GPU): the blend's overflow camera lists (more than
eight cameras on a tile), the tail kernel's multi-chunk units, and the
64-camera maximum, bit-exact against the oracle.  Coverage rectangles
overlap heavily and the seams are a random per-pixel partition, so every
tile of every level sees many cameras; one case has a camera that covers
nothing."""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P

from _util import diff_histogram

pytestmark = pytest.mark.gpu


def _overlapping(rng, n, H, W, empty=()):
    cov = np.zeros((n, H, W), np.uint8)
    for i in range(n):
        if i in empty:
            continue
        y0 = int(rng.integers(0, H // 2))
        y1 = int(rng.integers(H // 2 + 1, H + 1))
        x0 = int(rng.integers(0, W))
        cols = (x0 + np.arange(int(rng.integers(W // 2, W + 1)))) % W
        cov[i][y0:y1][:, cols] = 255
    score = rng.random((n, H, W))
    score[cov == 0] = -1
    best = score.argmax(0)
    covered = cov.max(0) > 0
    seams = np.zeros_like(cov)
    for i in range(n):
        seams[i][(best == i) & covered] = 255
    return cov, seams


@pytest.mark.parametrize("n,W,H,levels,empty", [(12, 130, 67, 6, ()), (20, 64, 32, 5, (3,)),
                                                (64, 96, 48, 5, ()), (64, 258, 130, 8, (0, 63))])
def test_blender_many_cameras_bit_exact(cuda, oracle_lib, n, W, H, levels, empty):
    import torch
    rng = np.random.default_rng(n * 7919 + W)
    cov, seams = _overlapping(rng, n, H, W, empty)
    ob = O.Blender(cov, seams, levels)
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(seams), levels), b.last_error
    imgs = []
    for i in range(n):
        im = rng.integers(0, 256, (H, W, 4)).astype(np.int16)
        im[..., 3] = 0
        im[cov[i] == 0] = 0
        imgs.append(im)
    ref = ob.blend(imgs)
    dev = [torch.from_numpy(im).cuda() for im in imgs]
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    for _ in range(2):  # the second run replays the same launches
        b.blend(dev, out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()[..., :3]
        assert np.array_equal(got, ref[..., :3]), diff_histogram(got, ref[..., :3])


def test_blender_more_than_max_cameras_rejected(cuda):
    n, H, W = 65, 16, 32
    cov = np.full((n, H, W), 255, np.uint8)
    b = P.CudaTilingMultibandBlendFast()
    assert not b.prepare(list(cov), None, 4)
    assert b.num_levels == 0


def test_intersecting_seams_rejected(cuda):
    """Explicit seams must not intersect, as getNonIntersectingMasks' never
    do: the collapsed levels are int16, bounded only while the seam weights
    at a pixel sum to at most 256.  Both prepares reject shared pixels and
    name the first one."""
    n, H, W = 3, 48, 96
    cov = np.full((n, H, W), 255, np.uint8)
    seams = np.zeros_like(cov)
    seams[0][:, :40] = 255
    seams[1][:, 40:] = 255
    seams[2][5, 41] = 255  # also camera 1's
    b = P.CudaTilingMultibandBlendFast()
    assert not b.prepare(list(cov), list(seams), 4)
    assert "intersect at (41, 5)" in b.last_error and b.num_levels == 0
    seams[2][5, 41] = 0
    assert b.prepare(list(cov), list(seams), 4), b.last_error
    # the render's prepare with explicit seams
    from panostitcher_gb300 import synth as S
    cfg = S.scaled_rig(S.rig("c2"), 8)
    W, H = cfg.dst_size
    full = np.zeros((cfg.num_cams, H, W), np.uint8)
    full[0][:, : W // 2] = 255
    full[1][:, W // 2:] = 255
    full[1][3, 7] = 255
    r = P.CudaPanoramaRender2()
    assert not r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, seams=list(full))
    assert "seam masks 0 and 1 intersect at (7, 3)" in r.last_error and r.getNumImages() == 0
