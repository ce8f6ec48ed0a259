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


@pytest.mark.parametrize("n,W,H,levels", [(3, 130, 67, 6), (12, 96, 48, 5)])
def test_blender_overlapping_seams_bit_exact(cuda, oracle_lib, n, W, H, levels):
    """Explicit seams that overlap (each camera's seam is its whole
    coverage): weight sums reach 256 n, so the normalisation divides by sums
    from 256 up to 768 (three cameras) and past the 1024 of its table (twelve
    cameras), with partial coverage."""
    import torch
    rng = np.random.default_rng(n * 104729 + W)
    cov, _ = _overlapping(rng, n, H, W)
    cov[:, :2, :3] = 0  # an uncovered corner: the weighted normalisation, not the full-mask shift
    ob = O.Blender(cov, cov, levels)
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(cov), levels), b.last_error
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
    got = out.cpu().numpy()[..., :3]
    assert np.array_equal(got, ref[..., :3]), diff_histogram(got, ref[..., :3])
