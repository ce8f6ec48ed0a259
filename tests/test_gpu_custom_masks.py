"""Custom masks (GPU): CudaTilingMultibandBlendFast::blend(images, masks,
blendImage) (source/CudaAccel/CudaMultibandBlend.cpp:825-893) as the Tasks
use it per frame interval (source/Task/PanoramaPreviewTask.cpp:382-400).
Weights from the custom masks, the weighted normalisation whatever the
coverage, zeros outside the masks' union; bit-exact against the oracle, for
the blender and the render, with overlapping masks, with full and partial
coverage, switched while frames are in flight, and back to the unique
masks."""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu


def _blender_case(rng, n, H, W, full):
    cov = np.zeros((n, H, W), np.uint8)
    step = W // n
    for i in range(n):
        cols = (np.arange(i * step - step // 3, (i + 1) * step + step // 3)) % W
        cov[i][:, cols] = 255
    if not full:
        cov[:, : H // 4, : W // 5] = 0
    seams = np.zeros_like(cov)
    own = (np.arange(W) // step).clip(0, n - 1)
    for i in range(n):
        seams[i][:, own == i] = 255
    seams &= cov
    return cov, seams


@pytest.mark.parametrize("full", [False, True], ids=["partial", "full"])
def test_blender_custom_masks_bit_exact(cuda, oracle_lib, full):
    torch = cuda
    rng = np.random.default_rng(77 + full)
    n, H, W, levels = 4, 96, 192, 5
    cov, seams = _blender_case(rng, n, H, W, full)
    ob = O.Blender(cov, seams, levels)
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(seams), levels), b.last_error
    imgs = []
    for i in range(n):
        im = rng.integers(0, 256, (H, W, 4)).astype(np.int16)
        im[..., 3] = 0
        im[cov[i] == 0] = 0
        imgs.append(im)
    dev = [torch.from_numpy(im).cuda() for im in imgs]
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")

    def check(tag):
        ref = ob.blend(imgs)
        b.blend(dev, out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()[..., :3]
        assert np.array_equal(got, ref[..., :3]), (tag, diff_histogram(got, ref[..., :3]))
        return got

    check("unique")
    # overlapping custom masks: a band shared by cameras 1 and 2, and camera 0 given a disc
    custom = seams.copy()
    custom[1][:, W // 4: W // 2 + 20] = 255
    custom[2][:, W // 2 - 20: 3 * W // 4] = 255
    yy, xx = np.mgrid[:H, :W]
    custom[0][(yy - H // 2) ** 2 + (xx - W // 3) ** 2 < (H // 4) ** 2] = 255
    custom[3][: H // 3] = 0  # a strip no mask covers: zero in the output
    for tag, masks in (("custom", custom), ("unique as custom", seams), ("unique", None), ("custom again", custom)):
        ob.set_custom_masks(masks)
        assert b.set_custom_masks(None if masks is None else list(masks)), b.last_error
        got = check(tag)
    outside = custom.max(0) == 0  # no custom mask: zero, whatever the coverage
    assert outside.any() and not got[outside].any()


def test_render_custom_masks_bit_exact_and_in_flight(cuda, oracle_lib):
    torch = cuda
    cfg = S.scaled_rig(S.rig("c2"), 8)
    p = Prepared(cfg)
    W, H = cfg.dst_size
    n = cfg.num_cams
    # an interval's masks: camera 0 takes over a band of camera 1's seam, camera 2 a disc that overlaps others
    custom = p.seams.copy()
    band = (p.cov[0] > 0) & (p.seams[1] > 0)
    band[: H // 2] = False
    custom[0][band] = 255
    custom[1][band] = 0
    yy, xx = np.mgrid[:H, :W]
    custom[2][((yy - H // 2) ** 2 + (xx - W // 2) ** 2 < (H // 5) ** 2) & (p.cov[2] > 0)] = 255
    frames = [p.frames.frame(k) for k in range(4)]
    refs_unique = [p.oracle_render(f, p.luts)[..., :3] for f in frames[:2]]
    p.ob.set_custom_masks(custom)
    refs_custom = [p.oracle_render(f, p.luts)[..., :3] for f in frames[2:]]
    p.ob.set_custom_masks(None)
    outs = [np.zeros((H, W, 4), np.uint8) for _ in frames]
    # two frames in flight with the unique masks, then the interval's masks, with no synchronisation
    assert p.r.render(frames[0], outs[0], p.luts, check=True)
    assert p.r.render(frames[1], outs[1], p.luts, check=True)
    assert p.r.set_custom_masks(list(custom), check=True)
    assert p.r.render(frames[2], outs[2], p.luts, check=True)
    assert p.r.render(frames[3], outs[3], p.luts, check=True)
    torch.cuda.synchronize()
    for k, ref in enumerate(refs_unique + refs_custom):
        assert np.array_equal(outs[k][..., :3], ref), (k, diff_histogram(outs[k][..., :3], ref))
    # back to the unique masks
    assert p.r.set_custom_masks(None, check=True)
    assert np.array_equal(p.product_render(frames[0], p.luts)[..., :3], refs_unique[0])
    # wrong count, and the linear-blend mode
    assert not p.r.set_custom_masks(list(custom[:2]))
    assert "custom masks given" in p.r.last_error
    lin = P.CudaPanoramaRender2()
    assert lin.prepare(cfg.cams, 0, 20, cfg.src_size, cfg.dst_size, check=True)
    assert not lin.set_custom_masks(list(custom))
    assert "multiband" in lin.last_error
