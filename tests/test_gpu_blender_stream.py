"""The blender fed one camera at a time, the memory queries and the render's
low-memory path (GPU).

CudaTilingMultibandBlendFast::begin / tile / end (source/CudaAccel/
CudaMultibandBlend.cpp:737-783) must give exactly the bytes of blend(), and,
with a camera left out, exactly the blend of the others with that camera's
image zero (the reference accumulates only the tiled cameras and still
divides by every camera's weights).  getUniqueMasks returns the seams,
calcUsedMemorySize stays within estimateMemorySize.  The render's low-memory
path (fewer frames in flight when the estimate does not fit the memory it
may take, source/Task/RicohUtil.cpp:1135-1170) stitches the same bytes.
"""
import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rig(cuda, oracle_lib):
    cfg = S.scaled_rig(S.rig("c2"), 8)
    maps = [O.reproject_map(c, cfg.src_size, cfg.dst_size) for c in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    frames = S.FrameSource(cfg).frame(2)
    luts = S.luts(cfg)
    level0 = [O.reproject_16s(frames[i], maps[i][0], maps[i][1], luts[i]) for i in range(cfg.num_cams)]
    return cfg, cov, seams, level0


def _blender(rig):
    cfg, cov, seams, level0 = rig
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(seams), cfg.levels), b.last_error
    return b


def test_tiles_equal_blend_and_oracle(rig):
    import torch
    cfg, cov, seams, level0 = rig
    H, W = cov.shape[1:]
    b = _blender(rig)
    ref = O.Blender(cov, seams, cfg.levels).blend(level0)[..., :3]
    whole = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    b.blend([torch.from_numpy(x).cuda() for x in level0], whole)
    buf = torch.empty((H, W, 4), dtype=torch.int16, device="cuda")  # one buffer serves every camera
    for rep in range(2):
        tiled = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
        b.begin()
        for i in reversed(range(cfg.num_cams)):  # any order
            buf.copy_(torch.from_numpy(level0[i]))
            b.tile(buf, i)
        b.end(tiled)
        torch.cuda.synchronize()
        got = tiled.cpu().numpy()[..., :3]
        assert np.array_equal(got, whole.cpu().numpy()[..., :3]), rep
        assert np.array_equal(got, ref), diff_histogram(got, ref)


def test_untiled_camera_contributes_nothing(rig):
    import torch
    cfg, cov, seams, level0 = rig
    H, W = cov.shape[1:]
    b = _blender(rig)
    skip = 1
    imgs = [x if i != skip else np.zeros_like(x) for i, x in enumerate(level0)]
    ref = O.Blender(cov, seams, cfg.levels).blend(imgs)[..., :3]
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    b.begin()
    for i in range(cfg.num_cams):
        if i != skip:
            b.tile(torch.from_numpy(level0[i]).cuda(), i)
    b.end(out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()[..., :3]
    assert np.array_equal(got, ref), diff_histogram(got, ref)


def test_tile_argument_checks(rig):
    import torch
    cfg, cov, seams, level0 = rig
    H, W = cov.shape[1:]
    b = _blender(rig)
    img = torch.from_numpy(level0[0]).cuda()
    with pytest.raises(P.PsError) as e:
        b.tile(img, 0)
    assert e.value.code == L.PS_ESTATE
    b.begin()
    b.tile(img, 0)
    with pytest.raises(P.PsError) as e:
        b.tile(img, 0)
    assert e.value.code == L.PS_EINVAL
    with pytest.raises(P.PsError) as e:
        b.tile(img, cfg.num_cams)
    assert e.value.code == L.PS_EINVAL
    bad = torch.zeros((H, W, 4), dtype=torch.int16, device="cuda")
    bad[0, 0, 0] = 300
    with pytest.raises(P.PsError) as e:
        b.tile(bad, 1)
    assert e.value.code == L.PS_EINVAL
    b.end(torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda"))
    with pytest.raises(P.PsError) as e:
        b.end(torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda"))
    assert e.value.code == L.PS_ESTATE


def test_unique_masks_and_memory(rig):
    cfg, cov, seams, level0 = rig
    H, W = cov.shape[1:]
    b = _blender(rig)
    got = b.get_unique_masks((W, H))
    assert all(np.array_equal(g, s) for g, s in zip(got, seams))
    used = b.calc_used_memory_size()
    est = P.CudaTilingMultibandBlendFast.estimate_memory_size(W, H, cfg.num_cams, cfg.levels)
    assert 0 < used <= est
    assert P.CudaTilingMultibandBlendFast.estimate_memory_size(0, H, 2) == -1


def test_render_low_memory_path(cuda, oracle_lib):
    cfg = S.scaled_rig(S.rig("c2"), 4)
    est = {k: P.CudaPanoramaRender2.estimate_memory(cfg.cams, cfg.levels, cfg.src_size, cfg.dst_size, k)
           for k in (1, 2, 8)}
    assert est[1] < est[2] < est[8]
    for budget, slots in ((est[2], 2), (est[1], 1), (0, 8)):
        r = P.CudaPanoramaRender2()
        r.set_memory_budget(budget)
        r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
        assert r.frames_in_flight == slots
        assert r.low_memory == (slots < 8) and not r.map_free  # one slot with maps still fits
        assert r.resident_bytes <= est[slots]
        seams = r.get_unique_masks()
        assert all(np.array_equal(s, r.seam(i, cfg.dst_size)) for i, s in enumerate(seams))
    p = Prepared(cfg)  # the oracle from the product's own geometry
    frames = [p.frames.frame(k) for k in range(3)]
    r.set_memory_budget(est[1])
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    assert r.frames_in_flight == 1 and not r.map_free
    W, H = cfg.dst_size
    for f in frames:  # consecutive frames share the one state slot
        out = np.zeros((H, W, 4), np.uint8)
        r.render(f, out, p.luts, check=True)
        import torch
        torch.cuda.synchronize()
        ref = p.oracle_render(f, p.luts)[..., :3]
        assert np.array_equal(out[..., :3], ref), diff_histogram(out[..., :3], ref)
