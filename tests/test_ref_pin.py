"""The oracle against the reference's own code, run here (CPU).

oracle/_ref/libpsref.so is the reference's geometry and CPU remap
(source/Warp/Remap.cpp, ZReproject.cpp), its integer pyramid kernels and
wrappers (source/CudaAccel/CudaPyramid2.cu) chained as
CudaTilingMultibandBlendFast::prepare/blend chains them, its YUV
conversions (source/CudaAccel/ImageProc.cu) and its CPU multiband blend
class TilingMultibandBlendFast (source/Blend/MultiBandBlend.cpp with
Pyramid.cpp), compiled unchanged by
`make -C oracle ref`; the kernels run on host cores under oracle/ref/cuda_emu.
It can only be built where the reference tree is present, so these tests
skip elsewhere; the committed fixtures of tests/golden/ carry the same pin
(tests/test_golden.py).

Bar: geometry, coverage, every pyramid, the blend and the YUV conversions
bit for bit; the remap bit for bit except where the reference reads one
pixel past the row end (floor(x) = W - 1), which the oracle clamps.
"""
import concurrent.futures as cf

import numpy as np
import pytest

import oracle as O
from oracle import ref as R
from panostitcher_gb300 import synth as S

pytestmark = pytest.mark.skipif(not R.available(), reason="reference tree absent: oracle/_ref not built")

SCALED = [("c1", 8), ("c2", 16), ("c3a", 16), ("c3c", 16), ("c3d", 32), ("c5", 32), ("ricoh", 8)]


def apply_luts(frame, lut):
    out = frame.copy()
    for c in range(3):
        out[..., c] = lut[c][frame[..., c]]
    return out


def geometry_pair(cfg, i):
    p = cfg.cams[i]
    xm, ym, mk, m64 = O.reproject_map(p, cfg.src_size, cfg.dst_size, with_double=True)
    rm, rk = R.reproject_map(p, cfg.src_size, cfg.dst_size)
    return m64, mk, rm, rk, xm, ym


@pytest.mark.parametrize("name,factor", SCALED + [("c1", 1), ("c2", 1)])
def test_geometry_bit_exact(oracle_lib, name, factor):
    cfg = S.rig(name) if factor == 1 else S.scaled_rig(S.rig(name), factor)
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        for m64, mk, rm, rk, _, _ in ex.map(lambda i: geometry_pair(cfg, i), range(cfg.num_cams)):
            assert np.array_equal(m64.view(np.uint64), rm.view(np.uint64))
            assert np.array_equal(mk, rk)


@pytest.mark.parametrize("channels", [4, 3])
@pytest.mark.parametrize("name,factor", SCALED)
def test_remap_matches_reference(oracle_lib, name, factor, channels):
    cfg = S.scaled_rig(S.rig(name), factor)
    frames = S.FrameSource(cfg, channels).frame(3)
    luts = S.luts(cfg)
    sw = cfg.src_size[0]
    for i in range(cfg.num_cams):
        _, mk, _, _, xm, ym = geometry_pair(cfg, i)
        ours = O.reproject_16s(frames[i], xm, ym, luts[i])
        m64 = np.stack([xm.astype(np.float64), ym.astype(np.float64)], -1)
        theirs = R.reproject_16s(apply_luts(frames[i], luts[i]), m64)
        bad = (ours[..., :3] != theirs[..., :3]).any(-1)
        quirk = (mk > 0) & (np.floor(xm) == sw - 1)
        assert not (bad & ~quirk).any()
        assert np.all(theirs[mk == 0] == 0)


def blend_case(cov, seams, level0, levels):
    ob = O.Blender(cov, seams, levels)
    out, norm, coll = ob.blend(level0, pyramids=True)
    rout, rp = R.mb_blend(cov, seams, level0, ob.levels, pyramids=True)
    assert np.array_equal(out[..., :3], rout[..., :3])
    for j in range(ob.levels + 1):
        assert np.array_equal(coll[j][..., :3], rp["coll"][j][..., :3]), f"collapsed level {j}"
        assert np.array_equal(norm[j][..., :3], rp["norm"][j][..., :3]), f"normalised level {j}"
        for i in range(cov.shape[0]):
            assert np.array_equal(ob.weight(i, j), rp["weight"][i][j]), f"weight {i} level {j}"
            if j:
                assert np.array_equal(ob.alpha(i, j), rp["alpha"][i][j]), f"alpha {i} level {j}"
    return ob


@pytest.mark.parametrize("name,factor", SCALED)
def test_rig_blend_bit_exact(oracle_lib, name, factor):
    cfg = S.scaled_rig(S.rig(name), factor)
    frames = S.FrameSource(cfg).frame(1)
    luts = S.luts(cfg)
    geo = [geometry_pair(cfg, i) for i in range(cfg.num_cams)]
    cov = np.stack([g[1] for g in geo])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    level0 = [O.reproject_16s(frames[i], geo[i][4], geo[i][5], luts[i]) for i in range(cfg.num_cams)]
    blend_case(cov, seams, level0, cfg.levels)


def random_partition(rng, W, H, n, full):
    cov = np.zeros((n, H, W), np.uint8)
    for i in range(n):
        y0, y1 = sorted(rng.integers(0, H + 1, 2))
        x0 = rng.integers(0, W)
        cols = (x0 + np.arange(rng.integers(1, W + 1))) % W
        cov[i][max(0, y0 - 1):max(y1, y0 + 1)][:, cols] = 255
    if full:
        cov[0][:] = 255
    best = np.where(cov > 0, rng.random((n, H, W)), -1).argmax(0)
    covered = cov.max(0) > 0
    seams = np.stack([((best == i) & covered).astype(np.uint8) * 255 for i in range(n)])
    imgs = rng.integers(0, 256, (n, H, W, 4)).astype(np.int16)
    imgs[..., 3] = 0
    imgs[cov == 0] = 0
    return cov, seams, list(imgs)


@pytest.mark.parametrize("W,H,n,levels,full", [(3, 2, 2, 4, False), (5, 3, 2, 4, True), (33, 17, 3, 5, False),
                                               (130, 67, 4, 8, False), (257, 129, 5, 8, True),
                                               (96, 48, 12, 6, False), (512, 256, 2, 8, False)])
def test_partition_blend_bit_exact(oracle_lib, W, H, n, levels, full):
    rng = np.random.default_rng(W * 31 + H + n)
    cov, seams, imgs = random_partition(rng, W, H, n, full)
    ob = blend_case(cov, seams, imgs, levels)
    if full:
        assert ob.full_mask


def cpu_blend_case(cov, seams, level0, max_levels, min_length=2):
    """The CPU-semantics restatement against the reference's own TilingMultibandBlendFast: output,
    collapsed pyramid, weight and alpha pyramids, at one and at several host threads."""
    ob = O.CpuBlender(cov, seams, max_levels, min_length)
    rout, rp = R.cpu_mb_blend(cov, seams, level0, max_levels, min_length)
    for nthreads in (1, 4):
        out, coll = ob.blend(level0, pyramids=True, nthreads=nthreads)
        assert np.array_equal(out, rout), f"output, {nthreads} threads"
        for j in range(ob.levels + 1):
            assert np.array_equal(coll[j], rp["coll"][j]), f"collapsed level {j}, {nthreads} threads"
    for i in range(cov.shape[0]):
        for j in range(ob.levels + 1):
            assert np.array_equal(ob.weight(i, j), rp["weight"][i][j]), f"weight {i} level {j}"
            if j:
                assert np.array_equal(ob.alpha(i, j), rp["alpha"][i][j]), f"alpha {i} level {j}"
    return ob


@pytest.mark.parametrize("name,factor", SCALED)
def test_rig_cpu_blend_bit_exact(oracle_lib, name, factor):
    cfg = S.scaled_rig(S.rig(name), factor)
    frames = S.FrameSource(cfg).frame(1)
    luts = S.luts(cfg)
    geo = [geometry_pair(cfg, i) for i in range(cfg.num_cams)]
    cov = np.stack([g[1] for g in geo])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    level0 = [O.reproject_16s(frames[i], geo[i][4], geo[i][5], luts[i]) for i in range(cfg.num_cams)]
    cpu_blend_case(cov, seams, level0, cfg.levels)


@pytest.mark.parametrize("W,H,n,levels,full", [(33, 17, 3, 5, False), (130, 67, 4, 8, False),
                                               (257, 129, 5, 8, True), (96, 48, 12, 6, False),
                                               (512, 256, 2, 8, False)])
def test_partition_cpu_blend_bit_exact(oracle_lib, W, H, n, levels, full):
    rng = np.random.default_rng(W * 31 + H + n)
    cov, seams, imgs = random_partition(rng, W, H, n, full)
    ob = cpu_blend_case(cov, seams, imgs, levels)
    if full:
        assert ob.full_mask


@pytest.mark.parametrize("W,H", [(1, 1), (2, 1), (1, 6), (3, 2), (5, 3), (7, 5), (9, 4), (4, 4)])
def test_tiny_cpu_blend_bit_exact(oracle_lib, W, H):
    """Sizes down to one pixel with the shortest side length 1, so that every level's border mapping
    (wrapped columns, reflected rows, the one-pixel cases) is exercised."""
    rng = np.random.default_rng(W * 7 + H)
    for full in (True, False):
        cov, seams, imgs = random_partition(rng, W, H, 2, full)
        cpu_blend_case(cov, seams, imgs, 16, 1)


@pytest.mark.parametrize("W,H", [(2, 2), (66, 34), (130, 66), (640, 360)])
def test_yuv_bit_exact(oracle_lib, W, H):
    rng = np.random.default_rng(W + H)
    bgr = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    for fmt in (O.FMT_YUV420P, O.FMT_NV12):
        for a, b in zip(O.bgr32_to_yuv(bgr, fmt), R.bgr32_to_yuv(bgr, fmt)):
            assert np.array_equal(a, b)
        planes = [rng.integers(0, 256, p.shape, dtype=np.uint8) for p in O.bgr32_to_yuv(bgr, fmt)]
        assert np.array_equal(O.yuv_to_bgr32(planes, fmt)[..., :3], R.yuv_to_bgr32(planes, fmt)[..., :3])
