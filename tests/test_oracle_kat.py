"""Known-answer tests pinning the CPU oracle's restatement (CPU only).

The reference ships no golden vectors, so these pin the oracle by
properties its cited code must have: exact border index formulas, constant
images through the filters, the single-camera identity of the multiband
blend, round-half-even LUTs, and the geometry invariants.
"""
import numpy as np
import pytest

import oracle as O
from panostitcher_gb300 import synth as S


def test_num_levels_matches_getTrueNumLevels(oracle_lib):
    # min(maxLevels<=16, floor(log2(W/2)), floor(log2(H/2)))
    assert O.num_levels(4096, 2048, 8) == 8
    assert O.num_levels(2048, 1024, 5) == 5
    assert O.num_levels(7680, 3840, 10) == 10
    assert O.num_levels(64, 32, 16) == 4
    assert O.num_levels(3, 2, 4) == 0
    assert O.num_levels(7680, 3840, 100) == 10   # floor(log2(3840 / 2))


def test_pyr_down_constant_and_borders(oracle_lib):
    for (h, w) in [(8, 8), (7, 9), (2, 3), (1, 5), (33, 65)]:
        a = np.full((h, w), 256, np.int16)
        s = O.pyr_down_16sc1_to_32sc1(a)
        assert (s == 256 * 256).all()
        assert (O.pyr_down_16sc1_to_16sc1(a) == 256).all()


def test_pyr_down_wrap_columns(oracle_lib):
    # a single bright column at x=0 leaks into the last output column via the horizontal wrap
    a = np.zeros((8, 16), np.int16)
    a[:, 0] = 256
    s = O.pyr_down_16sc1_to_32sc1(a)
    assert s[2, 0] == 6 * 256 * 16          # centre tap 6, column weights sum 16
    assert s[2, 7] == 1 * 256 * 16          # x = 2*7+2 = 16 wraps to column 0


def test_pyr_down_reflect101_rows(oracle_lib):
    a = np.zeros((8, 8), np.int16)
    a[1, :] = 256                           # row 1 is row -1's reflection
    s = O.pyr_down_16sc1_to_32sc1(a)
    assert s[0, 3] == (4 + 4) * 256 * 16    # taps -1 (-> 1) and +1 with weight 4 each


def test_masked_pyr_down_is_floor_of_weighted_mean(oracle_lib):
    rng = np.random.default_rng(0)
    img = rng.integers(0, 256, (10, 12, 4)).astype(np.int16)
    img[..., 3] = 0
    scale = np.full((5, 6), 256 * 256, np.int32)
    out = O.pyr_down_16sc4_masked(img, scale)
    ref = O.pyr_down_16sc1_to_32sc1(np.ascontiguousarray(img[..., 0]))
    assert np.array_equal(out[..., 0], ref * 256 // (256 * 256))
    zero = O.pyr_down_16sc4_masked(img, np.zeros((5, 6), np.int32))
    assert (zero == 0).all()


def test_pyr_up_constant(oracle_lib):
    for (h, w) in [(4, 4), (3, 5), (1, 1), (7, 2)]:
        a = np.zeros((h, w, 4), np.int16)
        a[..., :3] = 200
        for dsz in [(2 * w, 2 * h), (max(1, 2 * w - 1), max(1, 2 * h - 1))]:
            u = O.pyr_up_16sc4(a, dsz)
            assert (u[..., :3] == 200).all()
        b = np.zeros((h, w, 4), np.int32)
        b[..., :3] = -77
        assert (O.pyr_up_32sc4(b, (2 * w, 2 * h))[..., :3] == -77).all()


def test_blend_single_camera_identity(oracle_lib):
    rng = np.random.default_rng(3)
    for (H, W) in [(64, 128), (37, 91)]:
        img = rng.integers(0, 256, (H, W, 4)).astype(np.int16)
        img[..., 3] = 0
        mk = np.full((1, H, W), 255, np.uint8)
        b = O.Blender(mk, mk, 16)
        assert b.full_mask
        out = b.blend([img])
        assert np.array_equal(out[..., :3], img[..., :3].astype(np.uint8))


def test_blend_constant_images(oracle_lib):
    H, W = 48, 96
    cov = np.zeros((2, H, W), np.uint8)
    cov[0][:, :60] = 255
    cov[1][:, 40:] = 255
    seams = np.zeros_like(cov)
    seams[0][:, :50] = 255
    seams[1][:, 50:] = 255
    b = O.Blender(cov, seams, 4)
    imgs = []
    for i in range(2):
        im = np.zeros((H, W, 4), np.int16)
        im[cov[i] > 0, :3] = 123
        imgs.append(im)
    out = b.blend(imgs)
    assert (out[..., :3] == 123).all()


def test_blend_uncovered_pixels_are_zero(oracle_lib):
    H, W = 32, 64
    cov = np.zeros((1, H, W), np.uint8)
    cov[0][:, :40] = 255
    b = O.Blender(cov, cov, 3)
    assert not b.full_mask
    im = np.zeros((H, W, 4), np.int16)
    im[:, :40, :3] = 90
    out = b.blend([im])
    assert (out[:, 40:, :3] == 0).all()
    assert (out[:, :40, :3] == 90).all()


def test_lut_round_half_even(oracle_lib):
    l = O.get_lut(0.5)
    assert l[1] == 0 and l[3] == 2 and l[5] == 2 and l[255] == 128   # 0.5, 1.5, 2.5, 127.5
    assert np.array_equal(O.get_lut(1.0), np.arange(256))
    assert O.get_lut(2.0)[200] == 255
    for k in (0.8, 1.17, 1.3):
        assert np.array_equal(O.get_lut(k), S.lut_from_gain(k))


def test_bilinear_integer_coordinates_copy(oracle_lib):
    rng = np.random.default_rng(5)
    src = rng.integers(0, 256, (20, 30, 4)).astype(np.uint8)
    yy, xx = np.mgrid[0:20, 0:30].astype(np.float32)
    out = O.reproject_16s(src, xx, yy)
    assert np.array_equal(out[..., :3], src[..., :3].astype(np.int16))
    lut = np.stack([np.arange(256)[::-1]] * 3).astype(np.uint8)
    inv = O.reproject_16s(src, xx, yy, lut)
    assert np.array_equal(inv[..., :3], 255 - src[..., :3].astype(np.int16))


def test_bilinear_half_pixel_round_half_even(oracle_lib):
    src = np.zeros((2, 4, 3), np.uint8)
    src[0, :, 0] = [1, 2, 10, 11]
    xm = np.array([[0.5, 2.5]], np.float32)
    ym = np.zeros((1, 2), np.float32)
    out = O.reproject_16s(src, xm, ym)
    assert out[0, 0, 0] == 2 and out[0, 1, 0] == 10     # 1.5 -> 2, 10.5 -> 10


def test_maps_invalid_sentinel_and_mask(oracle_lib):
    cfg = S.scaled_rig(S.rig("c2"), 16)
    xm, ym, mk = O.reproject_map(cfg.cams[0], cfg.src_size, cfg.dst_size)
    assert ((xm == -1) == (mk == 0)).all() and ((ym == -1) == (mk == 0)).all()
    v = mk > 0
    assert (xm[v] >= 0).all() and (xm[v] < cfg.src_size[0]).all()
    # the yaw-0 rectilinear camera is centred on the canvas centre
    W, H = cfg.dst_size
    cx, cy = xm[H // 2, W // 2], ym[H // 2, W // 2]
    assert abs(cx - cfg.src_size[0] / 2) < 1.0 and abs(cy - cfg.src_size[1] / 2) < 1.0


def test_nearest_axis_seams_partition(oracle_lib):
    cfg = S.scaled_rig(S.rig("c2"), 16)
    cov = np.stack([O.reproject_map(c, cfg.src_size, cfg.dst_size)[2] for c in cfg.cams])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    assert ((seams > 0) <= (cov > 0)).all()
    assert ((seams > 0).sum(0) == (cov.max(0) > 0)).all()
    # the c2 rig leaves gaps between the side ring and the pole cameras
    assert not (cov.max(0) > 0).all()


def test_render_mt_equals_st(oracle_lib):
    cfg = S.scaled_rig(S.rig("c1"), 8)
    maps = [O.reproject_map(c, cfg.src_size, cfg.dst_size) for c in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    b = O.Blender(cov, seams, cfg.levels)
    fr = S.FrameSource(cfg).frame(0)
    a = b.render(fr, S.luts(cfg), [m[0] for m in maps], [m[1] for m in maps], 1)
    c = b.render(fr, S.luts(cfg), [m[0] for m in maps], [m[1] for m in maps], 3)
    assert np.array_equal(a, c)


# ---- encoder handoff (cvtBGR32ToYUV420P / NV12, ImageProc.cu:44-160) -------
@pytest.mark.parametrize("bgr,yuv", [
    ((0, 0, 0), (16, 128, 128)),        # black: studio-range floor
    ((255, 255, 255), (235, 128, 128)),  # white: studio-range ceiling
    ((0, 0, 255), (82, 90, 240)),        # red
    ((0, 255, 0), (145, 54, 34)),        # green
    ((255, 0, 0), (41, 240, 110)),       # blue
    ((128, 128, 128), (126, 128, 128)),
])
def test_yuv_known_answers(oracle_lib, bgr, yuv):
    img = np.zeros((2, 2, 4), np.uint8)
    img[..., :3] = bgr
    y, u, v = O.bgr32_to_yuv(img)
    assert (y == yuv[0]).all() and u[0, 0] == yuv[1] and v[0, 0] == yuv[2]
    # within one step of the real-valued BT.601 definition
    r, g, b = bgr[2], bgr[1], bgr[0]
    ref = (16 + (65.481 * r + 128.553 * g + 24.966 * b) / 255, 128 + (-37.797 * r - 74.203 * g + 112 * b) / 255,
           128 + (112 * r - 93.786 * g - 18.214 * b) / 255)
    assert all(abs(a - e) <= 1 for a, e in zip(yuv, ref))


def test_yuv_chroma_from_left_column_and_nv12_interleave(oracle_lib):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (6, 10, 4), dtype=np.uint8)
    y, u, v = O.bgr32_to_yuv(img)
    y2, uv = O.bgr32_to_yuv(img, O.FMT_NV12)
    assert np.array_equal(y, y2)
    assert np.array_equal(uv[:, 0::2], u) and np.array_equal(uv[:, 1::2], v)
    # the right column of every 2x2 block does not affect chroma
    img2 = img.copy()
    img2[:, 1::2, :3] = rng.integers(0, 256, img2[:, 1::2, :3].shape, dtype=np.uint8)
    _, u2, v2 = O.bgr32_to_yuv(img2)
    assert np.array_equal(u, u2) and np.array_equal(v, v2)
    # the 4th byte is ignored
    img3 = img.copy()
    img3[..., 3] = 255 - img3[..., 3]
    assert all(np.array_equal(a, b) for a, b in zip(O.bgr32_to_yuv(img3), (y, u, v)))


# ---- reference seams (getNonIntersectingMasks, Mask.cpp:376-398) ----------
def test_distance_transform_is_exact_l1(oracle_lib):
    rng = np.random.default_rng(11)
    for _ in range(40):
        H, W = rng.integers(1, 14, 2)
        m = (rng.random((H, W)) < rng.uniform(0.2, 1.0)).astype(np.uint8) * 255
        d = O.distance_transform_l1(m)
        zeros = np.argwhere(m == 0)
        if len(zeros) == 0:
            assert (d >= O.DT_FAR).all()
            continue
        yy, xx = np.mgrid[0:H, 0:W]
        brute = np.min(np.abs(yy[..., None] - zeros[:, 0]) + np.abs(xx[..., None] - zeros[:, 1]), axis=-1)
        assert np.array_equal(d, brute)


def test_non_intersecting_masks_split_overlaps_by_distance(oracle_lib):
    m = np.zeros((2, 20, 40), np.uint8)
    m[0, :, :25] = 255
    m[1, :, 15:] = 255
    u = O.non_intersecting_masks(m)
    # in the overlap (columns 15..24) column c goes to camera 1 where its distance to
    # camera 1's uncovered columns (c - 14) exceeds camera 0's (25 - c): c >= 20
    assert (u[0][:, :20] == 255).all() and (u[0][:, 20:] == 0).all()
    assert (u[1][:, 20:] == 255).all() and (u[1][:, :20] == 0).all()


def test_non_intersecting_masks_partition_random(oracle_lib):
    rng = np.random.default_rng(3)
    for n in (1, 2, 3, 5):
        m = np.zeros((n, 24, 48), np.uint8)
        for i in range(n):
            y0, x0 = rng.integers(0, 12), rng.integers(0, 30)
            m[i, y0:y0 + rng.integers(4, 14), x0:x0 + rng.integers(6, 20)] = 255
        u = O.non_intersecting_masks(m)
        assert ((u > 0) <= (m > 0)).all()
        assert ((u > 0).sum(0) == (m.max(0) > 0)).all()
        assert set(np.unique(u)) <= {0, 255}


# ---- linear blend (getWeightsLinearBlend32F + weighted accumulate) --------
def test_linear_weights_partition_of_unity(oracle_lib):
    cov = np.zeros((3, 24, 48), np.uint8)
    cov[0, :, :30] = 255
    cov[1, :, 18:] = 255
    cov[2, 4:20, 10:40] = 255
    seams = O.non_intersecting_masks(cov)
    for r in (1, 4, 9, 30):
        w = O.linear_weights(cov, seams, r)
        covered = cov.max(0) > 0
        s = w.sum(0)
        assert np.abs(s[covered] - 1).max() < 1e-6
        assert (s[~covered] == 0).all()
        assert (w[cov == 0] == 0).all()


def test_linear_render_identity_kat(oracle_lib):
    # two cameras with identical warped content: the weighted sum is the content
    H, W = 16, 32
    src = np.random.default_rng(0).integers(0, 256, (H, W, 4), dtype=np.uint8)
    yy, xx = np.mgrid[0:H, 0:W].astype(np.float32)
    cov = np.full((2, H, W), 255, np.uint8)
    cov[0, :, 24:] = 0
    cov[1, :, :8] = 0
    seams = O.non_intersecting_masks(cov)
    w = O.linear_weights(cov, seams, 3)
    xm = [np.where(cov[i] > 0, xx, -1).astype(np.float32) for i in range(2)]
    ym = [np.where(cov[i] > 0, yy, -1).astype(np.float32) for i in range(2)]
    out = O.linear_render([src, src], None, xm, ym, w)
    assert np.array_equal(out[..., :3], src[..., :3]) and (out[..., 3] == 0).all()


# ---- decoder frames: YUV420P / NV12 -> BGR32 (ImageProc.cu:165-222) ----------
def _yuv_to_bgr_numpy(y, u, v):
    """The reference arithmetic again, in numpy int64 (its >> is a floor)."""
    yy = np.maximum(y.astype(np.int64) - 16, 0) * 1220542
    cu = (u.astype(np.int64) - 128).repeat(2, 0).repeat(2, 1)
    cv = (v.astype(np.int64) - 128).repeat(2, 0).repeat(2, 1)
    half = 1 << 19
    out = np.zeros(y.shape + (4,), np.uint8)
    out[..., 0] = np.clip((yy + half + 2116026 * cu) >> 20, 0, 255)
    out[..., 1] = np.clip((yy + half - 852492 * cv - 409993 * cu) >> 20, 0, 255)
    out[..., 2] = np.clip((yy + half + 1673527 * cv) >> 20, 0, 255)
    return out


@pytest.mark.parametrize("yuv,bgr", [
    ((16, 128, 128), (0, 0, 0)),
    ((235, 128, 128), (255, 255, 255)),
    ((126, 128, 128), (128, 128, 128)),
    ((0, 128, 128), (0, 0, 0)),          # below the studio floor: max(Y - 16, 0)
    ((16, 0, 0), (0, 154, 0)),           # B and R sums negative: floor shift, then clamp
])
def test_yuv_to_bgr_known_answers(oracle_lib, yuv, bgr):
    y = np.full((2, 2), yuv[0], np.uint8)
    u = np.full((1, 1), yuv[1], np.uint8)
    v = np.full((1, 1), yuv[2], np.uint8)
    out = O.yuv_to_bgr32([y, u, v])
    assert (out[..., :3] == bgr).all(), out[0, 0]
    assert (out[..., 3] == 0).all()


def test_yuv_to_bgr_matches_restatement_and_nv12(oracle_lib):
    rng = np.random.default_rng(11)
    H, W = 34, 50
    y = rng.integers(0, 256, (H, W), dtype=np.uint8)
    u = rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8)
    v = rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8)
    u[0, :4] = [0, 255, 0, 255]  # extremes of both chroma planes
    v[0, :4] = [0, 0, 255, 255]
    out = O.yuv_to_bgr32([y, u, v])
    assert np.array_equal(out, _yuv_to_bgr_numpy(y, u, v))
    uv = np.empty((H // 2, W), np.uint8)
    uv[:, 0::2], uv[:, 1::2] = u, v
    assert np.array_equal(O.yuv_to_bgr32([y, uv], O.FMT_NV12), out)


def test_yuv_round_trip_of_block_constant_colours(oracle_lib):
    rng = np.random.default_rng(12)
    blk = rng.integers(0, 256, (16, 24, 3), dtype=np.uint8)
    img = np.zeros((32, 48, 4), np.uint8)
    img[..., :3] = blk.repeat(2, 0).repeat(2, 1)
    for fmt in (O.FMT_YUV420P, O.FMT_NV12):
        back = O.yuv_to_bgr32(O.bgr32_to_yuv(img, fmt), fmt)
        assert np.abs(back[..., :3].astype(int) - img[..., :3]).max() <= 2


def test_custom_masks_blend_properties(oracle_lib):
    """blend(images, masks, blendImage) (CudaMultibandBlend.cpp:825-893) in the oracle: with partial
    coverage, custom masks equal to the unique masks change nothing; another partition of the coverage
    blends as a blender prepared with it as its unique masks; masks narrower than the coverage zero the
    pixels outside their union; None restores the prepared blend; with full coverage the custom blend
    normalises by the weight sums."""
    rng = np.random.default_rng(2024)
    n, H, W, levels = 3, 40, 80, 4
    cov = np.zeros((n, H, W), np.uint8)
    cov[0][:, :34] = 255
    cov[1][:, 26:60] = 255
    cov[2][:, 52:] = 255
    cov[:, :3, :4] = 0  # an uncovered corner
    seams = np.zeros_like(cov)
    seams[0][:, :30] = 255
    seams[1][:, 30:56] = 255
    seams[2][:, 56:] = 255
    seams &= cov
    other = np.zeros_like(cov)
    other[0][:, :28] = 255
    other[1][:, 28:58] = 255
    other[2][:, 58:] = 255
    other &= cov
    imgs = []
    for i in range(n):
        im = rng.integers(0, 256, (H, W, 4)).astype(np.int16)
        im[..., 3] = 0
        im[cov[i] == 0] = 0
        imgs.append(im)
    b = O.Blender(cov, seams, levels)
    assert not b.full_mask
    ref = b.blend(imgs)
    b.set_custom_masks(seams)
    assert np.array_equal(b.blend(imgs), ref)
    b.set_custom_masks(other)
    assert np.array_equal(b.blend(imgs), O.Blender(cov, other, levels).blend(imgs))
    narrow = other.copy()
    narrow[:, :, :5] = 0
    b.set_custom_masks(narrow)
    out = b.blend(imgs)
    assert not out[:, :5].any() and out[:, 5:].any()
    b.set_custom_masks(None)
    assert not b.full_mask and np.array_equal(b.blend(imgs), ref)
    full = np.full_like(cov, 255)
    bf = O.Blender(full, seams, levels)
    assert bf.full_mask
    bf.set_custom_masks(seams)
    assert not bf.full_mask
    bf.set_custom_masks(None)
    assert bf.full_mask
