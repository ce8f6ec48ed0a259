"""Regenerates the golden fixtures of tests/golden/ from the reference's own code.

The reference ships no golden vectors, so these fixtures are written by the
reference itself: its geometry and CPU remap (source/Warp/Remap.cpp,
ZReproject.cpp), its integer pyramid kernels chained as
CudaTilingMultibandBlendFast::prepare/blend chains them
(source/CudaAccel/CudaPyramid2.cu, CudaMultibandBlend.cpp:549-642,785-823)
and its YUV conversions (source/CudaAccel/ImageProc.cu), compiled unchanged
into oracle/_ref/ by `make -C oracle ref` (oracle/ref.py).  It therefore runs
only where the reference tree is present.

Two inputs are not the reference's: the nearest-optical-axis seam masks
(the benchmark's seam rule; the oracle computes them) and the seeded
frames, LUTs and random masks.  Everything else is the reference's output:
  - cov, xmaps, ymaps: getReprojectMapAndMask, maps cast to float as
    getReprojectMap32FAndMask does;
  - level0: reprojectParallelTo16S of the LUT'd source through those maps
    (the reference reads one pixel past the row end where floor(x) = W - 1;
    `quirk` marks those pixels);
  - out, coll, norm1, alpha1, weight1: the blend, its collapsed pyramid
    (every level), the normalised level 1 and the level-1 alpha and weight
    pyramids;
  - cpu_out: the reference's CPU blend, TilingMultibandBlendFast
    (source/Blend/MultiBandBlend.cpp:906-1031 with Pyramid.cpp), of the same
    level-0 images and masks;
  - yuv_*: cvtBGR32ToYUV420P / cvtBGR32ToNV12 and the inverse conversions.

  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from oracle import ref as R  # noqa: E402
from panostitcher_gb300 import synth as S  # noqa: E402


def apply_luts(frame, lut):
    out = frame.copy()
    for c in range(3):
        out[..., c] = lut[c][frame[..., c]]
    return out


def rig_case(name, factor, frame):
    cfg = S.scaled_rig(S.rig(name), factor)
    sw = cfg.src_size[0]
    maps, covs = [], []
    for c in cfg.cams:
        m64, k = R.reproject_map(c, cfg.src_size, cfg.dst_size)
        maps.append((m64[..., 0].astype(np.float32), m64[..., 1].astype(np.float32)))
        covs.append(k)
    cov = np.stack(covs)
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    levels = O.num_levels(cfg.dst_size[0], cfg.dst_size[1], cfg.levels)
    frames = S.FrameSource(cfg).frame(frame)
    luts = S.luts(cfg)
    level0, quirk = [], []
    for i in range(cfg.num_cams):
        xm, ym = maps[i]
        m64 = np.stack([xm.astype(np.float64), ym.astype(np.float64)], -1)
        level0.append(R.reproject_16s(apply_luts(frames[i], luts[i]), m64))
        quirk.append((cov[i] > 0) & (np.floor(xm) == sw - 1))
    out, pyr = R.mb_blend(cov, seams, level0, levels, pyramids=True)
    cpu_out, _ = R.cpu_mb_blend(cov, seams, level0, cfg.levels)
    n = cfg.num_cams
    coll = np.concatenate([c.reshape(-1, 4) for c in pyr["coll"]])
    return dict(source=np.array("reference"), params=json.dumps(cfg.cams), src_size=np.array(cfg.src_size),
                dst_size=np.array(cfg.dst_size), levels=np.array(cfg.levels), num_levels=np.array(levels),
                frames=np.stack(frames), luts=luts, xmaps=np.stack([m[0] for m in maps]),
                ymaps=np.stack([m[1] for m in maps]), cov=cov, seams=seams, level0=np.stack(level0),
                quirk=np.stack(quirk), out=out, cpu_out=cpu_out, coll=coll, norm1=pyr["norm"][1],
                alpha1=np.stack([pyr["alpha"][i][1] for i in range(n)]),
                weight1=np.stack([pyr["weight"][i][1] for i in range(n)]))


def partition_case(W, H, n, levels, seed):
    rng = np.random.default_rng(seed)
    cov = np.zeros((n, H, W), np.uint8)
    for i in range(n):
        y0, y1 = sorted(rng.integers(0, H + 1, 2))
        x0 = rng.integers(0, W)
        cols = (x0 + np.arange(rng.integers(1, W + 1))) % W
        cov[i][max(0, y0 - 1):max(y1, y0 + 1)][:, cols] = 255
    best = np.where(cov > 0, rng.random((n, H, W)), -1).argmax(0)
    covered = cov.max(0) > 0
    seams = np.stack([((best == i) & covered).astype(np.uint8) * 255 for i in range(n)])
    imgs = rng.integers(0, 256, (n, H, W, 4)).astype(np.int16)
    imgs[..., 3] = 0
    imgs[cov == 0] = 0
    nl = O.num_levels(W, H, levels)
    out = R.mb_blend(cov, seams, list(imgs), nl)
    cpu_out, _ = R.cpu_mb_blend(cov, seams, list(imgs), levels)
    return dict(source=np.array("reference"), cov=cov, seams=seams, level0=imgs, levels=np.array(levels),
                out=out, cpu_out=cpu_out, num_levels=np.array(nl))


def yuv_case(W, H, seed):
    rng = np.random.default_rng(seed)
    bgr = rng.integers(0, 256, (H, W, 4), dtype=np.uint8)
    y, u, v = R.bgr32_to_yuv(bgr, R.FMT_YUV420P)
    ny, nuv = R.bgr32_to_yuv(bgr, R.FMT_NV12)
    py = rng.integers(0, 256, (H, W), dtype=np.uint8)
    pu = rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8)
    pv = rng.integers(0, 256, (H // 2, W // 2), dtype=np.uint8)
    puv = rng.integers(0, 256, (H // 2, W), dtype=np.uint8)
    return dict(source=np.array("reference"), bgr=bgr, y420=y, u420=u, v420=v, y12=ny, uv12=nuv,
                in_y=py, in_u=pu, in_v=pv, in_uv=puv,
                bgr_from_420=R.yuv_to_bgr32([py, pu, pv], R.FMT_YUV420P),
                bgr_from_12=R.yuv_to_bgr32([py, puv], R.FMT_NV12))


def main():
    if not R.available():
        raise SystemExit("the reference build (make -C oracle ref) needs the reference tree")
    cases = {
        "rig_c1_16": rig_case("c1", 16, 0),
        "rig_c2_32": rig_case("c2", 32, 1),
        "rig_ricoh_16": rig_case("ricoh", 16, 2),
        "part_33x17": partition_case(33, 17, 3, 5, 7),
        "part_130x67": partition_case(130, 67, 4, 8, 8),
        "yuv_66x34": yuv_case(66, 34, 9),
    }
    for name, d in cases.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: getattr(v, "shape", None) for k, v in d.items()})


if __name__ == "__main__":
    main()
