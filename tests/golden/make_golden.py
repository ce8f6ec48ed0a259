"""Regenerates the golden fixtures of tests/golden/ from the CPU oracle.

The reference ships no golden vectors and cannot be built here, so these
fixtures are the oracle's own answers on small seeded cases: they pin the
oracle against regressions (CPU tests) and give the GPU tests fixed inputs
and outputs that do not depend on the geometry code (level-0 images, maps
and masks are stored).

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
from panostitcher_gb300 import synth as S  # noqa: E402


def rig_case(name, factor, frame):
    cfg = S.scaled_rig(S.rig(name), factor)
    maps = [O.reproject_map(c, cfg.src_size, cfg.dst_size) for c in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov)
    b = O.Blender(cov, seams, cfg.levels)
    frames = S.FrameSource(cfg).frame(frame)
    luts = S.luts(cfg)
    level0 = np.stack([O.reproject_16s(frames[i], maps[i][0], maps[i][1], luts[i]) for i in range(cfg.num_cams)])
    out, norm, coll = b.blend(list(level0), pyramids=True)
    out2 = b.render(frames, luts, [m[0] for m in maps], [m[1] for m in maps])
    assert np.array_equal(out, out2)
    return dict(params=json.dumps(cfg.cams), src_size=np.array(cfg.src_size), dst_size=np.array(cfg.dst_size),
                levels=np.array(cfg.levels), frames=np.stack(frames), luts=luts,
                xmaps=np.stack([m[0] for m in maps]), ymaps=np.stack([m[1] for m in maps]), cov=cov, seams=seams,
                level0=level0, out=out, num_levels=np.array(b.levels),
                alpha1=np.stack([b.alpha(i, 1) for i in range(cfg.num_cams)]),
                weight1=np.stack([b.weight(i, 1) for i in range(cfg.num_cams)]),
                coll1=coll[1])


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
    b = O.Blender(cov, seams, levels)
    return dict(cov=cov, seams=seams, level0=imgs, levels=np.array(levels), out=b.blend(list(imgs)),
                num_levels=np.array(b.levels))


def main():
    cases = {
        "rig_c1_16": rig_case("c1", 16, 0),
        "rig_c2_32": rig_case("c2", 32, 1),
        "part_33x17": partition_case(33, 17, 3, 5, 7),
        "part_130x67": partition_case(130, 67, 4, 8, 8),
    }
    for name, d in cases.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: getattr(v, "shape", None) for k, v in d.items()})


if __name__ == "__main__":
    main()
