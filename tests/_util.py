"""Shared helpers of the parity tests: prepare a rig in the product and the
same rig (same maps and masks) in the oracle."""
from __future__ import annotations

import numpy as np

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S


def diff_histogram(a: np.ndarray, b: np.ndarray) -> dict:
    d = a.astype(np.int32) - b.astype(np.int32)
    vals, counts = np.unique(d, return_counts=True)
    return {int(v): int(c) for v, c in zip(vals, counts)}


class Prepared:
    """A product render and the oracle blender built from its exported state."""

    def __init__(self, cfg: S.RigConfig, seams=None, graph: bool = True):
        self.cfg = cfg
        self.r = P.CudaPanoramaRender2()
        self.r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, seams=seams, check=True)
        self.r.set_graph(graph)
        n = cfg.num_cams
        self.maps = [self.r.maps(i, cfg.dst_size) for i in range(n)]
        self.cov = np.stack([self.r.coverage(i, cfg.dst_size) for i in range(n)])
        self.seams = np.stack([self.r.seam(i, cfg.dst_size) for i in range(n)])
        self.ob = O.Blender(self.cov, self.seams, cfg.levels)
        self.frames = S.FrameSource(cfg)
        self.luts = S.luts(cfg)

    def oracle_render(self, frames, luts=None, nthreads: int = 4) -> np.ndarray:
        return self.ob.render(frames, luts, [m[0] for m in self.maps], [m[1] for m in self.maps], nthreads)

    def product_render(self, frames, luts=None, channels_out: int = 4) -> np.ndarray:
        W, H = self.cfg.dst_size
        dst = np.zeros((H, W, channels_out), np.uint8)
        self.r.render(frames, dst, luts, check=True)
        import torch
        torch.cuda.synchronize()
        return dst
