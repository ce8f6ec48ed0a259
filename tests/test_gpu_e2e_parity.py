"""End-to-end parity from camera parameters at full size (GPU).

The other parity tests give the oracle the product's own maps, coverage and
seams, which isolates the per-frame kernels.  Here nothing is shared: the
oracle derives its geometry from the camera parameters (the restatement of
Remap / getReprojectMapAndMask that tests/test_ref_pin.py pins bit for bit
to the reference's own Remap.cpp and ZReproject.cpp) and its nearest-axis
seams, then renders; the product prepares from the same parameters with its
FP64 device geometry and renders the same frames.  The report gives, per
rig, the map values whose float bits differ, the coverage and seam pixels
that differ, and the histogram of output differences per channel.

Bar: bit for bit.  The product's FP64 device geometry gives the oracle's
(and so the reference's) float maps, coverage and seams exactly on every
benchmark rig, and the output is then bit-exact.  The device's and the C
library's transcendental functions are not both correctly rounded, so a map
value could in principle round to the other float; the test therefore
reports each count before it asserts, and a differing output value must in
any case lie within the pyramid's reach of a geometry difference.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import diff_histogram

pytestmark = pytest.mark.gpu

RIGS = ["c1", "c2", "c3a", "c3c", "c3d", "c5", "ricoh"]


def reach(L: int) -> int:
    """Canvas distance over which a level-0 change can move the collapsed output: the 5-tap pyrDown
    and pyrUp footprints at every level up to L."""
    return 3 * (1 << L) + 4


def dilate(mask: np.ndarray, r: int) -> np.ndarray:
    """Chebyshev dilation by r, wrapping horizontally (the canvas is a 360-degree panorama)."""
    from scipy.ndimage import maximum_filter
    if not mask.any():
        return mask
    return maximum_filter(mask.astype(np.uint8), size=2 * r + 1, mode=("nearest", "wrap")) > 0


def geometry_report(cfg, r, threads):
    W, H = cfg.dst_size
    maps = [O.reproject_map(c, cfg.src_size, cfg.dst_size, threads=threads) for c in cfg.cams]
    cov = np.stack([m[2] for m in maps])
    seams = O.nearest_axis_seams(cfg.cams, cfg.src_size, cfg.dst_size, cov, threads=threads)
    pcov = np.stack([r.coverage(i, cfg.dst_size) for i in range(cfg.num_cams)])
    pseams = np.stack([r.seam(i, cfg.dst_size) for i in range(cfg.num_cams)])
    geo_diff = np.zeros((H, W), bool)
    map_diff = 0
    for i in range(cfg.num_cams):
        px, py = r.maps(i, cfg.dst_size)
        both = (cov[i] > 0) & (pcov[i] > 0)
        d = both & ((px.view(np.uint32) != maps[i][0].view(np.uint32)) |
                    (py.view(np.uint32) != maps[i][1].view(np.uint32)))
        map_diff += int(d.sum())
        geo_diff |= d | ((cov[i] > 0) != (pcov[i] > 0)) | ((seams[i] > 0) != (pseams[i] > 0))
    rep = {"map_values_differing": map_diff,
           "coverage_px_differing": int(((cov > 0) != (pcov > 0)).sum()),
           "seam_px_differing": int(((seams > 0) != (pseams > 0)).sum())}
    return maps, cov, seams, geo_diff, rep


@pytest.mark.parametrize("name", RIGS)
def test_end_to_end_from_camera_parameters(cuda, oracle_lib, name):
    threads = os.cpu_count() or 4
    cfg = S.rig(name)
    W, H = cfg.dst_size
    r = P.CudaPanoramaRender2()
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    maps, cov, seams, geo_diff, rep = geometry_report(cfg, r, threads)
    frames = S.FrameSource(cfg).frame(5)
    luts = S.luts(cfg)
    ob = O.Blender(cov, seams, cfg.levels)
    ref = ob.render(frames, luts, [m[0] for m in maps], [m[1] for m in maps], threads)[..., :3]
    got = np.zeros((H, W, 4), np.uint8)
    r.render(frames, got, luts, check=True)
    import torch
    torch.cuda.synchronize()
    got = got[..., :3]
    rep["output_delta_histogram"] = diff_histogram(got, ref)
    rep["levels"] = ob.levels
    print(f"\n{name} {json.dumps(rep)}")
    bad = (got != ref).any(-1)
    assert not (bad & ~dilate(geo_diff, reach(ob.levels))).any(), rep
    assert rep["map_values_differing"] == 0, rep
    assert rep["coverage_px_differing"] == 0 and rep["seam_px_differing"] == 0, rep
    assert not bad.any(), rep
