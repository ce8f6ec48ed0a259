"""The map-free remap of the low-memory path (GPU).

With ps_render_set_map_free the render keeps no maps: the remap computes each
pixel's source coordinate in fp32 (the reference's dstToSrc,
source/CudaAccel/CudaReproject.cu:81-264, does it in double), with the
coverage of the FP64 geometry.  Bar: level 0 within +-1 per channel of the
double-precision bilinear through the exact maps, with the histogram of the
differences printed; the rest of the render is the same code, so the output
stays close to the exact render.  The map path's level 0 is exact.
"""
import json

import numpy as np
import pytest

import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S

from _util import diff_histogram

pytestmark = pytest.mark.gpu

RIGS = [("c2", 4), ("c5", 8), ("c3a", 8), ("c1", 4), ("ricoh", 4)]


def _render(cfg, map_free, frames, luts):
    import torch
    r = P.CudaPanoramaRender2()
    r.set_map_free(map_free)
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    assert r.map_free == map_free
    W, H = cfg.dst_size
    out = np.zeros((H, W, 4), np.uint8)
    r.render(frames, out, luts, check=True)
    torch.cuda.synchronize()
    return r, out


@pytest.mark.parametrize("name,factor", RIGS)
def test_map_free_level0_within_one(cuda, oracle_lib, name, factor):
    cfg = S.scaled_rig(S.rig(name), factor)
    frames = S.FrameSource(cfg).frame(4)
    luts = S.luts(cfg)
    exact, out_exact = _render(cfg, False, frames, luts)
    free, out_free = _render(cfg, True, frames, luts)
    hist = {}
    for i in range(cfg.num_cams):
        xm, ym, mk = O.reproject_map(cfg.cams[i], cfg.src_size, cfg.dst_size, threads=8)
        ref = O.reproject_16s(frames[i], xm, ym, luts[i])[..., :3].astype(np.int16)
        assert np.array_equal(exact.level0(i)[..., :3], ref), "map path level 0 not exact"
        got = free.level0(i)[..., :3].astype(np.int16)
        for k, v in diff_histogram(got[mk > 0], ref[mk > 0]).items():
            hist[k] = hist.get(k, 0) + v
        assert not got[mk == 0].any()
    out_hist = diff_histogram(out_free[..., :3], out_exact[..., :3])
    print(f"\n{name}/{factor} level0 {json.dumps(hist)} output {json.dumps(out_hist)}")
    assert set(hist) <= {-1, 0, 1}, hist
    assert hist.get(0, 0) >= 0.9 * sum(hist.values()), hist
    assert max(abs(k) for k in out_hist) <= 3, out_hist


def test_map_free_memory_and_fallback(cuda):
    cfg = S.scaled_rig(S.rig("c2"), 2)
    est_maps = P.CudaPanoramaRender2.estimate_memory(cfg.cams, cfg.levels, cfg.src_size, cfg.dst_size, 1)
    r = P.CudaPanoramaRender2()
    r.set_map_free(True)
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    free_bytes = r.resident_bytes
    with pytest.raises(P.PsError) as e:
        r.maps(0, cfg.dst_size)
    assert e.value.code == L.PS_EINVAL
    m = P.CudaPanoramaRender2()
    m.set_frames_in_flight(1)
    m.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    # the same state but the maps: 8 bytes per covered pixel against 4 bits per pixel of every covered tile
    r1 = P.CudaPanoramaRender2()
    r1.set_frames_in_flight(1)
    r1.set_map_free(True)
    r1.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    assert r1.resident_bytes < m.resident_bytes
    assert free_bytes > r1.resident_bytes  # eight frames in flight against one
    # a budget that one frame in flight with maps does not fit: map-free by itself
    auto = P.CudaPanoramaRender2()
    auto.set_memory_budget(est_maps - 1)
    auto.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    assert auto.frames_in_flight == 1 and auto.map_free and auto.low_memory
