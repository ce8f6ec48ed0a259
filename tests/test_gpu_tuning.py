"""Launch shapes and the autotuner (GPU).

Every launch shape must stitch the same bytes: the tail split only moves
pyramid levels between kernels that run the same per-tile code, the tail's
half tiles change which threads own which pixels, and grid widths change
which CTA takes which tile.  Each shape's frames are compared with the
oracle, as are the frames after autotuning and a batch of rigs whose shapes
differ.
"""
import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu

SHAPES = [
    {},
    {"tail_max_items": 0},                     # no tail: every level in the per-level kernels
    {"tail_max_items": 4},
    {"tail_max_items": 1 << 20},               # the tail runs every pyramid level
    {"tail_half_tiles": 0},                    # whole tiles, 2x2 blocks, in the tail
    {"tail_cluster": 8},
    {"tail_cluster": 16},
    {"ctas_per_sm": (1, 1, 1)},
    {"ctas_per_sm": (2, 1, 3)},
    {"tail_max_items": 64, "tail_half_tiles": 0, "tail_cluster": 8, "ctas_per_sm": (3, 2, 1)},
    {"small_blend_max_items": 1 << 20},        # every blend level above 0 below the tail in half tiles
    {"small_blend_max_items": 64},
    {"tail_max_items": 0, "small_blend_max_items": 1 << 20},  # no tail: k_blend_small up to the top level
    {"remap_defer_ties": 0},                   # near-tie remap pixels recomputed inside k_remap
]


@pytest.fixture(scope="module", params=[("c2", 8), ("c1", 4), ("c3c", 8)], ids=lambda p: f"{p[0]}/{p[1]}")
def rig(request, cuda, oracle_lib):
    name, factor = request.param
    p = Prepared(S.scaled_rig(S.rig(name), factor))
    frames = [p.frames.frame(k) for k in (0, 1)]
    refs = [p.oracle_render(f, p.luts)[..., :3] for f in frames]
    return p, frames, refs


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: ",".join(f"{k}={v}" for k, v in s.items()) or "default")
def test_every_shape_stitches_the_same_bytes(rig, shape):
    p, frames, refs = rig
    p.r.set_launch_shape(**P.CudaPanoramaRender2.SHAPE_DEFAULT)
    p.r.set_launch_shape(**shape)
    got = p.r.launch_shape()
    for k, v in shape.items():
        assert got[k] == v
    for f, ref in zip(frames, refs):
        out = p.product_render(f, p.luts)[..., :3]
        assert np.array_equal(out, ref), diff_histogram(out, ref)
    p.r.set_launch_shape(**P.CudaPanoramaRender2.SHAPE_DEFAULT)


def test_autotune_keeps_the_output(rig):
    p, frames, refs = rig
    rep = p.r.autotune(frames_per_trial=4, force=True)
    assert rep["trials"] >= 2 and not rep["cached"]
    assert rep["ms_per_frame_default"] > 0 and 0 < rep["ms_per_frame_chosen"] <= rep["ms_per_frame_default"]
    assert p.r.launch_shape() == rep["shape"]
    # the tuner overwrote the render's slot-0 input staging; host frames go through it again
    for f, ref in zip(frames, refs):
        out = p.product_render(f, p.luts)[..., :3]
        assert np.array_equal(out, ref), diff_histogram(out, ref)
    again = p.r.autotune(frames_per_trial=4)
    assert again["cached"] and again["trials"] == 0 and again["shape"] == rep["shape"]
    p.r.set_launch_shape(**P.CudaPanoramaRender2.SHAPE_DEFAULT)


def test_autotune_one_stream_and_bad_arguments(cuda):
    cfg = S.scaled_rig(S.rig("c2"), 8)
    r = P.CudaPanoramaRender2()
    with pytest.raises(P.PsError):
        r.autotune()  # not prepared
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    rep = r.autotune(frames_per_trial=3, in_flight=1)
    assert rep["trials"] >= 2
    with pytest.raises(P.PsError):
        r.autotune(in_flight=9)  # more than the render's eight frames in flight
    with pytest.raises(P.PsError):
        r.autotune(frames_per_trial=-1)


def test_batch_of_rigs_with_different_shapes(cuda, oracle_lib):
    cfgs = [S.scaled_rig(S.rig("c1"), 8), S.scaled_rig(S.rig("c2"), 8), S.scaled_rig(S.rig("c3a"), 16)]
    ps = [Prepared(c) for c in cfgs]
    ps[0].r.set_launch_shape(tail_max_items=0, ctas_per_sm=(1, 2, 1))
    ps[1].r.set_launch_shape(tail_cluster=8, tail_half_tiles=0)
    ps[2].r.set_launch_shape(tail_max_items=1 << 20, ctas_per_sm=(2, 2, 2))
    ps[0].r.set_launch_shape(small_blend_max_items=1 << 20)  # one rig's levels in k_blend_small, the others not
    ps[2].r.set_launch_shape(remap_defer_ties=0)  # the launch still defers: the other rigs ask for it
    frames = [p.frames.frame(3) for p in ps]
    refs = [p.oracle_render(f, p.luts)[..., :3] for p, f in zip(ps, frames)]
    dsts = [np.zeros((c.dst_size[1], c.dst_size[0], 4), np.uint8) for c in cfgs]
    for _ in range(2):  # the second call replays the captured graph
        P.render_batch([p.r for p in ps], frames, dsts, [p.luts for p in ps])
        cuda.cuda.synchronize()
        for d, ref in zip(dsts, refs):
            assert np.array_equal(d[..., :3], ref), diff_histogram(d[..., :3], ref)
