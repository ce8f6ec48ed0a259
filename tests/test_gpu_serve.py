"""Serving loop (GPU): admission by budget, continuous batching, and each
stream's output identical alone and in the mix."""
import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S
from panostitcher_gb300.serve import StitchServer

pytestmark = pytest.mark.gpu


def _cfgs():
    return [S.scaled_rig(S.rig("c1"), 8), S.scaled_rig(S.rig("c2"), 8), S.scaled_rig(S.rig("c3c"), 8)]


def test_serve_mix_equals_alone(cuda):
    cfgs = _cfgs()
    srv = StitchServer(budget_bytes=8 << 30, max_batch=3)
    ids = [srv.admit(c.cams, c.levels, c.src_size, c.dst_size) for c in cfgs]
    assert all(i is not None for i in ids)
    assert srv.resident_bytes > 0
    # 5 frames per stream; bursts make several frames wait while a tick runs
    rng = np.random.default_rng(11)
    events = []
    for s, c in enumerate(cfgs):
        t = 0.0
        for k in range(5):
            events.append((t, s, k))
            t += float(rng.choice([0.0, 0.0005, 0.004]))
    events.sort()
    sources = {(s, k): S.FrameSource(cfgs[s]).frame(k + 10 * s) for s in range(3) for k in range(5)}
    luts = [S.luts(c) for c in cfgs]
    dsts = [np.zeros((cfgs[s].dst_size[1], cfgs[s].dst_size[0], 4), np.uint8) for (_, s, _) in events]
    lat, wall = srv.run_trace([ids[s] for (_, s, _) in events], [t for (t, _, _) in events],
                              [sources[(s, k)] for (_, s, k) in events], [luts[s] for (_, s, _) in events], dsts)
    assert (lat > 0).all() and wall > 0
    # the same frames rendered alone by their own render
    for c, cfg in enumerate(cfgs):
        r = P.CudaPanoramaRender2()
        r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
        for e, (t, s, k) in enumerate(events):
            if s != c:
                continue
            alone = np.zeros_like(dsts[e])
            r.render(sources[(s, k)], alone, luts[s], check=True)
            cuda.cuda.synchronize()
            assert np.array_equal(alone, dsts[e]), (s, k)
    srv.close()


def test_serve_admission_by_budget(cuda):
    cfg = _cfgs()[1]
    srv = StitchServer(budget_bytes=1 << 20, max_batch=2)   # 1 MiB: nothing fits
    assert srv.admit(cfg.cams, cfg.levels, cfg.src_size, cfg.dst_size) is None
    assert srv.resident_bytes == 0
    srv.close()
    srv = StitchServer(budget_bytes=8 << 30, max_batch=2)
    a = srv.admit(cfg.cams, cfg.levels, cfg.src_size, cfg.dst_size)
    assert a is not None
    used = srv.resident_bytes
    srv.remove(a)
    assert srv.resident_bytes == 0 and used > 0
    srv.close()


def test_serve_rejects_bad_traces(cuda):
    cfg = _cfgs()[0]
    srv = StitchServer(budget_bytes=8 << 30, max_batch=2)
    a = srv.admit(cfg.cams, cfg.levels, cfg.src_size, cfg.dst_size)
    fr = S.FrameSource(cfg).frame(0)
    with pytest.raises(P.PsError):
        srv.run_trace([a, a], [0.01, 0.0], [fr, fr])            # unsorted arrivals
    with pytest.raises(P.PsError):
        srv.run_trace([a + 7], [0.0], [fr])                     # unknown stream
    bad = [np.zeros((4, 4, 4), np.uint8)] * cfg.num_cams
    with pytest.raises(P.PsError):
        srv.run_trace([a], [0.0], [bad])                        # wrong frame size
    srv.close()
