"""Distinct renders used from different threads at once (GPU).  The C ABI
allows it; ctypes releases the GIL during the calls, so the renders' host
work, launches and the library's shared launch facts and caches are
exercised concurrently.  Every frame must still equal the oracle's.

A render records its launch graph with stream capture on its first frames
and throughout autotuning; CUDA forbids synchronising the whole device while
any stream captures, so each thread waits on its own stream only."""
import threading

import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu


def test_distinct_renders_on_threads(cuda, oracle_lib):
    torch = cuda
    cfgs = [S.scaled_rig(S.rig("c1"), 8), S.scaled_rig(S.rig("c2"), 8), S.scaled_rig(S.rig("c3c"), 8),
            S.scaled_rig(S.rig("ricoh"), 4)]
    preps = [Prepared(c) for c in cfgs]
    frames = [[p.frames.frame(k) for k in range(4)] for p in preps]
    refs = [[p.oracle_render(f, p.luts)[..., :3] for f in fs] for p, fs in zip(preps, frames)]
    outs = [[None] * 4 for _ in preps]
    errors = []
    start = threading.Barrier(len(preps))

    streams = [torch.cuda.Stream() for _ in preps]

    def work(t):
        try:
            p = preps[t]
            W, H = p.cfg.dst_size
            start.wait()
            if t == 1:  # one thread tunes while the others render
                p.r.autotune(frames_per_trial=3, in_flight=2, force=True)
            for k in range(4):
                o = np.zeros((H, W, 4), np.uint8)
                assert p.r.render(frames[t][k], o, p.luts, stream=streams[t], check=True)
                outs[t][k] = o
            streams[t].synchronize()  # this thread's stream only
        except Exception as e:  # reported on the main thread
            errors.append((t, repr(e)))

    threads = [threading.Thread(target=work, args=(t,)) for t in range(len(preps))]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=300)
    assert not any(th.is_alive() for th in threads)
    assert not errors, errors
    for t in range(len(preps)):
        for k in range(4):
            got = outs[t][k][..., :3]
            assert np.array_equal(got, refs[t][k]), (t, k, diff_histogram(got, refs[t][k]))
