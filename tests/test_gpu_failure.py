"""The failure path of the bounded kernel waits (GPU), without a GPU fault.

Every wait of the blend kernel's bulk-copy ring is bounded; one that runs out
sets a status bit on every frame of the launch and the kernel carries on.
The test hook ps_render_set_wait_probe makes each blend launch wait on a
barrier that nothing completes, for a short, fixed number of polls, so the
wait runs out by construction.  The caller must then see PS_ETIMEOUT from
ps_render_check, and the render must stay usable: with the probe off, the
next frames are bit-exact again and the check is clean.
"""
import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S

from _util import Prepared, diff_histogram

pytestmark = pytest.mark.gpu

POLLS = 1000  # a few milliseconds at most per CTA


@pytest.fixture(scope="module")
def prepared(cuda, oracle_lib):
    return Prepared(S.scaled_rig(S.rig("c2"), 4))  # 1024x512: level 0 runs in k_blend


def test_wait_probe_reports_timeout_and_render_recovers(prepared):
    p = prepared
    frames = p.frames.frame(0)
    ref = p.oracle_render(frames, p.luts)[..., :3]
    assert p.r.check_status()  # nothing pending
    p.r.set_wait_probe(POLLS)
    p.product_render(frames, p.luts)
    assert not p.r.check_status(check=False)
    assert "bounded wait" in p.r.last_error
    assert p.r.check_status()  # read and cleared
    p.r.set_wait_probe(0)
    for _ in range(2):
        out = p.product_render(frames, p.luts)[..., :3]
        assert np.array_equal(out, ref), diff_histogram(out, ref)
    assert p.r.check_status()


def test_wait_probe_on_the_blender(cuda, oracle_lib):
    import torch
    import oracle as O
    rng = np.random.default_rng(11)
    n, W, H = 3, 256, 128
    cov = np.zeros((n, H, W), np.uint8)
    for i in range(n):
        cov[i][:, (i * W // n + np.arange(W // 2)) % W] = 255
    best = np.where(cov > 0, rng.random((n, H, W)), -1).argmax(0)
    seams = np.stack([((best == i) & (cov.max(0) > 0)).astype(np.uint8) * 255 for i in range(n)])
    imgs = rng.integers(0, 256, (n, H, W, 4)).astype(np.int16)
    imgs[..., 3] = 0
    imgs[cov == 0] = 0
    ref = O.Blender(cov, seams, 6).blend(list(imgs))[..., :3]
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(seams), 6)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in imgs]
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    b.set_wait_probe(POLLS)
    b.blend(dev, out)
    assert b.check_status() == L.PS_ETIMEOUT
    assert b.check_status() == L.PS_OK
    b.set_wait_probe(0)
    b.blend(dev, out)
    torch.cuda.synchronize()
    assert b.check_status() == L.PS_OK
    assert np.array_equal(out.cpu().numpy()[..., :3], ref)


def test_wait_probe_argument_checks(cuda):
    r = P.CudaPanoramaRender2()
    with pytest.raises(P.PsError) as e:
        r.set_wait_probe(10)  # not prepared
    assert e.value.code == L.PS_ESTATE
    cfg = S.scaled_rig(S.rig("c1"), 8)
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    with pytest.raises(P.PsError) as e:
        r.set_wait_probe(-1)
    assert e.value.code == L.PS_EINVAL
