"""The bounds-checked build (GPU).

libpanostitch_checked.so is the library compiled with every global access
of the stitch kernels checked against the extent of its buffer: an access
outside is not made and is counted (ps_debug_bounds_violations).  Here it
runs every kind of launch in a fresh process (PS_LIBRARY=checked) -- the
remap (BGR32 and BGR24 sources, resident maps and map-free), every pyrDown
and blend level in k_pyrdown / k_blend / k_blend_small / k_tail with whole
and half tiles, border tiles of odd sizes, the encoder and decoder handoffs,
the linear-blend mode, a batch of two rigs and the streaming blender -- and
requires zero refused accesses and the oracle's bytes.  Nothing is made to
go out of bounds on purpose.

The checked build keeps one near-tie pixel per warp in the remap's own list,
so the launch's list and k_remap_fix run on every frame; a second run sets
that list's room to zero (PS_CHECKED_TIE_LIST_PER_TILE=0), which sends every
frame with a listed pixel down k_remap_fix's overflow path (every pixel
recomputed exactly).
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + "/tests")
import torch
import oracle as O
import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S
from _util import Prepared
assert L.LIB_PATH.endswith("libpanostitch_checked.so"), L.LIB_PATH
assert L.lib().ps_debug_bounds_violations(1) == 0
torch.cuda.set_device(0)

def check(tag):
    v = L.lib().ps_debug_bounds_violations(1)
    assert v == 0, f"{tag}: {v} accesses refused"
    print("ok", tag, flush=True)

def same(a, b, tag):
    assert np.array_equal(a[..., :3], b[..., :3]), tag

shapes = [dict(), dict(tail_max_items=0, small_blend_max_items=128), dict(tail_half_tiles=0, tail_cluster=8)]
for name, f in (("c2", 4), ("c1", 4), ("ricoh", 4), ("c3c", 8)):
    p = Prepared(S.scaled_rig(S.rig(name), f))
    W, H = p.cfg.dst_size
    fr = p.frames.frame(1)
    ref = p.oracle_render(fr, p.luts)
    for sh in shapes:
        p.r.set_launch_shape(**{**P.CudaPanoramaRender2.SHAPE_DEFAULT, **sh})
        same(p.product_render(fr, p.luts), ref, name)
    bgr24 = [np.ascontiguousarray(x[..., :3]) for x in fr]
    same(p.product_render(bgr24, p.luts), ref, name + " bgr24")
    check(name)

# encoder and decoder handoffs
p = Prepared(S.scaled_rig(S.rig("c2"), 4))
W, H = p.cfg.dst_size
fr = p.frames.frame(2)
ref = p.oracle_render(fr, p.luts)
y = np.zeros((H, W), np.uint8); uv = np.zeros((H // 2, W), np.uint8)
p.r.render_yuv(fr, [y, uv], p.luts, P.PS_FMT_NV12, check=True)
torch.cuda.synchronize()
for a, b in zip((y, uv), O.bgr32_to_yuv(ref, O.FMT_NV12)):
    assert np.array_equal(a, b)
planes = [O.bgr32_to_yuv(x, O.FMT_NV12) for x in fr]
dst = np.zeros((H, W, 4), np.uint8)
p.r.render_planar(planes, dst, p.luts, src_fmt=P.PS_FMT_NV12, check=True)
torch.cuda.synchronize()
check("handoffs")

# a batch of two rigs
q = Prepared(S.scaled_rig(S.rig("c1"), 4))
outs = [torch.zeros((c.cfg.dst_size[1], c.cfg.dst_size[0], 4), dtype=torch.uint8, device="cuda") for c in (p, q)]
frs = [[torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in c.frames.frame(3)] for c in (p, q)]
P.render_batch([p.r, q.r], frs, outs, [p.luts, q.luts])
torch.cuda.synchronize()
for c, o, f in zip((p, q), outs, ((p.frames.frame(3)), (q.frames.frame(3)))):
    same(o.cpu().numpy(), c.oracle_render(f, c.luts), "batch")
check("batch")

# linear-blend mode and map-free remap
cfg = S.scaled_rig(S.rig("c2"), 4)
lin = P.CudaPanoramaRender2()
lin.prepare(cfg.cams, 0, 40, cfg.src_size, cfg.dst_size, check=True)
lin.render(S.FrameSource(cfg).frame(0), np.zeros((cfg.dst_size[1], cfg.dst_size[0], 4), np.uint8), S.luts(cfg),
           check=True)
mf = P.CudaPanoramaRender2()
mf.set_map_free(True)
mf.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
mf.render(S.FrameSource(cfg).frame(0), np.zeros((cfg.dst_size[1], cfg.dst_size[0], 4), np.uint8), S.luts(cfg),
          check=True)
torch.cuda.synchronize()
check("linear, map-free")

# blender on odd sizes (border tiles everywhere), whole and streamed
rng = np.random.default_rng(3)
for (Wb, Hb, n) in ((33, 17, 3), (130, 67, 4), (257, 129, 5)):
    cov = np.zeros((n, Hb, Wb), np.uint8)
    for i in range(n):
        cov[i][:, (i * Wb // n + np.arange(Wb // 2 + 1)) % Wb] = 255
    best = np.where(cov > 0, rng.random((n, Hb, Wb)), -1).argmax(0)
    seams = np.stack([((best == i) & (cov.max(0) > 0)).astype(np.uint8) * 255 for i in range(n)])
    imgs = rng.integers(0, 256, (n, Hb, Wb, 4)).astype(np.int16); imgs[..., 3] = 0; imgs[cov == 0] = 0
    ref = O.Blender(cov, seams, 8).blend(list(imgs))
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(cov), list(seams), 8)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in imgs]
    out = torch.zeros((Hb, Wb, 4), dtype=torch.uint8, device="cuda")
    b.blend(dev, out)
    torch.cuda.synchronize()
    same(out.cpu().numpy(), ref, f"blender {Wb}x{Hb}")
    b.begin()
    for i, d in enumerate(dev):
        b.tile(d, i)
    b.end(out)
    torch.cuda.synchronize()
    same(out.cpu().numpy(), ref, f"tiles {Wb}x{Hb}")
check("blender")
print("ALL OK", flush=True)
"""


def test_checked_build_refuses_nothing(cuda):
    env = dict(os.environ, PS_LIBRARY="checked")
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT))], env=env, capture_output=True,
                       text=True, timeout=900)
    sys.stdout.write(r.stdout[-3000:])
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stderr[-4000:]


OVERFLOW_SCRIPT = r"""
import sys
import numpy as np
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + "/tests")
import torch
import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S
from _util import Prepared
assert L.LIB_PATH.endswith("libpanostitch_checked.so"), L.LIB_PATH
assert L.lib().ps_debug_bounds_violations(1) == 0
torch.cuda.set_device(0)
for name, f in (("c2", 4), ("ricoh", 4), ("c3c", 8)):
    p = Prepared(S.scaled_rig(S.rig(name), f))
    for k in (1, 2):
        fr = p.frames.frame(k)
        assert np.array_equal(p.product_render(fr, p.luts)[..., :3], p.oracle_render(fr, p.luts)[..., :3]), name
    assert L.lib().ps_debug_bounds_violations(1) == 0, name
print("ALL OK", flush=True)
"""


def test_checked_build_tie_list_overflow(cuda):
    env = dict(os.environ, PS_LIBRARY="checked", PS_CHECKED_TIE_LIST_PER_TILE="0")
    r = subprocess.run([sys.executable, "-c", OVERFLOW_SCRIPT.replace("ROOT", repr(ROOT))], env=env,
                       capture_output=True, text=True, timeout=600)
    sys.stdout.write(r.stdout[-3000:])
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stderr[-4000:]
