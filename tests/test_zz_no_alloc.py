"""The allocation-free seam entry point (GPU).

ps_nearest_axis_seams_no_alloc serves callers that cannot call cudaMalloc;
its scratch is a fixed device array inside the library.  Its masks must equal
the ones the existing path (ps_render_prepare, read back with
ps_render_export) derives, on two calls in a row (the second call reuses the
array the first one left behind).  This file is collected last so a run that
stops at the first failure has run everything else first; it also passes
alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import panostitcher_gb300 as P
from panostitcher_gb300 import _lib as L
from panostitcher_gb300 import synth as S

pytestmark = pytest.mark.gpu


def _call(cfg, out):
    arr = (L.PhotoParam * cfg.num_cams)(*[L.PhotoParam.from_dict(p) for p in cfg.cams])
    return L.lib().ps_nearest_axis_seams_no_alloc(arr, cfg.num_cams, cfg.src_size[0], cfg.src_size[1],
                                                  cfg.dst_size[0], cfg.dst_size[1], out.data_ptr(), None)


@pytest.mark.parametrize("name,factor", [("c2", 8), ("c1", 4)])
def test_no_alloc_seams_equal_prepare(cuda, name, factor):
    torch = cuda
    cfg = S.scaled_rig(S.rig(name), factor)
    r = P.CudaPanoramaRender2()
    r.prepare(cfg.cams, 1, cfg.levels, cfg.src_size, cfg.dst_size, check=True)
    ref = np.stack([r.seam(i, cfg.dst_size) for i in range(cfg.num_cams)])
    W, H = cfg.dst_size
    outs = [torch.full((cfg.num_cams, H, W), 7, dtype=torch.uint8, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    for call, out in enumerate(outs):
        # the first call may load the library's device code (and its array);
        # the second must leave the device's free memory as it found it
        free_before = torch.cuda.mem_get_info()[0]
        L.check(_call(cfg, out))
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before, "the second call changed free device memory"
        assert np.array_equal(out.cpu().numpy(), ref), f"call {call}"


def test_no_alloc_rejects_oversize(cuda):
    torch = cuda
    cfg = S.rig("c3d")                   # 8 cameras x 7680 x 3840: far beyond the 16 MiB scratch
    out = torch.empty(16, dtype=torch.uint8, device="cuda")
    st = _call(cfg, out)
    assert st == L.PS_EINVAL
    assert "scratch" in L.lib().ps_last_error().decode()


def test_no_alloc_rejects_tall_canvas(cuda):
    torch = cuda
    cfg = S.scaled_rig(S.rig("c1"), 8)
    cfg.dst_size = (64, 70000)            # 4.5 MB of coverage fits the scratch; 70000 rows do not fit a grid
    out = torch.empty(16, dtype=torch.uint8, device="cuda")
    st = _call(cfg, out)
    assert st == L.PS_EINVAL
    assert "65535" in L.lib().ps_last_error().decode()
