"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle still reproduces every fixture bit for bit.
GPU: the product's blender and remap primitives reproduce them from the
stored level-0 images, maps and masks."""
import json
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RIGS = ["rig_c1_16", "rig_c2_32"]
PARTS = ["part_33x17", "part_130x67"]


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


@pytest.mark.parametrize("name", RIGS)
def test_oracle_reproduces_rig_fixture(oracle_lib, name):
    d = load(name)
    cams = json.loads(str(d["params"]))
    src, dst = tuple(d["src_size"]), tuple(d["dst_size"])
    for i, c in enumerate(cams):
        xm, ym, mk = O.reproject_map(c, src, dst)
        assert np.array_equal(mk, d["cov"][i])
        assert np.array_equal(xm, d["xmaps"][i]) and np.array_equal(ym, d["ymaps"][i])
    assert np.array_equal(O.nearest_axis_seams(cams, src, dst, d["cov"]), d["seams"])
    for i in range(len(cams)):
        l0 = O.reproject_16s(d["frames"][i], d["xmaps"][i], d["ymaps"][i], d["luts"][i])
        assert np.array_equal(l0, d["level0"][i])
    b = O.Blender(d["cov"], d["seams"], int(d["levels"]))
    out, norm, coll = b.blend(list(d["level0"]), pyramids=True)
    assert np.array_equal(out, d["out"])
    assert np.array_equal(coll[1], d["coll1"])
    for i in range(len(cams)):
        assert np.array_equal(b.alpha(i, 1), d["alpha1"][i])
        assert np.array_equal(b.weight(i, 1), d["weight1"][i])


@pytest.mark.parametrize("name", PARTS)
def test_oracle_reproduces_partition_fixture(oracle_lib, name):
    d = load(name)
    b = O.Blender(d["cov"], d["seams"], int(d["levels"]))
    assert b.levels == int(d["num_levels"])
    assert np.array_equal(b.blend(list(d["level0"])), d["out"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", RIGS + PARTS)
def test_product_blender_reproduces_fixture(cuda, name):
    import panostitcher_gb300 as P
    torch = cuda
    d = load(name)
    H, W = d["cov"].shape[1:]
    b = P.CudaTilingMultibandBlendFast()
    assert b.prepare(list(d["cov"]), list(d["seams"]), int(d["levels"])), b.last_error
    out = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    b.blend([torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in d["level0"]], out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy()[..., :3], d["out"][..., :3])


@pytest.mark.gpu
@pytest.mark.parametrize("name", RIGS)
def test_product_remap_reproduces_fixture(cuda, name):
    import panostitcher_gb300 as P
    torch = cuda
    d = load(name)
    H, W = d["cov"].shape[1:]
    for i in range(d["frames"].shape[0]):
        out = torch.empty((H, W, 4), dtype=torch.int16, device="cuda")
        P.reproject_to_16s(torch.from_numpy(np.ascontiguousarray(d["frames"][i])).cuda(),
                           torch.from_numpy(np.ascontiguousarray(d["xmaps"][i])).cuda(),
                           torch.from_numpy(np.ascontiguousarray(d["ymaps"][i])).cuda(), out,
                           torch.from_numpy(np.ascontiguousarray(d["luts"][i].reshape(-1))).cuda())
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), d["level0"][i])
