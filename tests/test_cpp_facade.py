"""The header-only C++ facade compiles against the C ABI and behaves like the
reference class (bool returns, lastError, lenient LUT handling)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def demo(built_lib, tmp_path_factory):
    out = str(tmp_path_factory.mktemp("facade") / "facade_demo")
    lib_dir = os.path.join(ROOT, "panostitcher_gb300")
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "cpp", "facade_demo.cpp"), "-o", out, "-L", lib_dir, "-lpanostitch",
           "-L", "/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{lib_dir}", "-Wl,-rpath,/usr/local/cuda/lib64"]
    subprocess.run(cmd, check=True)
    return out


def test_facade_argument_checks(demo):
    r = subprocess.run([demo, "check"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "facade check ok" in r.stdout


@pytest.mark.gpu
def test_facade_render(demo, cuda):
    r = subprocess.run([demo, "render"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert "skip correction" in r.stderr
    assert "facade render ok" in r.stdout
