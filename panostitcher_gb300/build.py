"""Builds libpanostitch.so in-tree with nvcc for sm_103a (no CMake, no torch).

Each translation unit compiles in parallel into panostitcher_gb300/_build/,
then nvcc links the shared library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpanostitch.so")
# the bounds-checked build: the kernels' translation unit again with
# -DPS_CHECK_BOUNDS, linked with the same other objects
LIB_CHECKED = os.path.join(HERE, "libpanostitch_checked.so")
CHECKED_SRC = "csrc/ps_kernels.cu"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "csrc/ps_kernels.cu": [],
    "csrc/ps_prepare.cu": ["--fmad=false"],
    "csrc/ps_rig.cpp": [],
    "csrc/ps_capi.cpp": [],
    "csrc/ps_server.cpp": [],
    "csrc/ps_params.cpp": [],
    "csrc/ps_tune.cpp": [],
}
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    d = os.path.join(HERE, "csrc")
    hs = [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    """Builds libpanostitch.so and its bounds-checked twin libpanostitch_checked.so."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for src, extra in SOURCES.items():
        path = os.path.join(HERE, src)
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + hdrs):
            cmd = [cc] + COMMON + extra + (["-Xptxas", "-v"] if ptxas_info and src.endswith(".cu") else []) + \
                  ["-c", path, "-o", obj]
            jobs.append(cmd)
    checked_obj = os.path.join(BUILD, "ps_kernels_checked.cu.o")
    checked_path = os.path.join(HERE, CHECKED_SRC)
    checked_new = force or _stale(checked_obj, [checked_path] + hdrs)
    if checked_new:
        jobs.append([cc] + COMMON + SOURCES[CHECKED_SRC] + ["-DPS_CHECK_BOUNDS", "-c", checked_path, "-o", checked_obj])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0 or ptxas_info:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed on {cmd[-3]}")
    kernels_obj = os.path.join(BUILD, os.path.basename(CHECKED_SRC) + ".o")
    for lib, lib_objs in ((LIB, objs), (LIB_CHECKED, [checked_obj if o == kernels_obj else o for o in objs])):
        if not (force or jobs or not os.path.exists(lib)):
            continue
        cmd = [cc] + ARCH + ["-shared", "-o", lib] + lib_objs + ["-cudart", "static", "-Xlinker", "-z,defs"] + \
              ["-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
