"""Build libcmg_c.so in-tree (CUDA kernels for sm_103a + the C ABI).

    python -m cybermeshgenerator_gb300.build [--jobs N]

Each .cu file is compiled by nvcc for sm_103a only, the C ABI by g++, in
parallel; objects go to _build/ at the repository root, the library next to
this file. Host code is compiled with -ffp-contract=off: make_grid must round as
the reference does on every host (aarch64 GCC would otherwise fuse a
multiply-add).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(HERE, "libcmg_c.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["scan.cu", "occupancy.cu", "sdf.cu", "sdf_sub.cu", "engine.cu", "peak.cu", "noalloc.cu", "predicates.cu", "adjoint.cu", "stl.cu", "detect.cu", "simplify.cu", "sizing.cu"]
# per-file flags: sizing.cu rounds every product and sum separately, as the reference does
CU_FLAGS = {"sizing.cu": ["-fmad=false"]}
CXX_SOURCES = ["cmg_c.cpp", "cmg_cpp.cpp"]
# per-file language standard: the C++ surface (cmg::voxelize::voxelize) is built as
# C++20, as the reference is, so cmg::expected has the same layout on both sides
CXX_STD = {"cmg_cpp.cpp": "-std=c++20"}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    inc = os.path.join(_cuda_home(nvcc), "include")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    for sub in ("cmg_c", os.path.join("cmg", "core"), os.path.join("cmg", "voxelize")):
        d = os.path.join(ROOT, "include", sub)
        headers += [os.path.join(d, f) for f in os.listdir(d)]
    steps, objs = [], []
    for src in CU_SOURCES:
        s, o = os.path.join(CSRC, src), os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            steps.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", *CU_FLAGS.get(src, []),
                          "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s, o = os.path.join(CSRC, src), os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            steps.append(["g++", "-O2", CXX_STD.get(src, "-std=c++17"), "-fPIC", "-ffp-contract=off",
                          "-fvisibility=default", "-I" + inc, "-I" + os.path.join(ROOT, "include"),
                          "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for log in ex.map(_run, steps):
            if verbose and log.strip():
                print(log)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    jobs = None
    if "--jobs" in sys.argv:
        jobs = int(sys.argv[sys.argv.index("--jobs") + 1])
    print(build(jobs, verbose="-v" in sys.argv))
