"""The C++ surface cmg::voxelize::voxelize (include/cmg/voxelize/voxelize.hpp) of
libcmg_c.so, exercised by a C++ program (tests/cpp/test_voxelize.cpp) compiled
against the headers and linked to the library:

* on the CPU: the reference's InvalidInput answers and messages (no GPU call), and,
  where the reference source tree is present (CMG_REFERENCE_ROOT), that a call
  compiled against the reference's own headers binds to the symbol this library
  exports (the drop-in is link-compatible);
* on the GPU: occupancy and float distance through the C++ call equal the
  reference's outputs on the golden fixtures (one output per mode).
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, unpack_occ

SRC = os.path.join(ROOT, "tests", "cpp", "test_voxelize.cpp")


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    from cybermeshgenerator_gb300 import build
    lib = build.build()
    exe = str(tmp_path_factory.mktemp("cpp") / "test_voxelize")
    cmd = ["g++", "-std=c++20", "-O1", "-I", os.path.join(ROOT, "include"), SRC, lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_validation_errors(prog):
    r = subprocess.run([prog, "validate"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr


def test_cpp_symbol_matches_reference_headers(tmp_path):
    root = os.environ.get("CMG_REFERENCE_ROOT")
    gen = os.path.join(ROOT, "oracle", "_ref", "gen")  # the reference's generated config header
    if not root or not os.path.exists(os.path.join(root, "include", "cmg", "voxelize")) \
            or not os.path.isdir(gen):
        pytest.skip("the reference source tree (CMG_REFERENCE_ROOT) and its harness build are not present")
    from cybermeshgenerator_gb300 import build
    lib = build.build()
    tu = tmp_path / "call.cpp"
    tu.write_text('#include "cmg/voxelize/voxelize.hpp"\n'
                  "auto call(const cmg::PLC& p) { return cmg::voxelize::voxelize(p); }\n")
    obj = str(tmp_path / "call.o")
    r = subprocess.run(["g++", "-std=c++20", "-c", "-I", os.path.join(root, "include"), "-I", gen,
                        str(tu), "-o", obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    und = subprocess.run(["nm", "-u", obj], capture_output=True, text=True).stdout
    want = [ln.split()[-1] for ln in und.splitlines() if "voxelize8voxelize" in ln]
    assert len(want) == 1
    exported = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    assert want[0] in exported.split()


CASES = ["cube4_r16p1", "brick312_r20p1", "icosphere_s3_r58p3", "shsphere64_r30p1", "cube4deg_r16p1"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cpp_voxelize_matches_reference(prog, golden, tmp_path, name):
    g = golden(name)
    pts = np.ascontiguousarray(g["points"], np.float64)
    tri = np.ascontiguousarray(g["triangles"], np.int32)
    with open(tmp_path / "in.bin", "wb") as f:
        f.write(np.int64(len(pts)).tobytes() + pts.tobytes() + np.int64(len(tri)).tobytes())
        for t in tri:
            f.write(np.int64(3).tobytes() + t.tobytes())
        f.write(np.int32(int(g["resolution"])).tobytes() + np.int32(int(g["pad"])).tobytes())
    r = subprocess.run([prog, "run", str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    raw = (tmp_path / "out.bin").read_bytes()
    dims = tuple(int(d) for d in np.frombuffer(raw[:12], np.int32))
    origin = np.frombuffer(raw[12:36], np.float64)
    spacing = float(np.frombuffer(raw[36:44], np.float64)[0])
    n = int(np.prod(dims))
    occ = np.frombuffer(raw[44:44 + n], np.uint8)
    sdf = np.frombuffer(raw[44 + n:44 + 5 * n], np.float32)
    assert dims == tuple(int(d) for d in g["dims"])
    assert np.array_equal(origin, g["origin"]) and spacing == float(g["spacing"])
    assert np.array_equal(occ, unpack_occ(g))
    assert hashlib.sha256(sdf.tobytes()).hexdigest() == str(g["sdf32_sha"])
