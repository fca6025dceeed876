"""The reference's own Python binding (bindings/python/src/cybermesh/__init__.py),
unmodified, loaded on this library through CMG_C_LIB, on the CPU: it binds all 41
symbols at import, builds PLCs through the C ABI, and gets the reference's
validation errors back. No GPU call is made. Skipped where the reference source tree
(CMG_REFERENCE_ROOT) is not present."""
import os
import subprocess
import sys

import pytest

PROBE = r"""
import cybermesh as cm
plc = cm.PLC()
plc.add_points([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])
for f in ([0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]):
    plc.add_facet(f)
print("backend", cm._BACKEND)
try:
    cm.voxelize(plc, resolution=0)
except RuntimeError as e:
    print("error", e)
try:
    cm.voxelize(cm.PLC(), resolution=8)
except RuntimeError as e:
    print("error", e)
"""


def test_reference_binding_binds_this_library():
    root = os.environ.get("CMG_REFERENCE_ROOT")
    src = os.path.join(root or "", "bindings", "python", "src")
    if not root or not os.path.exists(os.path.join(src, "cybermesh", "__init__.py")):
        pytest.skip("the reference source tree (CMG_REFERENCE_ROOT) is not present")
    from cybermeshgenerator_gb300 import build
    lib = build.build()
    env = dict(os.environ, CMG_C_LIB=lib, PYTHONPATH=src)
    r = subprocess.run([sys.executable, "-c", PROBE], env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert "backend ctypes" in lines
    assert "error resolution must be >= 1" in lines
    assert "error voxelize: PLC has no points" in lines
