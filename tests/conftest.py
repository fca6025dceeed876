"""Shared fixtures. Tests marked `gpu` need a CUDA device and the built library;
everything else runs on the CPU (the oracle, the host logic, the C ABI surface)."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libcmg_c.so")


@pytest.fixture(scope="session")
def orc():
    import oracle as O
    O.build()
    return O.Oracle()


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def load(name):
        if name not in cache:
            with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
                cache[name] = {k: z[k] for k in z.files}
        return cache[name]
    return load


@pytest.fixture(scope="session")
def cm():
    """The product package with its library built (GPU tests only)."""
    from cybermeshgenerator_gb300 import build
    build.build()
    import cybermeshgenerator_gb300 as cmg
    return cmg


def unpack_occ(g):
    n = int(np.prod(g["dims"]))
    return np.unpackbits(g["occ_bits"])[:n]
