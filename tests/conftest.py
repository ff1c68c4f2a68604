import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mini-fem_gb300")
for p in (PKG, os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 host)")
    config.addinivalue_line("markers", "slow: full-size cases")


def _ensure_built():
    so = os.path.join(PKG, "lib", "libminifem_gb300.so")
    sys.path.insert(0, PKG)
    import build as pkg_build  # mini-fem_gb300/build.py
    pkg_build.build()
    import pyoracle
    pyoracle.build_port()
    return so


_ensure_built()


@pytest.fixture(scope="session")
def gpu():
    """An Assembler factory; skips nothing -- a gpu-marked test on a host without a
    device fails, because the GPU path has no fallback."""
    import minifem
    return minifem.Assembler


GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    import numpy as np
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}
