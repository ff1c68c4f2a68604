"""The integer-pipe double multiplication that the FP64 kernels use for part of
their products, and the integer hi/lo split of the FP32 path's coordinates, must
give the FP64 unit's bits.  On the CPU its portable form is
compared with the host's IEEE multiplication; on the GPU the library's
self-test compares the device form with the FP64 unit."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "mini-fem_gb300", "csrc")


def test_matches_host_multiplication(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "dmul_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}",
                    os.path.join(ROOT, "tests", "dmul_check.cc"), "-o", exe], check=True)
    out = subprocess.run([exe, "6000000", "7"], capture_output=True, text=True, check=True)
    fast, bad = (int(x) for x in out.stdout.split()[-2:])
    assert bad == 0, out.stdout
    assert fast > 11_000_000     # most products and splits take the fast path


@pytest.mark.gpu
def test_device_form_matches_fp64_unit(gpu):
    a = gpu(0)
    fast, bad = a.selftest_dmul(1 << 28, seed=11)
    assert bad == 0
    assert fast > (1 << 27)
