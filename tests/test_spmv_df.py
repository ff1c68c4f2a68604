"""The double-float accumulation of the FP32-valued operator (csrc/spmv_df.cuh),
compiled for the host and run in the kernel's lane and chunk order, against
the exact sum of a x: the error relative to the row's sum of |a x| in units of
2^-48 stays below 16 for 3x3 blocks and 8 for scalars (the FP32 parts of x
alone carry 1), below 1 on average."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "mini-fem_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("spdf") / "spmv_df_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}",
                    os.path.join(ROOT, "tests", "spmv_df_check.cc"), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("dim,bound", [(1, 8.0), (3, 16.0)])
@pytest.mark.parametrize("seed", [7, 11, 12])
def test_spmv_double_float_error_bound(checker, dim, bound, seed):
    out = subprocess.run([checker, "200000", str(seed), str(dim)], capture_output=True, text=True, check=True)
    checked, worst, mean = out.stdout.split()
    assert int(checked) > 190_000 * dim, out.stdout
    assert float(worst) < bound, out.stdout
    assert float(mean) < 1.0, out.stdout
