"""The double-float gradients that the FP32 tile kernel gives to poorly shaped
elements (csrc/grad_df.cuh) match the FP64 gradients rounded to FP32: their
portable form, compiled for the host, is compared with the FP64 formula on
flattened elements down to quality 1e-7, the error measured relative to each
element's largest gradient component in units of 2^-24 (FP32 rounding alone
gives up to 1); elements below quality 1e-4 are handed back to the FP64
formula, and only those."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "mini-fem_gb300", "csrc")


def test_double_float_gradients_match_fp64(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "df_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{CSRC}",
                    os.path.join(ROOT, "tests", "df_check.cc"), "-o", exe], check=True)
    out = subprocess.run([exe, "400000", "5"], capture_output=True, text=True)
    checked, worst, over, refused = out.stdout.split()[-4:]
    assert int(over) == 0, out.stdout
    assert float(worst) < 1.5, out.stdout
    assert int(checked) > 200_000 and int(refused) > 50_000
