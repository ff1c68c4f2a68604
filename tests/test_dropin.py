"""The drop-in: the reference-signature operators (include/minifem_dropin.h) driven
by a FEM loop -- the reference's own main.cc/FEM.cc/IO.cc where the reference
tree exists (link check here), and the package's minifem_fem driver on the GPU."""
import os
import subprocess

import pytest

import pyoracle as O
from conftest import PKG, ROOT
from minifem.meshgen import cube_mesh, write_reference_tree

DRIVER = os.path.join(PKG, "lib", "minifem_fem")
REF = O.ref_available()


def tree(tmp_path, op, n=6, seed=9):
    m = cube_mesh(n, seed=seed, op=op, coefficients=False)
    r = O.full(m, op=op, coef=None)
    write_reference_tree(m, str(tmp_path), "LM6", op, O.norm(r["values"]), O.norm(r["prec"]))
    return m


def run(exe, tmp_path, op, iters=3, env=None):
    e = {**os.environ, "MINIFEM_DATA_PATH": str(tmp_path), **(env or {})}
    return subprocess.run([exe, "LM6", op, str(iters)], cwd=tmp_path, capture_output=True,
                          text=True, env=e, timeout=300)


def differences(out):
    return [float(l.split(":")[1]) for l in out.splitlines() if "difference" in l]


def _no_gpu():
    import torch
    return not torch.cuda.is_available()


@pytest.mark.skipif(not REF, reason="reference tree not present")
def test_reference_driver_links_against_dropin(tmp_path):
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = os.path.join(ROOT, "oracle", "_ref", "miniFEM_gpu")
    assert os.path.exists(exe)
    if _no_gpu():
        tree(tmp_path, "ela")
        out = run(exe, tmp_path, "ela")
        # no device: the operators fail loudly, there is no CPU path
        assert out.returncode != 0 and "no CUDA device" in out.stderr


def test_driver_fails_loudly_without_device(tmp_path):
    if not _no_gpu():
        pytest.skip("a device is present")
    tree(tmp_path, "lap")
    out = run(DRIVER, tmp_path, "lap")
    assert out.returncode != 0 and "no CUDA device" in out.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["lap", "ela"])
def test_driver_norm_check_bit_exact(tmp_path, op):
    tree(tmp_path, op)
    out = run(DRIVER, tmp_path, op)
    assert out.returncode == 0, out.stderr
    assert differences(out.stdout) == [0.0, 0.0], out.stdout


@pytest.mark.gpu
def test_driver_with_gpu_colouring(tmp_path):
    tree(tmp_path, "ela")
    out = run(DRIVER, tmp_path, "ela", env={"MINIFEM_COLORING": "1"})
    assert out.returncode == 0, out.stderr
    d = differences(out.stdout)
    assert len(d) == 2 and max(d) < 1e-13, out.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["lap", "ela"])
def test_driver_optimized_build_flow(tmp_path, op):
    """src/main.cc with COLORING and OPTIMIZED: colouring, in-place element
    permutation, CSR from the node -> element lists, create_elemToEdge, FEM loop."""
    tree(tmp_path, op)
    out = run(DRIVER, tmp_path, op, env={"MINIFEM_COLORING": "1", "MINIFEM_OPTIMIZED": "1"})
    assert out.returncode == 0, out.stderr
    assert "Edges index" in out.stdout
    d = differences(out.stdout)
    assert len(d) == 2 and max(d) < 1e-13, out.stdout
