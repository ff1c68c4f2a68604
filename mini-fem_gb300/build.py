"""In-tree build of the sm_103a library (no setuptools, no cmake).

    python mini-fem_gb300/build.py            # or __graft_entry__.build()

Compiles every csrc/*.cu with nvcc for sm_103a in parallel and links
lib/libminifem_gb300.so, then the C++ drop-in driver lib/minifem_fem, which
links the reference-signature operators of host/ against that library.
All translation units use -fmad=false: the FP64 path must not contract a
product and a sum into an FMA (the reference's arithmetic is unfused); the FP32
path asks for its FMAs explicitly with fmaf().
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
HOST = os.path.join(HERE, "host")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")
SO = os.path.join(LIB, "libminifem_gb300.so")
DRIVER = os.path.join(LIB, "minifem_fem")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-fno-strict-aliasing", f"-I{os.path.join(ROOT, 'include')}",
           f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "mfem_gpu.h"))
    nv = nvcc()
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s[:-3] + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append([nv, *ARCH, *NVFLAGS, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [os.path.join(OBJ, s[:-3] + ".o") for s in srcs]
    if force or _stale(SO, objs):
        _run([nv, *ARCH, "-shared", "-o", SO, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    # drop-in driver (reference signatures over the C ABI)
    hsrc = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cc")) \
        if os.path.isdir(HOST) else []
    if hsrc and (force or _stale(DRIVER, hsrc + [SO] + [os.path.join(HOST, f) for f in os.listdir(HOST)
                                                      if f.endswith(".h")])):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}",
              f"-I{HOST}", "-o", DRIVER, *hsrc, f"-L{LIB}", "-lminifem_gb300",
              f"-Wl,-rpath,{LIB}"])
    return SO


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
