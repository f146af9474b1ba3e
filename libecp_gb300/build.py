"""Builds libecp_gb300/libecp_gb300.so for sm_103a (in-tree, no cmake).

Each translation unit compiles in parallel with nvcc; the FP64 kernels get
--fmad=false so their arithmetic rounds like the reference's C.  Objects go to
libecp_gb300/_build/ (git-ignored); the shared object lands next to this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libecp_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("ecp_fp64.cu", ["--fmad=false"]),
    ("ecp_host.cu", []),
    ("ecp_peaks.cu", []),
    ("ecp_tables.cpp", []),
    ("ecp_capi.cpp", []),
    ("ecp_noalloc.cu", []),
    ("ecp_fast.cu", []),
    ("ecp_serve.cpp", []),
    ("ecp_io.cpp", []),
    ("ecp_grad.cu", []),
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the ECP engine needs the CUDA toolkit to build")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")] + \
        [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", path, "-o", obj, *extra]
    if src.endswith(".cu"):
        cmd += ["--extended-lambda", "-Xptxas", "-warn-spills"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda u: _compile(*u), UNITS))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
