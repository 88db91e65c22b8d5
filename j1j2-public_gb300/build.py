"""Build libj1j2cuda.so in-tree: nvcc for sm_103a, host C++ with g++, no CMake.

    python j1j2-public_gb300/build.py [--force]

Translation units are compiled in parallel into _build/ and linked next to this file.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libj1j2cuda.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    cu = [os.path.join(CSRC, f)
          for f in ("sweep_fixed.cu", "sweep_hbm.cu", "sweep_multi.cu", "kernels.cu", "wolff.cu",
                    "enumerate.cu", "disorder.cu", "api.cu")]
    cpp = [os.path.join(CSRC, f) for f in ("host_model.cpp", "results.cpp")]
    hdr = [os.path.join(CSRC, f) for f in ("device_common.cuh", "engine.h", "sweep_common.cuh",
                                           "quad_sweep.cuh")]
    hdr.append(os.path.join(ROOT, "include", "j1j2c.h"))
    return cu, cpp, hdr


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    cu, cpp, hdr = _sources()
    newest = max(os.path.getmtime(p) for p in cu + cpp + hdr + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    cmds = []
    objs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler",
                     "-fPIC,-ffp-contract=off", "-Xptxas", "-v" if verbose else "-O3",
                     "-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                     "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        logs = list(ex.map(_compile, cmds))
    if verbose:
        for log in logs:
            sys.stdout.write(log)
    tmp = LIB + ".tmp"
    _compile([nvcc, ARCH, "-shared", "-o", tmp] + objs + ["-lcufft", "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
