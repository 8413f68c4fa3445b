"""In-tree build of libnbots_gpu.so (CUDA kernels for sm_103a + C ABI + C
drop-in of nbots' entry points) and libnbots_host.so (standalone host
objects for nbots' mesh / bc / material / element interfaces).

    python -m nbots_gb300.build [--force]

Translation units compile in parallel; objects land in nbots_gb300/_build/,
the shared libraries next to this file.  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
INC = os.path.join(ROOT, "include")
GPU_SO = os.path.join(PKG, "libnbots_gpu.so")
HOST_SO = os.path.join(PKG, "libnbots_host.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INC,
              "-I" + CSRC, "--expt-relaxed-constexpr"]
CC_FLAGS = ["-std=c99", "-O2", "-fPIC", "-Wall", "-I" + INC]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _headers():
    return (glob.glob(os.path.join(INC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(HOST, "*.h")))


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs, objs = [], []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj] +
                        (["-Xptxas", "-v"] if verbose else []))
    host_objs = []
    for src in sorted(glob.glob(os.path.join(HOST, "*.c"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        (host_objs if os.path.basename(src).startswith("nbh_") else objs).append(obj)
        if force or _stale(obj, [src] + hdrs):
            jobs.append(["gcc"] + CC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        for err in ex.map(_compile, jobs):
            if verbose and err:
                sys.stderr.write(err)
    cuda_lib = os.path.join(_cuda_home(), "lib64")
    if not os.path.isdir(cuda_lib):
        cuda_lib = os.path.join(_cuda_home(), "lib")
    if host_objs and (force or _stale(HOST_SO, host_objs)):
        tmp = HOST_SO + ".tmp"
        _compile(["gcc", "-shared", "-o", tmp] + host_objs + ["-lm"])
        os.replace(tmp, HOST_SO)
    if force or _stale(GPU_SO, objs):
        tmp = GPU_SO + ".tmp"
        # static cudart; unresolved nbots mesh/bc/material symbols bind at load
        # time to libnbots or to libnbots_host.so
        _compile([nvcc] + ARCH + ["-shared", "-o", tmp] + objs +
                 ["-Xcompiler", "-fPIC", "-L" + cuda_lib, "-lm"])
        os.replace(tmp, GPU_SO)
    return GPU_SO


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(GPU_SO)
