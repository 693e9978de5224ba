"""Build libpfgpu.so from ../csrc for sm_103a (in-tree, git-ignored).

Each .cu translation unit compiles in parallel with
  nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo
and the objects link into pfgpu/libpfgpu.so (shared cudart, so the process
shares one CUDA runtime with PyTorch).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

from .abi import LIB_PATH, PKG_DIR

CSRC = os.path.join(os.path.dirname(PKG_DIR), "csrc")
BUILD = os.path.join(os.path.dirname(PKG_DIR), "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-cudart", "shared"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found")


def _deps():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + [
        os.path.join(os.path.dirname(os.path.dirname(PKG_DIR)), "include", "pfgpu.h")]


def build(force: bool = False, jobs: int | None = None, verbose: bool = False,
          extra_flags: list | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    dep_mtime = max(os.path.getmtime(p) for p in _deps())
    flags = NVCC_FLAGS + (extra_flags or [])
    cmds, objs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), dep_mtime):
            cmds.append([nvcc()] + flags + ["-c", s, "-o", o])
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 4))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    if cmds:
        with cf.ThreadPoolExecutor(jobs) as ex:
            for out in ex.map(run, cmds):
                if verbose and out.strip():
                    print(out)
    if cmds or not os.path.exists(LIB_PATH) or force:
        tmp = LIB_PATH + ".tmp"
        run([nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH
