"""In-tree build of the engine's shared library for sm_103a (no CMake).

Every CUDA / C++ translation unit under csrc/ is compiled in parallel by nvcc
with `-gencode arch=compute_103a,code=sm_103a`, then linked into
lib/libstellar_bh.so (CUDA runtime linked statically, so the library loads on
a host without a GPU).  The CLI app and the C++ host classes are built from
host/ against that library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libstellar_bh.so")
APP = os.path.join(LIB_DIR, "stellar_app")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off applies to host code only (device contraction is nvcc's --fmad):
# the reference's initial conditions must round the same on x86 and Arm hosts.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build")
    return exe


def _sources(folder, exts):
    if not os.path.isdir(folder):
        return []
    return sorted(os.path.join(folder, f) for f in os.listdir(folder) if f.endswith(exts))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    obj_dir = os.path.join(LIB_DIR, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    srcs = _sources(CSRC, (".cu", ".cpp"))
    objs, cmds = [], []
    for src in srcs:
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append([nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(cmds), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, cmds))
    _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs)
    host_srcs = _sources(HOST, (".cpp",))
    if host_srcs:
        _run([nvcc()] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off",
                                "-I" + INCLUDE, "-I" + HOST, "-o", APP]
             + host_srcs + ["-L" + LIB_DIR, "-lstellar_bh", "-Xlinker", "-rpath=$ORIGIN"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
