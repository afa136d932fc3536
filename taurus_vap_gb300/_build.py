"""In-tree build of the native libraries.

* ``libtvap_setup.so``  host C++ model-space setup (basis, interaction, operators)
* ``libtvap_gpu.so``    the sm_103a device path and its C ABI (include/tvap.h)

Both are compiled next to their sources with plain ``g++`` / ``nvcc``
invocations (no cmake), for the architecture of the machine running the build.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")

SETUP_LIB = os.path.join(PKG_DIR, "libtvap_setup.so")
GPU_LIB = os.path.join(PKG_DIR, "libtvap_gpu.so")

GPU_SOURCES = [
    "tvap_context.cu",
    "fields.cu",
    "dense.cu",
    "projection.cu",
    "gradient.cu",
    "ozaki.cu",
    "jacobi_cluster.cu",
    "field_blocks.cu",
    "linalg_abi.cu",
    "diag_hsp_h11.cu",
    "constraints.cu",
    "state_batch.cu",
]

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the device library cannot be built")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        sys.stderr.write(res.stdout)
        raise RuntimeError("build step failed: " + " ".join(cmd))


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_setup(force: bool = False) -> str:
    src = os.path.join(CSRC, "setup", "tvap_setup.cpp")
    hdr = os.path.join(INCLUDE, "tvap_setup.h")
    if force or _stale(SETUP_LIB, [src, hdr]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", SETUP_LIB, src])
    return SETUP_LIB


def build_gpu(force: bool = False, verbose_ptxas: bool = False) -> str:
    srcs = [os.path.join(CSRC, s) for s in GPU_SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in ("tvap_internal.cuh", "ozaki_core.cuh", "ozaki_tc.cuh",
                                                   "ozaki_scaled.h")] + [
        os.path.join(INCLUDE, "tvap.h")
    ]
    if not (force or _stale(GPU_LIB, deps)):
        return GPU_LIB
    nvcc = _nvcc()
    objdir = os.path.join(CSRC, "_obj")
    os.makedirs(objdir, exist_ok=True)
    flags = NVCC_ARCH + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler",
        "-fPIC",
        "-rdc=false",
        "-I" + INCLUDE,
        "-I" + CSRC,
    ]
    if verbose_ptxas:
        flags += ["-Xptxas", "-v"]

    def compile_one(src: str) -> str:
        obj = os.path.join(objdir, os.path.basename(src).replace(".cu", ".o"))
        _run([nvcc] + flags + ["-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run([nvcc] + NVCC_ARCH + ["-shared", "-o", GPU_LIB] + objs + ["-lcudart"])
    return GPU_LIB


def build_all(force: bool = False) -> None:
    build_setup(force)
    build_gpu(force)
