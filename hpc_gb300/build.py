"""Build recipe for libXilinxPcg.so (sm_103a) and the CPU oracle library.

The CUDA translation units are compiled in parallel with nvcc for
``-gencode arch=compute_103a,code=sm_103a`` only and linked into
``hpc_gb300/libXilinxPcg.so`` (with ``libXilinxPcgStatic.so``, the soname the
reference's dynamic loader opens, as a symlink).  Objects go to
``hpc_gb300/_build/``.  No cmake; a rebuild is skipped when every output is
newer than every source.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libXilinxPcg.so")
LIB_ALIAS = os.path.join(HERE, "libXilinxPcgStatic.so")
LOADER = os.path.join(HERE, "libXilinxPcg_loader.a")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
           "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include")]

SOURCES = ["spmv_kernels.cu", "spmv_sellpat.cu", "spmv_sellsort.cu", "spmv_merge.cu", "cg_kernels.cu", "mixed_kernels.cu", "convert_kernels.cu",
           "spmv_noalloc.cu", "batched_kernels.cu", "adjoint_kernels.cu", "signature_kernels.cu", "signature_export.cu", "fpga_order.cu", "pcg_handle.cpp", "pcg_api.cpp"]
HEADERS = ["xjpcg_device.cuh", "xjpcg_state.h", "xjpcg_internal.hpp", "pcg_handle.hpp"]


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(ROOT, "include", "pcg.h"), os.path.join(ROOT, "include", "xjpcg_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= _newest(deps):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else []
    cmd = [NVCC] + ARCH + NVFLAGS + lang + ["-c", src, "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, res.stdout, res.stderr))
    return obj


def build_library(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest(objs)):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-ldl", "-lrt", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (res.stdout, res.stderr))
    if os.path.lexists(LIB_ALIAS):
        os.remove(LIB_ALIAS)
    os.symlink(os.path.basename(LIB), LIB_ALIAS)
    build_loader()
    if verbose:
        print(LIB)
    return LIB


def build_loader() -> str:
    """libXilinxPcg_loader.a: the dlopen front end (csrc/pcg_loader.c) that an
    application links with -ldl instead of linking libXilinxPcg.so."""
    src = os.path.join(CSRC, "pcg_loader.c")
    obj = os.path.join(BUILD, "pcg_loader.o")
    deps = [src, os.path.join(ROOT, "include", "pcg.h")]
    if os.path.exists(LOADER) and os.path.getmtime(LOADER) >= _newest(deps):
        return LOADER
    cc = os.environ.get("CC", "gcc")
    for cmd in ([cc, "-std=c99", "-O2", "-fPIC", "-Wall", "-I" + os.path.join(ROOT, "include"), "-c", src, "-o", obj],
                ["ar", "rcs", LOADER + ".tmp", obj]):
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("loader build failed (%s):\n%s\n%s" % (cmd[0], res.stdout, res.stderr))
    os.replace(LOADER + ".tmp", LOADER)
    return LOADER


if __name__ == "__main__":
    build_library(verbose=True)
    sys.exit(0)
