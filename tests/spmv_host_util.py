"""Builds tests/c/spmv_host_app.cpp (an application of the SpMV host classes
in include/spmvHost_gb300.hpp) and lays out a partitioned matrix and its
vectors as the reference's SpMV test reads them."""
from __future__ import annotations

import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "hpc_gb300")


def build_app(outdir: str) -> str:
    from hpc_gb300 import build as B
    B.build_library()
    exe = os.path.join(outdir, "spmv_host_app")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I" + INCLUDE,
                    os.path.join(HERE, "c", "spmv_host_app.cpp"), "-L" + LIBDIR, "-lXilinxPcg",
                    "-Wl,-rpath," + LIBDIR, "-o", exe], check=True)
    return exe


def write_case(g: dict, sig_dir: str, vec_dir: str, x: np.ndarray, y_ref: np.ndarray) -> None:
    """The reference test's files: <sig_dir>/{nnzVal_0..15,parParam,rbParam,
    info}.dat from a golden fixture's raw partitioner output, and
    <vec_dir>/{inVec,refVec}.dat."""
    os.makedirs(sig_dir, exist_ok=True)
    os.makedirs(vec_dir, exist_ok=True)
    names = ["nnzVal_%d" % c for c in range(16)] + ["parParam", "rbParam", "info"]
    for nm in names:
        with open(os.path.join(sig_dir, nm + ".dat"), "wb") as f:
            f.write(np.asarray(g["sig_raw_" + nm], np.uint8).tobytes())
    np.asarray(x, np.float64).tofile(os.path.join(vec_dir, "inVec.dat"))
    np.asarray(y_ref, np.float64).tofile(os.path.join(vec_dir, "refVec.dat"))
