"""The oracle: a CPU restatement of the xJPCG hot path, used as the checker.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
cpu_baseline / reference arm of ``bench.py`` may import this package.  The
product (``hpc_gb300``) never imports, links or runs it.

``jpcg_oracle.c`` holds the restated algorithm (see its header for the
reference file each function follows); this module builds it with gcc +
OpenMP into ``oracle/_build/libjpcg_oracle.so`` and wraps it with ctypes.
``ref_partition_harness.cpp`` + ``build_ref.sh`` compile the reference's own
partitioner (only where the reference sources exist) to pin the conversion.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libjpcg_oracle.so")
SRC = os.path.join(HERE, "jpcg_oracle.c")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_partition_harness")

RECORD_DTYPE = np.dtype([("id", "<u4"), ("iter", "<u4"), ("vecSize", "<u4"), ("maxIter", "<u4"),
                         ("tols", "<f8"), ("res", "<f8"), ("rz", "<f8"), ("alpha", "<f8"), ("beta", "<f8"),
                         ("clock", "<u8")])

_lib = None


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-Wall", SRC, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    return LIB


def reference_root() -> Optional[str]:
    """The Xilinx/HPC source tree named by XJPCG_REFERENCE_ROOT, or None."""
    root = os.environ.get("XJPCG_REFERENCE_ROOT")
    return root if root and os.path.isdir(root) else None


def build_ref(reference_root: Optional[str]) -> Optional[str]:
    """Builds oracle/_ref/ref_partition_harness from the reference tree at
    reference_root; returns None when no tree is given or it does not exist."""
    if not reference_root or not os.path.isdir(reference_root):
        return None
    subprocess.run([os.path.join(HERE, "build_ref.sh"), reference_root], check=True, capture_output=True)
    return REF_HARNESS


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.orc_coo_to_csr.argtypes = [C.c_uint32, C.c_uint64, P, P, C.c_int, P, P, P]
        L.orc_coo_to_csr.restype = C.c_int
        L.orc_cscsym_expand.argtypes = [C.c_uint32, C.c_uint64, P, P, P, C.c_int, P, P, P]
        L.orc_cscsym_expand.restype = C.c_int
        L.orc_spmv.argtypes = [C.c_uint32, P, P, P, P, P, C.c_int]
        L.orc_jpcg.argtypes = [C.c_uint32, P, P, P, P, P, C.c_uint32, C.c_double, P, C.POINTER(C.c_uint32),
                               C.POINTER(C.c_double), C.POINTER(C.c_uint32), P, C.c_uint64, C.c_uint32, C.c_int]
        L.orc_jpcg.restype = C.c_int
        L.orc_true_relres.argtypes = [C.c_uint32, P, P, P, P, P, C.c_int]
        L.orc_true_relres.restype = C.c_double
        L.orc_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def max_threads() -> int:
    return lib().orc_max_threads()


def coo_to_csr(n, row, col, base=0):
    """Returns (rowptr, col, perm) or raises ValueError on a bad index."""
    row = np.ascontiguousarray(row, np.uint32)
    col = np.ascontiguousarray(col, np.uint32)
    nnz = row.size
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(max(nnz, 1), np.int32)
    perm = np.zeros(max(nnz, 1), np.uint32)
    rc = lib().orc_coo_to_csr(n, nnz, _p(row), _p(col), base, _p(rp), _p(ci), _p(perm))
    if rc != 0:
        raise ValueError("index out of range (rc=%d)" % rc)
    return rp, ci[:nnz], perm[:nnz]


def cscsym_expand(n, row_idx, col_ptr, data, base=0):
    """Returns (row, col, val) of the full matrix in the reference's emission order."""
    row_idx = np.ascontiguousarray(row_idx, np.int64)
    col_ptr = np.ascontiguousarray(col_ptr, np.int64)
    data = np.ascontiguousarray(data, np.float64)
    full = (2 * data.size - n) & 0xffffffff
    r = np.zeros(full, np.uint32)
    c = np.zeros(full, np.uint32)
    v = np.zeros(full, np.float64)
    rc = lib().orc_cscsym_expand(n, full, _p(row_idx), _p(col_ptr), _p(data), base, _p(r), _p(c), _p(v))
    if rc != 0:
        raise ValueError("symmetric expansion failed (rc=%d)" % rc)
    return r, c, v


def spmv(rowptr, col, val, x, nthreads=0):
    n = rowptr.size - 1
    y = np.zeros(n, np.float64)
    lib().orc_spmv(n, _p(rowptr), _p(col), _p(val), _p(np.ascontiguousarray(x, np.float64)), _p(y), nthreads)
    return y


def jpcg(rowptr, col, val, diag, b, max_iter, tol, records=False, max_run=0, nthreads=0):
    """Jacobi-PCG with the xJPCG contract.  Returns dict(x, iters, res, k, status, records)."""
    n = rowptr.size - 1
    x = np.zeros(n, np.float64)
    it, res, k = C.c_uint32(0), C.c_double(0.0), C.c_uint32(0)
    rec = None
    cap = 0
    if records:
        cap = min(max_iter + 2, 1 << 20)
        rec = np.zeros(cap, RECORD_DTYPE)
    st = lib().orc_jpcg(n, _p(rowptr), _p(col), _p(val), _p(np.ascontiguousarray(diag, np.float64)),
                        _p(np.ascontiguousarray(b, np.float64)), max_iter, tol, _p(x), C.byref(it), C.byref(res),
                        C.byref(k), _p(rec), cap, max_run, nthreads)
    return {"x": x, "iters": it.value, "res": res.value, "k": k.value, "status": st, "records": rec}


def true_relres(rowptr, col, val, b, x, nthreads=0) -> float:
    n = rowptr.size - 1
    return lib().orc_true_relres(n, _p(rowptr), _p(col), _p(val), _p(np.ascontiguousarray(b, np.float64)),
                                 _p(np.ascontiguousarray(x, np.float64)), nthreads)


def ref_mismatches(x, ref, rtol=1e-4, atol=3e-6) -> int:
    """Mismatch count of the reference's test compare for doubles
    (utils/include/sw/utils.hpp:82-97, compare<double> -> isClose<float>(1e-4,
    3e-6)): both values are taken to float and |x - ref| <= atol + rtol |ref| is
    evaluated in float.  pcgtest.cpp:115-116 and the SpMV test
    (L2/sparse/tests/fp64/spmv/main.cpp:180-190) pass on zero mismatches."""
    xf = np.asarray(x, np.float64).astype(np.float32)
    rf = np.asarray(ref, np.float64).astype(np.float32)
    diff = np.abs(xf - rf)
    bound = np.float32(atol) + np.float32(rtol) * np.abs(rf)
    return int(np.count_nonzero(~(diff <= bound)))
