"""The C-ABI library: it loads without a GPU, exports every symbol the public
headers declare, and answers the calls that need no device exactly like the
reference (pcg/sw/src/pcg.cpp:54-59, 175-215)."""
import ctypes as C
import os
import re
import subprocess

import pytest

import hpc_gb300 as X

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    syms = set()
    for h in ("pcg.h", "xjpcg_gb300.h"):
        with open(os.path.join(ROOT, "include", h)) as f:
            text = f.read()
        syms |= set(re.findall(r"\b(xJPCG_\w+)\s*\(", text))
    return syms


def test_library_exports_every_declared_symbol(built):
    lib = X.load()
    declared = _declared_symbols()
    assert declared == set(X.EXPORTED_SYMBOLS)
    out = subprocess.run(["nm", "-D", "--defined-only", X.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (xJPCG_\w+)", out))
    assert declared <= exported, declared - exported
    for s in declared:
        assert hasattr(lib, s)


def test_loader_soname_alias(built):
    alias = os.path.join(os.path.dirname(X.LIB_PATH), "libXilinxPcgStatic.so")
    assert os.path.islink(alias) and os.path.realpath(alias) == os.path.realpath(X.LIB_PATH)


def test_error_strings(built):
    names = ["XJPCG_STATUS_SUCCESS", "XJPCG_STATUS_NOT_INITIALIZED", "XJPCG_STATUS_ALLOC_FAILED",
             "XJPCG_STATUS_INVALID_VALUE", "XJPCG_STATUS_EXECUTION_FAILED", "XJPCG_STATUS_INTERNAL_ERROR",
             "XJPCG_STATUS_DYNAMIC_LOADING_ERROR"]
    for i, nm in enumerate(names):
        assert X.error_string(i) == nm
    assert X.error_string(7) == "Unknown Error Code!"
    assert X.error_string(-1) == "Unknown Error Code!"


def test_null_handle_paths(built):
    lib = X.load()
    assert lib.xJPCG_destroyHandle(None) == X.NOT_INITIALIZED
    assert lib.xJPCG_peekAtLastStatus(None) == X.NOT_INITIALIZED
    assert lib.xJPCG_getLastMessage(None) == b"Can't retrieve last error message from a null JPCG handle."
    m = X.Metric()
    assert lib.xJPCG_getMetrics(None, C.byref(m)) == X.NOT_INITIALIZED
    it, res = C.c_uint32(0), C.c_double(0)
    assert lib.xJPCG_cooSolver(None, 4, 4, None, None, None, None, None, None, 10, 1e-10, C.byref(it),
                               C.byref(res), 0) == X.NOT_INITIALIZED
    it64 = C.c_int64(0)
    assert lib.xJPCG_cscSymSolver(None, 4, 4, None, None, None, None, None, None, 10, 1e-10, C.byref(it64),
                                  C.byref(res), 0) == X.NOT_INITIALIZED
    assert lib.xJPCG_gbSpmv(None, None, None, 0) == X.NOT_INITIALIZED
    info = X.GbInfo()
    assert lib.xJPCG_gbGetInfo(None, C.byref(info)) == X.NOT_INITIALIZED
    assert lib.xJPCG_gbSetSpmvLanes(None, 4) == X.NOT_INITIALIZED
    assert lib.xJPCG_gbSetSpmvConfig(None, 0) == X.NOT_INITIALIZED
    assert lib.xJPCG_gbSetSpmvConfig32(None, 0) == X.NOT_INITIALIZED
    assert lib.xJPCG_gbSetSignatureSumOrder(None, 1) == X.NOT_INITIALIZED
    dev, ns = C.c_uint32(0), C.c_uint64(0)
    assert lib.xJPCG_gbDiagWaitTimeout(None, 1000, C.byref(dev), C.byref(ns)) == X.NOT_INITIALIZED
    assert lib.xJPCG_gbDiagCheckGuards(None, C.byref(dev)) == X.NOT_INITIALIZED
    r, ms = C.c_double(0.0), C.c_double(0.0)
    assert lib.xJPCG_gbDiagFp64Rate(None, 16, C.byref(r), C.byref(ms)) == X.NOT_INITIALIZED


def test_struct_layouts():
    assert C.sizeof(X.Metric) == 32
    assert X.RECORD_DTYPE.itemsize == 64
    assert list(X.RECORD_DTYPE.names) == ["id", "iter", "vecSize", "maxIter", "tols", "res", "rz", "alpha",
                                          "beta", "clock"]


def test_ctypes_mirrors_match_the_header(tmp_path):
    """The binding's ctypes structs have the C header's sizes and offsets."""
    import subprocess
    exe = str(tmp_path / "abi_layout")
    subprocess.run(["gcc", "-std=c99", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_layout.c"), "-o", exe], check=True)
    out = dict(line.split("=") for line in subprocess.run([exe], capture_output=True, text=True,
                                                         check=True).stdout.split())
    mirrors = {"XJPCG_GbInfo_t": X.GbInfo, "XJPCG_GbSignature_t": X.GbSignature}
    for cname, py in mirrors.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for key, val in out.items():
            if key.startswith(cname + "."):
                assert int(val) == getattr(py, key.split(".")[1]).offset, key
    assert int(out["XJPCG_GbBatchResult_t"]) == X.BATCH_RESULT_DTYPE.itemsize
    assert int(out["XJPCG_GbBatchResult_t.res"]) == X.BATCH_RESULT_DTYPE.fields["res"][1]
    assert int(out["XJPCG_Metric_t"]) == C.sizeof(X.Metric)
