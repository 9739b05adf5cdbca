"""hpc_gb300 -- GB300-native xJPCG (Jacobi-preconditioned CG with an fp64 CSR SpMV).

The product is ``libXilinxPcg.so`` (C ABI in ``include/pcg.h`` and
``include/xjpcg_gb300.h``).  This module loads it with ctypes and mirrors the
reference's xJPCG API (Xilinx/HPC pcg/sw/include/pcg.h) for Python callers and
tests: the same entry points, argument meaning, status codes and messages.

There is no CPU fallback: if the CUDA library is missing or cannot be loaded,
``load()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libXilinxPcg.so")

# XJPCG_Status_t (pcg.h:41-49)
SUCCESS, NOT_INITIALIZED, ALLOC_FAILED, INVALID_VALUE, EXECUTION_FAILED, INTERNAL_ERROR, \
    DYNAMIC_LOADING_ERROR = range(7)
STATUS_NAMES = ["XJPCG_STATUS_SUCCESS", "XJPCG_STATUS_NOT_INITIALIZED", "XJPCG_STATUS_ALLOC_FAILED",
                "XJPCG_STATUS_INVALID_VALUE", "XJPCG_STATUS_EXECUTION_FAILED", "XJPCG_STATUS_INTERNAL_ERROR",
                "XJPCG_STATUS_DYNAMIC_LOADING_ERROR"]
# XJPCG_Mode_t (pcg.h:79-85)
MODE_DEFAULT, MODE_KEEP_NZ_LAYOUT, MODE_KEEP_MATRIX = 0x00, 0x01, 0x02
MODE_C_INDEX, MODE_FORTRAN_INDEX = 0x00, 0x10

# Symbols declared in include/pcg.h and include/xjpcg_gb300.h.
EXPORTED_SYMBOLS = [
    "xJPCG_getErrorString", "xJPCG_createHandle", "xJPCG_destroyHandle", "xJPCG_cscSymSolver",
    "xJPCG_cooSolver", "xJPCG_peekAtLastStatus", "xJPCG_getLastMessage", "xJPCG_getMetrics",
    "xJPCG_gbCsrSolver", "xJPCG_gbSolveDevice", "xJPCG_gbMixedSolve", "xJPCG_gbSpmv", "xJPCG_gbGetCsr",
    "xJPCG_gbGetRecords", "xJPCG_gbGetInfo", "xJPCG_gbGetStream", "xJPCG_gbSetSpmvLanes", "xJPCG_gbSetSpmvConfig", "xJPCG_gbSetSpmvConfig32",
    "xJPCG_gbGetSpmvTuning", "xJPCG_gbSpmvDotNoAlloc", "xJPCG_gbBatchSolve",
    "xJPCG_gbAdjointSolve", "xJPCG_gbEdgeGrad", "xJPCG_gbSetSignatureMatrix", "xJPCG_gbSignatureSpmv", "xJPCG_gbSetSignatureSumOrder",
    "xJPCG_gbExportSignature", "xJPCG_gbGetSignature", "xJPCG_gbGetSpmvTuning32", "xJPCG_gbDiagWaitTimeout",
    "xJPCG_gbDiagCheckGuards", "xJPCG_gbDiagFp64Rate", "xJPCG_gbCreateHandleOnDevice", "xJPCG_gbStoreYFrames",
    "xJPCG_gbSignatureSolve",
]


class Metric(C.Structure):
    """XJPCG_Metric_t (pcg.h:62-67)."""
    _fields_ = [("m_objInit", C.c_double), ("m_matProc", C.c_double), ("m_vecProc", C.c_double),
                ("m_solver", C.c_double)]


class GbInfo(C.Structure):
    """XJPCG_GbInfo_t (xjpcg_gb300.h)."""
    _fields_ = [("n", C.c_uint32), ("n4", C.c_uint32), ("nnz", C.c_uint64), ("itersRun", C.c_uint32),
                ("spmvLanes", C.c_uint32), ("spmvGrid", C.c_uint32), ("statusBits", C.c_uint32),
                ("outerSweeps", C.c_uint32), ("innerIters", C.c_uint32), ("bb", C.c_double),
                ("rrLast", C.c_double), ("solveMs", C.c_double), ("loopMode", C.c_uint32),
                ("spmvLayout", C.c_uint32), ("batchThreads", C.c_uint32), ("batchLanes", C.c_uint32),
                ("batchSmemRows", C.c_uint32), ("batchGrid", C.c_uint32), ("batchMs", C.c_double),
                ("spmvCfg", C.c_uint32), ("spmvCfg32", C.c_uint32), ("spmvLayout32", C.c_uint32),
                ("batchSliced", C.c_uint32), ("tuneMs", C.c_double), ("uploadMs", C.c_double),
                ("uploadIdxMs", C.c_double), ("uploadValMs", C.c_double), ("loopUnroll", C.c_uint32),
                ("kernelsPerIter", C.c_uint32)]


class GbSignature(C.Structure):
    """XJPCG_GbSignature_t (xjpcg_gb300.h)."""
    _fields_ = [("info", C.c_uint32 * 6), ("rowBlocks", C.c_uint32), ("partitions", C.c_uint32),
                ("rbParamBytes", C.c_uint64), ("parParamBytes", C.c_uint64), ("nnzValBytes", C.c_uint64 * 16)]


BATCH_RESULT_DTYPE = np.dtype([("iters", "<u4"), ("itersRun", "<u4"), ("outer", "<u4"), ("status", "<u4"),
                               ("res", "<f8")])
assert BATCH_RESULT_DTYPE.itemsize == 24


RECORD_DTYPE = np.dtype([("id", "<u4"), ("iter", "<u4"), ("vecSize", "<u4"), ("maxIter", "<u4"),
                         ("tols", "<f8"), ("res", "<f8"), ("rz", "<f8"), ("alpha", "<f8"), ("beta", "<f8"),
                         ("clock", "<u8")])
assert RECORD_DTYPE.itemsize == 64

_lib = None
_P = C.c_void_p


def _ptr(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data


def load(path: str = LIB_PATH) -> C.CDLL:
    """Loads libXilinxPcg.so and declares its signatures.  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libXilinxPcg.so is not built (run __graft_entry__.build()); no CPU fallback exists")
    lib = C.CDLL(path)
    u32, i64, u64, dbl = C.c_uint32, C.c_int64, C.c_uint64, C.c_double
    lib.xJPCG_getErrorString.restype = C.c_char_p
    lib.xJPCG_getErrorString.argtypes = [C.c_int]
    lib.xJPCG_createHandle.argtypes = [C.POINTER(_P), C.c_char_p]
    lib.xJPCG_destroyHandle.argtypes = [_P]
    lib.xJPCG_cscSymSolver.argtypes = [_P, i64, i64, _P, _P, _P, _P, _P, _P, i64, dbl, C.POINTER(i64),
                                       C.POINTER(dbl), C.c_int]
    lib.xJPCG_cooSolver.argtypes = [_P, u32, u32, _P, _P, _P, _P, _P, _P, u32, dbl, C.POINTER(u32), C.POINTER(dbl),
                                    C.c_int]
    lib.xJPCG_peekAtLastStatus.argtypes = [_P]
    lib.xJPCG_getLastMessage.restype = C.c_char_p
    lib.xJPCG_getLastMessage.argtypes = [_P]
    lib.xJPCG_getMetrics.argtypes = [_P, C.POINTER(Metric)]
    lib.xJPCG_gbCsrSolver.argtypes = [_P, u32, u32, _P, _P, _P, _P, _P, _P, u32, dbl, C.POINTER(u32),
                                      C.POINTER(dbl), C.c_int]
    lib.xJPCG_gbSolveDevice.argtypes = [_P, _P, _P, _P, u32, dbl, C.POINTER(u32), C.POINTER(dbl)]
    lib.xJPCG_gbMixedSolve.argtypes = [_P, _P, _P, _P, u32, dbl, C.POINTER(u32), C.POINTER(dbl), C.c_int]
    lib.xJPCG_gbSpmv.argtypes = [_P, _P, _P, C.c_int]
    lib.xJPCG_gbGetCsr.argtypes = [_P, _P, _P, _P, _P]
    lib.xJPCG_gbGetRecords.argtypes = [_P, _P, u64, C.POINTER(u64)]
    lib.xJPCG_gbGetInfo.argtypes = [_P, C.POINTER(GbInfo)]
    lib.xJPCG_gbGetStream.argtypes = [_P, C.POINTER(_P)]
    lib.xJPCG_gbSetSpmvLanes.argtypes = [_P, C.c_int]
    lib.xJPCG_gbSetSpmvConfig.argtypes = [_P, C.c_int]
    lib.xJPCG_gbSetSpmvConfig32.argtypes = [_P, C.c_int]
    lib.xJPCG_gbDiagWaitTimeout.argtypes = [_P, u64, C.POINTER(u32), C.POINTER(u64)]
    lib.xJPCG_gbDiagCheckGuards.argtypes = [_P, C.POINTER(u32)]
    lib.xJPCG_gbDiagFp64Rate.argtypes = [_P, C.c_int32, C.POINTER(dbl), C.POINTER(dbl)]
    lib.xJPCG_gbCreateHandleOnDevice.argtypes = [C.POINTER(_P), C.c_int, C.c_char_p]
    lib.xJPCG_gbStoreYFrames.argtypes = [_P, u64, u32, _P, u64, C.POINTER(u64)]
    lib.xJPCG_gbSignatureSolve.argtypes = [_P, u32, _P, _P, _P, u32, dbl, C.POINTER(u32), C.POINTER(dbl)]
    lib.xJPCG_gbGetSpmvTuning.argtypes = [_P, _P, _P, C.c_int32, C.POINTER(C.c_int32)]
    lib.xJPCG_gbGetSpmvTuning32.argtypes = [_P, _P, C.c_int32, C.POINTER(C.c_int32)]
    lib.xJPCG_gbSpmvDotNoAlloc.argtypes = [u32, _P, _P, _P, _P, _P, _P, _P]
    lib.xJPCG_gbAdjointSolve.argtypes = [_P, _P, _P, _P, _P, u32, dbl, C.POINTER(u32), C.POINTER(dbl), C.c_int]
    lib.xJPCG_gbEdgeGrad.argtypes = [_P, i64, _P, _P, _P, _P, C.c_int]
    lib.xJPCG_gbSetSignatureMatrix.argtypes = [_P, u32, _P, _P, _P, u64, _P, u64]
    lib.xJPCG_gbSignatureSpmv.argtypes = [_P, _P, u32, _P, u32, u32, _P, u64]
    lib.xJPCG_gbSetSignatureSumOrder.argtypes = [_P, C.c_int]
    lib.xJPCG_gbExportSignature.argtypes = [_P, _P]
    lib.xJPCG_gbGetSignature.argtypes = [_P, _P, _P, _P]
    lib.xJPCG_gbBatchSolve.argtypes = [_P, u32, _P, _P, _P, _P, _P, _P, _P, u32, dbl, C.c_int, _P, C.c_int]
    for name in EXPORTED_SYMBOLS:
        fn = getattr(lib, name)
        if name not in ("xJPCG_getErrorString", "xJPCG_getLastMessage"):
            fn.restype = C.c_int
    _lib = lib
    return lib


def spmv_dot_no_alloc(n: int, d_rowptr: int, d_col: int, d_val: int, d_x: int, d_y: int, d_dot: int,
                      stream: int = 0) -> int:
    """xJPCG_gbSpmvDotNoAlloc: y = A x and x.y on caller-owned device memory,
    with no device allocation (see include/xjpcg_gb300.h).  Returns the status."""
    return load().xJPCG_gbSpmvDotNoAlloc(n, d_rowptr, d_col, d_val, d_x, d_y, d_dot, stream or None)


def store_y_frames(frames: bytes, num_nodes: int, y) -> tuple:
    """xJPCG_gbStoreYFrames: writes num_nodes transY frames into the float64
    array y in place (host only).  Returns (status, bytes of frames read)."""
    buf = np.frombuffer(bytes(frames), np.uint8)
    assert y.dtype == np.float64 and y.flags["C_CONTIGUOUS"]
    used = C.c_uint64(0)
    st = load().xJPCG_gbStoreYFrames(buf.ctypes.data if buf.size else None, buf.size, num_nodes,
                                     y.ctypes.data, y.nbytes, C.byref(used))
    return st, used.value


def error_string(code: int) -> str:
    return load().xJPCG_getErrorString(code).decode()


class XJPCGError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < 7 else status, message))
        self.status = status
        self.message = message


@dataclass
class SolveResult:
    status: int
    x: np.ndarray
    iters: int
    res: float
    message: str


class JPCG:
    """One xJPCG handle (xJPCG_createHandle / xJPCG_destroyHandle).

    Methods mirror the reference's C API; each returns the XJPCG status and the
    outputs, and never raises for a solver status (check ``.status``).
    """

    def __init__(self, xclbin: str = "", device: Optional[int] = None):
        self.lib = load()
        self.h = _P()
        if device is None:
            st = self.lib.xJPCG_createHandle(C.byref(self.h), xclbin.encode())
        else:
            st = self.lib.xJPCG_gbCreateHandleOnDevice(C.byref(self.h), device, xclbin.encode())
        if st != SUCCESS:
            msg = self.last_message()
            raise XJPCGError(st, msg)

    def close(self):
        if self.h:
            self.lib.xJPCG_destroyHandle(self.h)
            self.h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- status ---
    def last_status(self) -> int:
        return self.lib.xJPCG_peekAtLastStatus(self.h)

    def last_message(self) -> str:
        return self.lib.xJPCG_getLastMessage(self.h).decode()

    def metrics(self) -> Metric:
        m = Metric()
        self.lib.xJPCG_getMetrics(self.h, C.byref(m))
        return m

    def info(self) -> GbInfo:
        i = GbInfo()
        self.lib.xJPCG_gbGetInfo(self.h, C.byref(i))
        return i

    def stream(self) -> int:
        s = _P()
        self.lib.xJPCG_gbGetStream(self.h, C.byref(s))
        return s.value or 0

    # --- solvers (pcg.h) ---
    def coo_solve(self, n, row, col, data, diag, b, max_iter, tol, mode=MODE_DEFAULT, nnz=None,
                  x: Optional[np.ndarray] = None) -> SolveResult:
        x = np.zeros(n, np.float64) if x is None else x
        it, res = C.c_uint32(0), C.c_double(0.0)
        if nnz is None:
            nnz = len(data) if data is not None else (len(row) if row is not None else 0)
        st = self.lib.xJPCG_cooSolver(self.h, n, nnz, _ptr(row), _ptr(col), _ptr(data), _ptr(diag), _ptr(b), _ptr(x),
                                      max_iter, tol, C.byref(it), C.byref(res), mode)
        return SolveResult(st, x, it.value, res.value, self.last_message())

    def csc_sym_solve(self, n, row_idx, col_ptr, data, diag, b, max_iter, tol, mode=MODE_DEFAULT, nnz=None,
                      x: Optional[np.ndarray] = None) -> SolveResult:
        x = np.zeros(n, np.float64) if x is None else x
        it, res = C.c_int64(0), C.c_double(0.0)
        if nnz is None:
            nnz = len(data) if data is not None else (len(row_idx) if row_idx is not None else 0)
        st = self.lib.xJPCG_cscSymSolver(self.h, n, nnz, _ptr(row_idx), _ptr(col_ptr), _ptr(data), _ptr(diag),
                                         _ptr(b), _ptr(x), max_iter, tol, C.byref(it), C.byref(res), mode)
        return SolveResult(st, x, it.value, res.value, self.last_message())

    # --- extensions (xjpcg_gb300.h) ---
    def csr_solve(self, n, rowptr, col, data, diag, b, max_iter, tol, mode=MODE_DEFAULT,
                  x: Optional[np.ndarray] = None) -> SolveResult:
        x = np.zeros(n, np.float64) if x is None else x
        it, res = C.c_uint32(0), C.c_double(0.0)
        nnz = len(data)
        st = self.lib.xJPCG_gbCsrSolver(self.h, n, nnz, _ptr(rowptr), _ptr(col), _ptr(data), _ptr(diag), _ptr(b),
                                        _ptr(x), max_iter, tol, C.byref(it), C.byref(res), mode)
        return SolveResult(st, x, it.value, res.value, self.last_message())

    def solve_device(self, d_b: int, d_diag: int, d_x: int, max_iter: int, tol: float):
        it, res = C.c_uint32(0), C.c_double(0.0)
        st = self.lib.xJPCG_gbSolveDevice(self.h, d_b, d_diag, d_x, max_iter, tol, C.byref(it), C.byref(res))
        return st, it.value, res.value

    def mixed_solve(self, b, diag, max_iter, tol, x=None, on_device=False):
        if not on_device:
            x = np.zeros(len(b), np.float64) if x is None else x
        it, res = C.c_uint32(0), C.c_double(0.0)
        st = self.lib.xJPCG_gbMixedSolve(self.h, _ptr(b), _ptr(diag), _ptr(x), max_iter, tol, C.byref(it),
                                         C.byref(res), 1 if on_device else 0)
        return SolveResult(st, x, it.value, res.value, self.last_message())

    def spmv(self, x, y=None, on_device=False):
        if not on_device and y is None:
            y = np.zeros(len(x), np.float64)
        st = self.lib.xJPCG_gbSpmv(self.h, _ptr(x), _ptr(y), 1 if on_device else 0)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        return y

    def get_csr(self):
        inf = self.info()
        n, nnz = inf.n, inf.nnz
        rp = np.zeros(n + 1, np.int32)
        ci = np.zeros(nnz, np.int32)
        v = np.zeros(nnz, np.float64)
        perm = np.zeros(nnz, np.uint32)
        st = self.lib.xJPCG_gbGetCsr(self.h, _ptr(rp), _ptr(ci), _ptr(v), _ptr(perm))
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        return rp, ci, v, perm

    def records(self, cap: int = 1 << 20) -> np.ndarray:
        buf = np.zeros(cap, RECORD_DTYPE)
        cnt = C.c_uint64(0)
        st = self.lib.xJPCG_gbGetRecords(self.h, _ptr(buf), cap, C.byref(cnt))
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        return buf[:cnt.value]

    def adjoint(self, g, diag, max_iter, tol, grad_a=False, lam=None):
        """lambda = A^-1 g for the last solve's matrix; optionally dL/dA per
        input entry.  `lam` (float64, n) receives lambda if given.  Returns
        (status, lambda, gradA or None, iters, res)."""
        n = len(g)
        if lam is None:
            lam = np.zeros(n, np.float64)
        elif lam.dtype != np.float64 or lam.size != n or not lam.flags["C_CONTIGUOUS"]:
            raise ValueError("lam must be a contiguous float64 array of length n")
        ga = np.zeros(self.info().nnz, np.float64) if grad_a else None
        it, res = C.c_uint32(0), C.c_double(0.0)
        st = self.lib.xJPCG_gbAdjointSolve(self.h, _ptr(np.ascontiguousarray(g, np.float64)),
                                           _ptr(np.ascontiguousarray(diag, np.float64)), _ptr(lam), _ptr(ga),
                                           max_iter, tol, C.byref(it), C.byref(res), 0)
        return st, lam, ga, it.value, res.value

    def edge_grad(self, ei, ej, c, out=None):
        """dL/dtheta per edge, -c (lambda_i - lambda_j)(x_i - x_j), after an
        adjoint solve; `out` (float64, one per edge) receives it if given."""
        ei = np.ascontiguousarray(ei, np.int32)
        ej = np.ascontiguousarray(ej, np.int32)
        c = np.ascontiguousarray(c, np.float64)
        if out is None:
            out = np.zeros(ei.size, np.float64)
        elif out.dtype != np.float64 or out.size != ei.size or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float64 array with one entry per edge")
        st = self.lib.xJPCG_gbEdgeGrad(self.h, ei.size, _ptr(ei), _ptr(ej), _ptr(c), _ptr(out), 0)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        return out

    def batch_solve(self, systems, max_iter, tol, precision=0):
        """Concatenates `systems` (objects with n, rowptr, col, val, diag, b),
        solves them in one batched launch and returns (status, [x_s], results)."""
        n = np.array([s.n for s in systems], np.int64)
        sys_row = np.zeros(len(systems) + 1, np.int32)
        np.cumsum(n, out=sys_row[1:])
        nnz = np.array([s.nnz for s in systems], np.int64)
        offs = np.zeros(len(systems) + 1, np.int64)
        np.cumsum(nnz, out=offs[1:])
        rowptr = np.concatenate([systems[0].rowptr[:1].astype(np.int64) * 0] +
                                [s.rowptr[1:].astype(np.int64) + offs[i] for i, s in enumerate(systems)])
        rowptr = rowptr.astype(np.int32)
        col = np.concatenate([s.col for s in systems]).astype(np.int32)
        val = np.concatenate([s.val for s in systems])
        diag = np.concatenate([s.diag for s in systems])
        b = np.concatenate([s.b for s in systems])
        x = np.zeros(int(sys_row[-1]), np.float64)
        res = np.zeros(len(systems), BATCH_RESULT_DTYPE)
        st = self.lib.xJPCG_gbBatchSolve(self.h, len(systems), _ptr(sys_row), _ptr(rowptr), _ptr(col), _ptr(val),
                                         _ptr(diag), _ptr(b), _ptr(x), max_iter, tol, precision, _ptr(res), 0)
        xs = [x[sys_row[i]:sys_row[i + 1]] for i in range(len(systems))]
        return st, xs, res

    def set_signature_matrix(self, nnz_bufs, par_param, rb_param):
        """Loads the reference's partitioned-matrix buffers (16 nnzVal channel
        buffers, parParam, rbParam as numpy uint8 arrays)."""
        bufs = [np.ascontiguousarray(b, np.uint8) for b in nnz_bufs]
        ptrs = (C.c_void_p * len(bufs))(*[b.ctypes.data for b in bufs])
        sizes = (C.c_uint64 * len(bufs))(*[b.size for b in bufs])
        par = np.ascontiguousarray(par_param, np.uint8)
        rb = np.ascontiguousarray(rb_param, np.uint8)
        st = self.lib.xJPCG_gbSetSignatureMatrix(self.h, len(bufs), C.cast(ptrs, C.c_void_p), C.cast(sizes, C.c_void_p),
                                                 _ptr(par), par.size, _ptr(rb), rb.size)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        self._sig_keep = (bufs, par, rb)

    def set_signature_sum_order(self, order: int):
        """0: tuned SpMV kernels; 1: the reference FPGA's summation order (bit-exact C semantics)."""
        st = self.lib.xJPCG_gbSetSignatureSumOrder(self.h, order)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())

    def signature_spmv(self, x, y_rows, start_addr=0, frame=False):
        """y = A x on the partitioned matrix; optionally the transY frame."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros(y_rows, np.float64)
        fb = 64 + 64 * max(1, (y_rows + 7) // 8)
        fr = np.zeros(fb, np.uint8) if frame else None
        st = self.lib.xJPCG_gbSignatureSpmv(self.h, _ptr(x), x.size, _ptr(y), y_rows, start_addr, _ptr(fr),
                                            fb if frame else 0)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        return (y, fr) if frame else y

    def signature_solve(self, b, diag, max_iter, tol):
        """JPCG on the partitioned matrix (xJPCG_gbSignatureSolve); with sum
        order 1, in the reference FPGA's arithmetic order.  Returns a result
        with status, x, iters, res and message."""
        b = np.ascontiguousarray(b, np.float64)
        diag = np.ascontiguousarray(diag, np.float64)
        x = np.zeros(b.size, np.float64)
        it, res = C.c_uint32(0), C.c_double(0.0)
        st = self.lib.xJPCG_gbSignatureSolve(self.h, b.size, _ptr(b), _ptr(diag), _ptr(x), max_iter, tol,
                                             C.byref(it), C.byref(res))
        return SolveResult(st, x, it.value, res.value, self.last_message())

    def export_signature(self) -> dict:
        """The stored matrix in the reference's partitioned format:
        {"rbParam", "parParam", "nnzVal_0".."nnzVal_15", "info"} -> bytes, the
        contents of the files storeMatPar writes (xJPCG_gbExportSignature)."""
        sig = GbSignature()
        st = self.lib.xJPCG_gbExportSignature(self.h, C.byref(sig))
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        rb = np.zeros(sig.rbParamBytes, np.uint8)
        par = np.zeros(sig.parParamBytes, np.uint8)
        chans = [np.zeros(sig.nnzValBytes[c], np.uint8) for c in range(16)]
        ptrs = (C.c_void_p * 16)(*[c.ctypes.data for c in chans])
        st = self.lib.xJPCG_gbGetSignature(self.h, _ptr(rb), _ptr(par), ptrs)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        out = {"rbParam": rb.tobytes(), "parParam": par.tobytes(),
               "info": np.array(list(sig.info), np.uint32).tobytes()}
        for c in range(16):
            out["nnzVal_%d" % c] = chans[c].tobytes()
        return out

    def store_signature(self, path: str) -> dict:
        """Writes rbParam.dat, parParam.dat, nnzVal_<c>.dat and info.dat into
        the directory `path` (storeMatPar, gen_signature.cpp:58-81)."""
        import os
        files = self.export_signature()
        os.makedirs(path, exist_ok=True)
        for name, data in files.items():
            with open(os.path.join(path, name + ".dat"), "wb") as f:
                f.write(data)
        return files

    def spmv_tuning(self):
        """[(lanes, consumers, chunk, stages, ms)] of the last SpMV tuning."""
        ms = np.zeros(64, np.float32)
        shape = np.zeros(256, np.int32)
        cnt = C.c_int32(0)
        self.lib.xJPCG_gbGetSpmvTuning(self.h, _ptr(ms), _ptr(shape), 64, C.byref(cnt))
        return [tuple(int(v) for v in shape[4 * i:4 * i + 4]) + (float(ms[i]),) for i in range(cnt.value)]

    def spmv_tuning32(self):
        """[ms] of the mixed solver's FP32 SpMV tuning (-1: not timed)."""
        ms = np.zeros(64, np.float32)
        cnt = C.c_int32(0)
        self.lib.xJPCG_gbGetSpmvTuning32(self.h, _ptr(ms), 64, C.byref(cnt))
        return [float(v) for v in ms[:cnt.value]]

    def set_spmv_lanes(self, lanes: int):
        st = self.lib.xJPCG_gbSetSpmvLanes(self.h, lanes)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())

    def set_spmv_config32(self, cfg: int):
        """Force the mixed solver's FP32 SpMV configuration (index of spmv_tuning(); -1: tuned)."""
        st = self.lib.xJPCG_gbSetSpmvConfig32(self.h, cfg)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())

    def diag_wait_timeout(self, budget_ns: int):
        """Failure-detection diagnostic (xJPCG_gbDiagWaitTimeout): a bounded
        device wait that nothing completes.  Returns (status, device status
        bits, wait duration in ns); status is INTERNAL_ERROR when the wait
        gave up, as a timed-out solve reports it."""
        dev, ns = C.c_uint32(0), C.c_uint64(0)
        st = self.lib.xJPCG_gbDiagWaitTimeout(self.h, budget_ns, C.byref(dev), C.byref(ns))
        return st, dev.value, ns.value

    def fp64_rate(self, iters: int = 16384):
        """FP64 issue-rate diagnostic (xJPCG_gbDiagFp64Rate): (DFMA per second
        over the whole GPU, best launch time in ms)."""
        rate, ms = C.c_double(0.0), C.c_double(0.0)
        st = self.lib.xJPCG_gbDiagFp64Rate(self.h, iters, C.byref(rate), C.byref(ms))
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
        return rate.value, ms.value

    def check_guards(self):
        """Memory-overrun diagnostic (xJPCG_gbDiagCheckGuards) of a handle
        created with XJPCG_GUARD_BYTES set: (status, buffers whose guard
        bytes changed)."""
        bad = C.c_uint32(0)
        st = self.lib.xJPCG_gbDiagCheckGuards(self.h, C.byref(bad))
        return st, bad.value

    def set_spmv_config(self, cfg: int):
        """Force the FP64 SpMV configuration with index cfg of spmv_tuning() (-1: tuned)."""
        st = self.lib.xJPCG_gbSetSpmvConfig(self.h, cfg)
        if st != SUCCESS:
            raise XJPCGError(st, self.last_message())
