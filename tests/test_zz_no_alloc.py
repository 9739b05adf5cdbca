"""The allocation-free SpMV + dot entry point (xJPCG_gbSpmvDotNoAlloc).

It exists for callers that cannot allocate device memory when they call: a
framework allocator may own the device memory, the caller may not synchronise
the device, or the caller may only own the buffers it was handed.  Its y must
match the oracle's CSR SpMV, and its dot the host FP64 dot of the oracle's y,
within the SpMV tolerance the other tests use, on two calls in a row (the
second call reuses the static scratch the first one left).  The handle-based
SpMV (xJPCG_gbSpmv) of the same matrix is checked beside it.

This file is named to be collected last, so a stop-at-first-failure run has
already run every other test when it gets here; it also passes alone in a
fresh process (the scratch is set up by its first call on the device).
"""
import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from hpc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MAX_ROWS = 524288  # the documented limit: 16384 tiles of 32 rows


def _tridiagonal(n):
    """SPD tridiagonal CSR (diag 2.2, off-diagonals 1.0, as in the reference's
    example), int32 row pointers and columns."""
    rp = np.zeros(n + 1, np.int32)
    counts = np.full(n, 3, np.int32)
    counts[0] = counts[-1] = 2
    rp[1:] = np.cumsum(counts)
    col = np.empty(int(rp[-1]), np.int32)
    val = np.empty(int(rp[-1]), np.float64)
    i = np.arange(n)
    for off, v in ((-1, 1.0), (0, 2.2), (1, 1.0)):
        ok = (i + off >= 0) & (i + off < n)
        rows = i[ok]
        slot = rp[rows] + (off + 1) - (rows == 0).astype(np.int32) * 1
        col[slot] = rows + off
        val[slot] = v
    return rp, col, val


def _check(n, rp, ci, va, x, y, dot):
    y_ref = oracle.spmv(rp, ci, va, x)  # the oracle's CSR SpMV
    scale_abs = oracle.spmv(rp, ci, np.abs(va), np.abs(x))
    assert np.all(np.abs(y - y_ref) <= 1e-13 * scale_abs)
    dot_ref = float(np.dot(x, y_ref))
    assert abs(dot - dot_ref) <= 1e-12 * float(np.dot(np.abs(x), scale_abs))
    return y_ref


def _call(n, d_rp, d_ci, d_v, d_x, d_y, d_dot, stream=0):
    st = X.spmv_dot_no_alloc(n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_x.data_ptr(), d_y.data_ptr(),
                             d_dot.data_ptr(), stream)
    assert st == X.SUCCESS


def test_no_alloc_spmv_dot_matches_oracle(gpu_lib):
    import torch

    s = W.diffusion27(50, seed=21)  # n = 125000 rows, within the 524288-row limit
    rows, cols, vals = s.coo()
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(s.rowptr).to(dev)
    d_ci = torch.from_numpy(s.col).to(dev)
    d_v = torch.from_numpy(s.val).to(dev)
    d_y = torch.empty(s.n, dtype=torch.float64, device=dev)
    d_dot = torch.empty(1, dtype=torch.float64, device=dev)
    with X.JPCG() as h:
        h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 0, 1e-10)  # store the same matrix in a handle
        for call in range(2):
            x = np.random.default_rng(100 + call).standard_normal(s.n)
            d_x = torch.from_numpy(x).to(dev)
            torch.cuda.synchronize()
            _call(s.n, d_rp, d_ci, d_v, d_x, d_y, d_dot)
            torch.cuda.synchronize()
            y = d_y.cpu().numpy()
            y_ref = _check(s.n, s.rowptr, s.col, s.val, x, y, float(d_dot.cpu().numpy()[0]))
            # the handle's SpMV of the same matrix, as a second check
            scale_abs = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
            assert np.all(np.abs(h.spmv(x) - y_ref) <= 1e-13 * scale_abs)


def test_no_alloc_at_the_row_limit_on_a_caller_stream(gpu_lib):
    """n = 524288 fills every partial sum of the static array exactly; the
    calls run on a caller-created stream, twice in a row."""
    import torch

    n = MAX_ROWS
    rp, ci, va = _tridiagonal(n)
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(rp).to(dev)
    d_ci = torch.from_numpy(ci).to(dev)
    d_v = torch.from_numpy(va).to(dev)
    d_y = torch.empty(n, dtype=torch.float64, device=dev)
    d_dot = torch.empty(1, dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(device=dev)
    for call in range(2):
        x = np.random.default_rng(300 + call).uniform(-1.0, 1.0, n)
        d_x = torch.from_numpy(x).to(dev)
        torch.cuda.synchronize()
        _call(n, d_rp, d_ci, d_v, d_x, d_y, d_dot, stream=side.cuda_stream)
        side.synchronize()
        _check(n, rp, ci, va, x, d_y.cpu().numpy(), float(d_dot.cpu().numpy()[0]))


def test_no_alloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    # 524289 rows would need one more partial sum than the static array holds;
    # the call refuses before launching, so the pointers are never touched.
    fake = 1 << 20
    assert X.spmv_dot_no_alloc(MAX_ROWS + 1, fake, fake, fake, fake, fake, fake) == X.INVALID_VALUE
    assert X.spmv_dot_no_alloc(0, fake, fake, fake, fake, fake, fake) == X.INVALID_VALUE
