"""The allocation-free SpMV + dot entry point (xJPCG_gbSpmvDotNoAlloc).

It exists for callers that cannot allocate device memory when they call: a
framework allocator may own the device memory, the caller may not synchronise
the device, or the caller may only own the buffers it was handed.  Its result
must equal what the handle-based SpMV (xJPCG_gbSpmv) returns for the same
matrix and vector, within the SpMV tolerance the other tests use, on two calls
in a row (the second call reuses the static scratch the first one left).

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


def test_no_alloc_spmv_dot_matches_handle_spmv(gpu_lib):
    import torch

    s = W.diffusion27(50, seed=21)  # n = 125000 rows, within the 524288-row limit
    rows, cols, vals = s.coo()
    dev = torch.device("cuda", 0)
    d_rp = torch.from_numpy(s.rowptr).to(dev)
    d_ci = torch.from_numpy(s.col).to(dev)
    d_v = torch.from_numpy(s.val).to(dev)
    d_y = torch.empty(s.n, dtype=torch.float64, device=dev)
    d_dot = torch.empty(1, dtype=torch.float64, device=dev)
    scale_abs = None
    with X.JPCG() as h:
        h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 0, 1e-10)  # store the same matrix in a handle
        for call in range(2):
            x = np.random.default_rng(100 + call).standard_normal(s.n)
            d_x = torch.from_numpy(x).to(dev)
            torch.cuda.synchronize()
            st = X.spmv_dot_no_alloc(s.n, d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), d_x.data_ptr(),
                                     d_y.data_ptr(), d_dot.data_ptr())
            assert st == X.SUCCESS
            torch.cuda.synchronize()
            y = d_y.cpu().numpy()
            dot = float(d_dot.cpu().numpy()[0])
            y_ref = h.spmv(x)                       # the existing entry point
            scale_abs = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
            assert np.all(np.abs(y - y_ref) <= 1e-13 * scale_abs)
            dot_ref = float(np.dot(x, y_ref))
            assert abs(dot - dot_ref) <= 1e-12 * float(np.dot(np.abs(x), scale_abs))


def test_no_alloc_rejects_sizes_beyond_its_scratch(gpu_lib):
    # 524289 rows would need one more partial sum than the static array holds;
    # the call refuses before launching, so the pointers are never touched.
    fake = 1 << 20
    assert X.spmv_dot_no_alloc(524289, fake, fake, fake, fake, fake, fake) == X.INVALID_VALUE
    assert X.spmv_dot_no_alloc(0, fake, fake, fake, fake, fake, fake) == X.INVALID_VALUE
