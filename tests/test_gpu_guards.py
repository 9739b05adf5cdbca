"""Memory-overrun check of every device path (the stand-in for a memory
checker, which this GPU pool does not offer).

A handle created with XJPCG_GUARD_BYTES allocates each of its device buffers
with guard bytes after the end.  One handle runs every SpMV configuration in
fp64 and FP32, the fp64, mixed, batched (every kernel shape, both
precisions), adjoint and edge-gradient paths, the COO, CSC and CSR entry
points with their reuse modes, the SpmvHost drop-in and the signature
exporter; then no guard byte may have changed (xJPCG_gbDiagCheckGuards)."""
import numpy as np
import pytest

import hpc_gb300 as X
from hpc_gb300 import workloads as W
import oracle

pytestmark = pytest.mark.gpu

GUARD = 4096


@pytest.fixture
def guarded(gpu_lib, monkeypatch):
    monkeypatch.setenv("XJPCG_GUARD_BYTES", str(GUARD))
    h = X.JPCG()
    yield h
    h.close()


def _every_config(h, s):
    h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    x = np.random.default_rng(1).standard_normal(s.n)
    yref = oracle.spmv(s.rowptr, s.col, s.val, x)
    scale = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
    ran = 0
    for c in range(len(h.spmv_tuning())):
        try:
            h.set_spmv_config(c)
        except X.XJPCGError:
            continue
        assert np.all(np.abs(h.spmv(x) - yref) <= 1e-13 * scale), c
        r = h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
        assert r.status == X.SUCCESS, (c, r.message)
        try:
            h.set_spmv_config32(c)
            m = h.mixed_solve(s.b, s.diag, 20000, 1e-10)
            assert m.status == X.SUCCESS, (c, m.message)
        except X.XJPCGError:
            pass
        ran += 1
    h.set_spmv_config(-1)
    h.set_spmv_config32(-1)
    return ran


def test_guards_intact_after_every_path(guarded, monkeypatch):
    h = guarded
    # every SpMV layout in both precisions, on a stencil and on power-law rows
    assert _every_config(h, W.diffusion27(14, seed=9)) >= 11
    assert _every_config(h, W.zipf_spd(30000, hi=1500, seed=5)) >= 11
    assert h.check_guards() == (X.SUCCESS, 0), h.last_message()

    # the reference entry points and their reuse modes
    s = W.poisson7(12)
    rows, cols, vals = s.coo()
    assert h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10).status == X.SUCCESS
    assert h.coo_solve(s.n, None, None, vals * 2.0, s.diag * 2.0, s.b, 2000, 1e-10,
                       mode=X.MODE_KEEP_NZ_LAYOUT).status == X.SUCCESS
    assert h.coo_solve(s.n, None, None, vals * 2.0, s.diag * 2.0, s.b * 0.5, 2000, 1e-10,
                       mode=X.MODE_KEEP_MATRIX).status == X.SUCCESS
    low = rows >= cols
    order = np.lexsort((rows[low], cols[low]))
    r_idx = rows[low][order].astype(np.int64)
    c_ptr = np.zeros(s.n + 1, np.int64)
    np.add.at(c_ptr, cols[low][order].astype(np.int64) + 1, 1)
    c_ptr = np.cumsum(c_ptr)
    assert h.csc_sym_solve(s.n, r_idx, c_ptr, vals[low][order], s.diag, s.b, 2000, 1e-10).status == X.SUCCESS
    h.records()
    assert h.check_guards() == (X.SUCCESS, 0), h.last_message()

    # batched: every kernel shape, both precisions
    batch = W.batched_stencils(count=24, lo=200, hi=3000, seed=3)
    for precision in (0, 1):
        for cfg in range(9):
            monkeypatch.setenv("XJPCG_BATCH_CFG", str(cfg))
            st, _, _ = h.batch_solve(batch, 20000, 1e-10, precision=precision)
            assert st == X.SUCCESS, (precision, cfg, h.last_message())
    monkeypatch.delenv("XJPCG_BATCH_CFG")
    assert h.check_guards() == (X.SUCCESS, 0), h.last_message()

    # adjoint solve and the per-edge gradient
    prob = W.adjoint_problem(12, seed=4)
    n = 12 ** 3
    ghost = W.ghost_diagonal7(prob.shape, prob.ghost)
    a = W.assemble_edges(n, prob.edge_i, prob.edge_j, np.exp(prob.theta), ghost)
    r = h.csr_solve(n, a.rowptr, a.col, a.val, a.diag, prob.b, 20000, 1e-12)
    assert r.status == X.SUCCESS
    st, lam, _, _, _ = h.adjoint(r.x - 1.0, a.diag, 20000, 1e-12)
    assert st == X.SUCCESS
    h.edge_grad(prob.edge_i, prob.edge_j, np.exp(prob.theta))
    assert h.check_guards() == (X.SUCCESS, 0), h.last_message()

    # the signature exporter and the SpmvHost drop-in on its buffers
    d = W.diffusion27(10, seed=2)
    h.csr_solve(d.n, d.rowptr, d.col, d.val, d.diag, d.b, 0, 1e-10)
    files = h.export_signature()
    bufs = [np.frombuffer(files["nnzVal_%d" % c], np.uint8) for c in range(16)]
    par = np.frombuffer(files["parParam"], np.uint8)
    rb = np.frombuffer(files["rbParam"], np.uint8)
    h.set_signature_matrix(bufs, par, rb)
    xp = np.zeros(-(-d.n // 4) * 4)
    xp[:d.n] = np.random.default_rng(2).standard_normal(d.n)
    for order in (0, 1):
        h.set_signature_sum_order(order)
        y = h.signature_spmv(xp, d.n)
        yref = oracle.spmv(d.rowptr, d.col, d.val, xp[:d.n])
        assert np.max(np.abs(y - yref)) <= 1e-12 * (np.abs(yref).max() + 1.0)
    h.set_signature_sum_order(0)
    assert h.check_guards() == (X.SUCCESS, 0), h.last_message()


def test_guards_off_is_refused(handle):
    # a handle created without guard bytes has nothing to check
    assert handle.check_guards()[0] == X.INVALID_VALUE
