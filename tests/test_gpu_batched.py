"""Batched JPCG (one persistent launch, per-system convergence) against the
oracle, system by system: fp64 with the xJPCG bar (iterations within 1 %,
x within 1e-8, true residual 1e-10) and the FP32-inner / FP64-refinement
form against a tight FP64 oracle solve."""
import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from hpc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    return W.batched_stencils(count=48, lo=200, hi=4000, seed=3)


def test_batched_fp64_matches_oracle(handle, batch):
    st, xs, res = handle.batch_solve(batch, 20000, 1e-10, precision=0)
    assert st == X.SUCCESS, handle.last_message()
    for s, x, r in zip(batch, xs, res):
        ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
        assert r["status"] == 0
        assert abs(int(r["iters"]) - ref["iters"]) <= max(1, int(0.01 * ref["iters"])), (r["iters"], ref["iters"])
        err = np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])
        assert err <= 1e-8, err
        assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, x) <= 1.5e-10
        assert r["res"] <= 1e-10


def test_batched_mixed_reaches_fp64_accuracy(handle, batch):
    st, xs, res = handle.batch_solve(batch, 20000, 1e-10, precision=1)
    assert st == X.SUCCESS, handle.last_message()
    for s, x, r in zip(batch, xs, res):
        rel = oracle.true_relres(s.rowptr, s.col, s.val, s.b, x)
        assert rel <= 1.5e-10, rel
        assert r["outer"] >= 1 and r["status"] == 0
        tight = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 200000, 1e-14)
        ref64 = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
        err = np.linalg.norm(x - tight["x"]) / np.linalg.norm(tight["x"])
        err64 = np.linalg.norm(ref64["x"] - tight["x"]) / np.linalg.norm(tight["x"])
        assert err <= max(10 * err64, 1e-9), (err, err64)
        # reliable updates keep the search direction: about the FP64 count
        assert int(r["iters"]) <= 1.25 * ref64["iters"] + 5, (int(r["iters"]), ref64["iters"])


def test_batched_maxiter_and_mask(handle, batch):
    # a cap of 5 iterations: every system stops on its own at the cap and
    # reports it the way xJPCG does (iters = maxIter, K = maxIter + 1)
    st, xs, res = handle.batch_solve(batch[:8], 5, 1e-10, precision=0)
    assert st == X.EXECUTION_FAILED
    for s, x, r in zip(batch[:8], xs, res):
        ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 5, 1e-10)
        assert int(r["iters"]) == ref["iters"] == 5 and int(r["itersRun"]) == ref["k"] == 6
        assert abs(r["res"] - ref["res"]) <= 1e-9 * ref["res"]


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_every_kernel_shape(handle, batch, precision, monkeypatch):
    # every kernel shape forced in turn (CSR with 1 or 2 lanes per row, and
    # the sliced kernels over the per-system SELL-32 copy) meets the bar
    sub = batch[:16]
    refs = [oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10) for s in sub]
    shapes = 0
    for cfg in range(9):
        monkeypatch.setenv("XJPCG_BATCH_CFG", str(cfg))
        st, xs, res = handle.batch_solve(sub, 20000, 1e-10, precision=precision)
        assert st == X.SUCCESS, (cfg, handle.last_message())
        shapes += handle.info().batchSliced
        for s, x, r, ref in zip(sub, xs, res, refs):
            assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, x) <= 1.5e-10
            if precision == 0:
                assert abs(int(r["iters"]) - ref["iters"]) <= max(1, int(0.01 * ref["iters"]))
                assert np.linalg.norm(x - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"])
    assert shapes == 3  # the three sliced shapes ran


def test_batched_rejects_bad_columns(handle, batch):
    bad = [W.System(s.n, s.rowptr, s.col.copy(), s.val, s.diag, s.b) for s in batch[:2]]
    bad[1].col[3] = bad[1].n  # outside its own system
    st, _, _ = handle.batch_solve(bad, 100, 1e-10)
    assert st == X.INVALID_VALUE


def _irregular_batch():
    """Systems whose 32-row slices cannot all share column offsets: rows with
    shuffled column order, a random banded SPD matrix with more than 8 offsets
    per slice, systems shorter than a slice or not a multiple of 32 rows, next
    to plain stencils whose first and last slices reach outside the system."""
    rng = np.random.default_rng(11)
    out = []
    st = W.batched_stencils(count=6, lo=300, hi=3000, seed=5)
    for k, s in enumerate(st):
        if k % 2 == 0:
            # the same matrix, each row's entries in a random order
            col, val = s.col.copy(), s.val.copy()
            for i in range(s.n):
                a, b = s.rowptr[i], s.rowptr[i + 1]
                p = rng.permutation(b - a)
                col[a:b], val[a:b] = col[a:b][p], val[a:b][p]
            s = W.System(s.n, s.rowptr, col, val, s.diag, s.b, s.name + "_shuffled")
        out.append(s)
    for n, band, dens in ((300, 24, 0.4), (17, 5, 0.6), (45, 9, 0.5), (97, 40, 0.2)):
        a = np.zeros((n, n))
        for i in range(n):
            for j in range(max(0, i - band), i):
                if rng.random() < dens:
                    a[i, j] = a[j, i] = rng.normal()
        np.fill_diagonal(a, np.abs(a).sum(1) * 1.05 + 0.5)
        rows, cols = np.nonzero(a)
        rowptr = np.zeros(n + 1, np.int32)
        np.add.at(rowptr, rows + 1, 1)
        rowptr = np.cumsum(rowptr).astype(np.int32)
        out.append(W.System(n, rowptr, cols.astype(np.int32), a[rows, cols], np.diag(a).copy(),
                            rng.uniform(-1, 1, n), "banded_%d" % n))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_sliced_irregular_slices(handle, precision, monkeypatch):
    # the sliced shapes on slices that fall back to per-entry columns (and on
    # the shared-offset slices beside them) meet the bar in both precisions
    sub = _irregular_batch()
    refs = [oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10) for s in sub]
    for cfg in (6, 7, 8):
        monkeypatch.setenv("XJPCG_BATCH_CFG", str(cfg))
        st, xs, res = handle.batch_solve(sub, 20000, 1e-10, precision=precision)
        assert st == X.SUCCESS, (cfg, handle.last_message())
        assert handle.info().batchSliced == 1
        for s, x, r, ref in zip(sub, xs, res, refs):
            assert r["status"] == 0, (cfg, s.name)
            assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, x) <= 1.5e-10, (cfg, s.name)
            if precision == 0:
                assert abs(int(r["iters"]) - ref["iters"]) <= max(1, int(0.01 * ref["iters"])), (cfg, s.name)
                assert np.linalg.norm(x - ref["x"]) <= 1e-8 * np.linalg.norm(ref["x"]), (cfg, s.name)


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_shared_offsets_same_bits(handle, precision, monkeypatch):
    # slices whose rows share column offsets store them once; every row then
    # sums the same products in the same order, with exact zeros between
    # them, so the solutions equal those of the per-entry layout bit for bit
    sub = W.batched_stencils(count=24, lo=200, hi=6000, seed=9) + _irregular_batch()
    # the sliced 512-thread shape with p in shared memory for every system (7),
    # and with p in global memory for the systems above 4,096 rows (16)
    for cfg in ("7", "16"):
        monkeypatch.setenv("XJPCG_BATCH_CFG", cfg)
        out = {}
        for pat in ("1", "0"):
            monkeypatch.setenv("XJPCG_BATCH_PATTERNS", pat)
            st, xs, res = handle.batch_solve(sub, 20000, 1e-10, precision=precision)
            assert st == X.SUCCESS, handle.last_message()
            assert handle.info().batchSliced == 1
            out[pat] = (xs, res)
        for a, b in zip(out["1"][0], out["0"][0]):
            assert np.array_equal(a, b), cfg
        assert np.array_equal(out["1"][1]["itersRun"], out["0"][1]["itersRun"]), cfg
