"""Parity of the CUDA JPCG path against the oracle, through the C ABI.

Bar (from the workload contract): true ||b - A x|| / ||b|| <= 1e-10,
||x - x_oracle|| / ||x_oracle|| <= 1e-8, iteration count within 1 % of the
oracle's; integer/index outputs (CSR conversion, iteration counters, record
fields) bit-exact.
"""
import os

import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from hpc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

X_TOL = 1e-8      # ||x - x_ref|| / ||x_ref||
RES_TOL = 1e-10   # true relative residual


def _check_solve(sysm, r, tol=1e-10, max_iter=20000):
    ref = oracle.jpcg(sysm.rowptr, sysm.col, sysm.val, sysm.diag, sysm.b, max_iter, tol)
    assert r.status == X.SUCCESS, r.message
    assert abs(r.iters - ref["iters"]) <= max(1, int(0.01 * ref["iters"])), (r.iters, ref["iters"])
    err = np.linalg.norm(r.x - ref["x"]) / np.linalg.norm(ref["x"])
    assert err <= X_TOL, err
    rel = oracle.true_relres(sysm.rowptr, sysm.col, sysm.val, sysm.b, r.x)
    assert rel <= RES_TOL * 1.5, rel
    assert r.res <= tol
    return ref


def test_poisson7_32_coo(handle):
    s = W.poisson7(32)
    rows, cols, vals = s.coo()
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10)
    _check_solve(s, r, max_iter=2000)


def test_diffusion27_small_csr(handle):
    s = W.diffusion27(20, sigma=1.5, seed=1)
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
    _check_solve(s, r)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8, 16, 32, -1, -2, -3, -5])
def test_every_spmv_shape_solves(handle, lanes):
    s = W.diffusion27(12, sigma=1.5, seed=7)
    rows, cols, vals = s.coo()
    handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 5, 1e-10)  # set the matrix
    handle.set_spmv_lanes(lanes)
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    if lanes > 0:
        assert handle.info().spmvLanes == lanes and handle.info().spmvLayout == 0
    else:
        assert handle.info().spmvLayout == {-1: 1, -2: 2, -3: 3, -5: 5}[lanes]
    _check_solve(s, r)


def test_narrow_sliced_columns_rejected_when_too_wide(handle):
    # one entry 40000 columns from its row: int16 offsets cannot hold it
    n = 50000
    rows = np.concatenate([np.arange(n), [0, 40000]]).astype(np.uint32)
    cols = np.concatenate([np.arange(n), [40000, 0]]).astype(np.uint32)
    vals = np.concatenate([np.full(n, 4.0), [-1.0, -1.0]])
    diag = np.full(n, 4.0)
    b = np.ones(n)
    r = handle.coo_solve(n, rows, cols, vals, diag, b, 100, 1e-10)
    assert r.status == X.SUCCESS
    with pytest.raises(X.XJPCGError) as e:
        handle.set_spmv_lanes(-3)
    assert e.value.status == X.INVALID_VALUE
    handle.set_spmv_lanes(-1)
    r = handle.coo_solve(n, rows, cols, vals, diag, b, 100, 1e-10, mode=X.MODE_KEEP_MATRIX)
    assert r.status == X.SUCCESS and handle.info().spmvLayout == 1


@pytest.mark.parametrize("n", [1, 31, 33, 1000, 40961])
def test_narrow_sliced_spmv_ragged(handle, n):
    # ragged last slice (rows past n read x[n-1] with value 0); every row holds
    # its diagonal and 5 random entries within 30000 columns, so slices are
    # nearly uniform (the sliced layout rejects heavy padding)
    rng = np.random.default_rng(n)
    w = min(n - 1, 30000)
    rows = np.repeat(np.arange(n), 5)
    cols = np.clip(rows + rng.integers(-w, w + 1, rows.size), 0, n - 1)
    rows = np.concatenate([np.arange(n), rows]).astype(np.uint32)
    cols = np.concatenate([np.arange(n), cols]).astype(np.uint32)
    vals = rng.standard_normal(rows.size)
    handle.coo_solve(n, rows, cols, vals, np.ones(n), np.ones(n), 1, 1e-10)
    rp, cc, vv, _ = handle.get_csr()
    x = rng.standard_normal(n)
    handle.set_spmv_lanes(-1)
    y32 = handle.spmv(x)
    handle.set_spmv_lanes(-3)
    y16 = handle.spmv(x)
    assert handle.info().spmvLayout == 3
    assert np.array_equal(y16, y32)  # same entries, same order
    yref = oracle.spmv(rp, cc, vv, x)
    scale = oracle.spmv(rp, cc, np.abs(vv), np.abs(x))
    assert np.all(np.abs(y16 - yref) <= 1e-13 * scale)


def test_conversion_bitexact_unsorted_fortran(handle):
    rng = np.random.default_rng(11)
    s = W.diffusion27(10, seed=3)
    rows, cols, vals = s.coo()
    # shuffle, add exact duplicates split in two, switch to 1-based
    perm = rng.permutation(rows.size)
    rows, cols, vals = rows[perm], cols[perm], vals[perm]
    dup = rng.choice(rows.size, 50, replace=False)
    half = vals[dup] / 2
    vals = vals.copy()
    vals[dup] = half
    rows = np.concatenate([rows, rows[dup]])
    cols = np.concatenate([cols, cols[dup]])
    vals = np.concatenate([vals, half])
    r = handle.coo_solve(s.n, rows + 1, cols + 1, vals, s.diag, s.b, 20000, 1e-10,
                         mode=X.MODE_DEFAULT | X.MODE_FORTRAN_INDEX)
    assert r.status == X.SUCCESS, r.message
    rp, ci, v, pm = handle.get_csr()
    orp, oci, opm = oracle.coo_to_csr(s.n, rows + 1, cols + 1, base=1)
    assert np.array_equal(rp, orp)
    assert np.array_equal(ci, oci)
    assert np.array_equal(pm, opm)
    assert np.array_equal(v, vals[opm])


def test_conversion_long_rows(handle):
    # rows longer than 32 and 4096 exercise the CTA sorters and multi-chunk SpMV
    rng = np.random.default_rng(12)
    n = 9000
    rows = [np.arange(n)]
    cols = [np.arange(n)]
    for r_, L in [(5, 6000), (77, 300), (4000, 40), (8999, 5000)]:
        c = rng.choice(n, L, replace=False)
        rows.append(np.full(L, r_))
        cols.append(c)
    rows = np.concatenate(rows).astype(np.uint32)
    cols = np.concatenate(cols).astype(np.uint32)
    perm = rng.permutation(rows.size)
    rows, cols = rows[perm], cols[perm]
    vals = rng.standard_normal(rows.size)
    diag = np.ones(n)
    b = rng.uniform(-1, 1, n)
    # A non-SPD matrix: only the conversion and the SpMV are checked.
    handle.coo_solve(n, rows, cols, vals, diag, b, 1, 1e-10)
    rp, ci, v, pm = handle.get_csr()
    orp, oci, opm = oracle.coo_to_csr(n, rows, cols)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci) and np.array_equal(pm, opm)
    x = rng.standard_normal(n)
    for lanes in [1, 4, 32, -2]:
        handle.set_spmv_lanes(lanes)
        y = handle.spmv(x)
        yref = oracle.spmv(orp, oci, vals[opm], x)
        scale = oracle.spmv(orp, oci, np.abs(vals[opm]), np.abs(x))
        assert np.all(np.abs(y - yref) <= 1e-13 * scale + 1e-300)


def test_cscsym_bitexact(handle):
    s = W.poisson7(12)
    A_rows, A_cols, A_vals = s.coo()
    lower = A_rows >= A_cols
    # lower triangle as CSC: column-major order of (row >= col) entries
    r, c, v = A_rows[lower], A_cols[lower], A_vals[lower]
    order = np.lexsort((r, c))
    r, c, v = r[order], c[order], v[order]
    colptr = np.zeros(s.n + 1, np.int64)
    np.cumsum(np.bincount(c, minlength=s.n), out=colptr[1:])
    for base in (0, 1):
        mode = X.MODE_DEFAULT | (X.MODE_FORTRAN_INDEX if base else 0)
        res = handle.csc_sym_solve(s.n, r.astype(np.int64) + base, colptr + base, v, s.diag, s.b, 2000, 1e-10,
                                   mode=mode)
        assert res.status == X.SUCCESS, res.message
        er, ec, ev = oracle.cscsym_expand(s.n, r.astype(np.int64) + base, colptr + base, v, base=base)
        orp, oci, opm = oracle.coo_to_csr(s.n, er, ec)
        rp, ci, vv, pm = handle.get_csr()
        assert np.array_equal(rp, orp) and np.array_equal(ci, oci) and np.array_equal(pm, opm)
        assert np.array_equal(vv, ev[opm])
        _check_solve(s, res, max_iter=2000)


@pytest.mark.parametrize("lanes", [0, 1, 2, 4, 8, 16, 32, -1, -2])
def test_spmv_matches_oracle(handle, lanes):
    s = W.diffusion27(24, seed=5)
    rows, cols, vals = s.coo()
    handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 1, 1e-10)
    handle.set_spmv_lanes(lanes)
    x = np.random.default_rng(1).standard_normal(s.n)
    y = handle.spmv(x)
    yref = oracle.spmv(s.rowptr, s.col, s.val, x)
    scale = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
    assert np.all(np.abs(y - yref) <= 1e-13 * scale)


def test_every_forced_config(handle, zipf_small):
    # every configuration of the tuner report, forced by index: the SpMV
    # matches the oracle and a solve through it meets the bar; a configuration
    # whose layout is not offered is refused and the previous choice stays
    for s in (W.diffusion27(12, seed=9), zipf_small):
        handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
        tuning = handle.spmv_tuning()
        x = np.random.default_rng(3).standard_normal(s.n)
        yref = oracle.spmv(s.rowptr, s.col, s.val, x)
        scale = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
        ran = 0
        for c in range(len(tuning)):
            before = handle.info().spmvCfg
            try:
                handle.set_spmv_config(c)
            except X.XJPCGError as e:
                assert e.status == X.INVALID_VALUE
                assert handle.info().spmvCfg == before
                continue
            assert handle.info().spmvCfg == c
            y = handle.spmv(x)
            assert np.all(np.abs(y - yref) <= 1e-13 * scale), c
            _check_solve(s, handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10,
                                             mode=X.MODE_KEEP_MATRIX))
            ran += 1
        assert ran >= 11  # the CSR, merge-path and one family of sliced kernels at least
        with pytest.raises(X.XJPCGError):
            handle.set_spmv_config(len(tuning))
        with pytest.raises(X.XJPCGError):
            handle.set_spmv_config(-2)
        handle.set_spmv_config(-1)


@pytest.mark.parametrize("nx", [30, 41])
def test_forced_fp32_config_same_bits(handle, nx):
    # the mixed solver's FP32 SpMV forced to each shared-offset form (unroll
    # 4 and 8; plain loads, TMA-fed values, or run-aware gathers that pass
    # consecutive offsets' x values by shuffle): none changes the values or
    # the order of a row's FMAs, so the mixed solves agree bit for bit; the
    # TMA-fed forms are FP32 only; a configuration index out of range is
    # refused.  The FP64 SpMV's run-aware forms give the plain forms' bits.
    s = W.diffusion27(nx, seed=14)
    handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    shapes = [t[:4] for t in handle.spmv_tuning()]
    cfgs = [shapes.index((1, 2, u, t)) for t in (0, 1, 2) for u in (4, 8)]
    with pytest.raises(X.XJPCGError):
        handle.set_spmv_config(cfgs[2])
    x = np.random.default_rng(5).standard_normal(s.n)
    ys = []
    for c in (cfgs[0], cfgs[1], cfgs[4], cfgs[5]):
        handle.set_spmv_config(c)
        ys.append(handle.spmv(x))
    for y in ys[1:]:
        assert np.array_equal(y, ys[0])
    handle.set_spmv_config(-1)
    out = []
    for c in cfgs:
        handle.set_spmv_config32(c)
        m = handle.mixed_solve(s.b, s.diag, 20000, 1e-10)
        assert m.status == X.SUCCESS and handle.info().spmvCfg32 == c
        out.append((m.iters, m.x.copy()))
    for it, xs in out[1:]:
        assert it == out[0][0] and np.array_equal(xs, out[0][1])
    assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, out[0][1]) <= RES_TOL * 1.5
    with pytest.raises(X.XJPCGError):
        handle.set_spmv_config32(len(shapes))
    handle.set_spmv_config32(-1)


@pytest.mark.parametrize("case", ["poisson7_24", "diffusion27_20", "zipf_30k"])
def test_pcgtest_flow_known_x(handle, case, zipf_small):
    # pcg/sw/tests/pcgtest.cpp:104-135 with pcg/sw/utils/genMat.py:38-98 data:
    # x = rand(n), b = A x, diag from the matrix; maxIter 5000, tol 1e-12
    # (runAllPcgTests.sh); a DEFAULT solve, then KEEP_NZ_LAYOUT re-solves.
    # pcgtest passes on zero mismatches of its compare against x, or when the
    # solve ran to maxIter.  A residual-based stop leaves components on tiny
    # diagonals loosely determined (the Zipf system scales rows by 10^+-3): the
    # oracle's own solve has the same mismatches there, so the bar is no more
    # mismatches than the oracle's, zero where the oracle has zero.
    s = {"poisson7_24": lambda: W.poisson7(24), "diffusion27_20": lambda: W.diffusion27(20, seed=15),
         "zipf_30k": lambda: zipf_small}[case]()
    rng = np.random.default_rng(16)
    x_true = rng.random(s.n)
    b = oracle.spmv(s.rowptr, s.col, s.val, x_true)
    ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, b, 5000, 1e-12)
    ref_bad = oracle.ref_mismatches(ref["x"], x_true)
    if case != "zipf_30k":
        assert ref_bad == 0
    rows, cols, vals = s.coo()
    for run in range(3):
        mode = X.MODE_DEFAULT if run == 0 else X.MODE_KEEP_NZ_LAYOUT
        r = handle.coo_solve(s.n, rows if run == 0 else None, cols if run == 0 else None, vals, s.diag, b,
                             5000, 1e-12, mode=mode, nnz=len(vals))
        assert r.status in (X.SUCCESS, X.EXECUTION_FAILED), r.message
        assert oracle.ref_mismatches(r.x, x_true) <= ref_bad or r.iters == 5000, (run, r.iters)
        assert abs(r.iters - ref["iters"]) <= max(1, int(0.01 * ref["iters"]))
        assert np.linalg.norm(r.x - ref["x"]) <= X_TOL * np.linalg.norm(ref["x"])


def test_spmv_gen_vectors_refvec(handle):
    # L2/sparse/tests/fp64/spmv/python/gen_vectors.py:43-67: refVec =
    # scipy coo.dot(x) with x = rand; the SpMV run passes on zero mismatches of
    # the reference's compare (main.cpp:180-190)
    sp = pytest.importorskip("scipy.sparse")
    s = W.diffusion27(18, seed=17)
    rows, cols, vals = s.coo()
    handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 1, 1e-10)
    x = np.random.default_rng(18).random(s.n)
    ref = sp.coo_matrix((vals, (rows, cols)), shape=(s.n, s.n)).dot(x)
    y = handle.spmv(x)
    assert oracle.ref_mismatches(y, ref) == 0
    assert np.allclose(y, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())


def test_tuning_reused_for_same_structure(handle):
    # a new matrix (MODE_DEFAULT) with the structure of the last tuned one keeps
    # its SpMV choice without timing again; another structure is timed anew
    s = W.diffusion27(24, seed=13)
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
    _check_solve(s, r)
    cfg, t1 = handle.info().spmvCfg, handle.info().tuneMs
    s2 = W.System(s.n, s.rowptr, s.col, s.val * 1.5, s.diag * 1.5, s.b)
    r = handle.csr_solve(s.n, s2.rowptr, s2.col, s2.val, s2.diag, s2.b, 20000, 1e-10)
    _check_solve(s2, r)
    assert handle.info().spmvCfg == cfg and handle.info().tuneMs < t1
    s3 = W.diffusion27(25, seed=13)
    r = handle.csr_solve(s3.n, s3.rowptr, s3.col, s3.val, s3.diag, s3.b, 20000, 1e-10)
    _check_solve(s3, r)
    assert min(t for t in (e[4] for e in handle.spmv_tuning()) if t > 0) > 0


def test_sliced_layout_follows_value_updates(handle):
    s = W.diffusion27(14, seed=6)
    rows, cols, vals = s.coo()
    handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 1, 1e-10)
    handle.set_spmv_lanes(-1)
    r = handle.coo_solve(s.n, None, None, vals * 3.0, s.diag * 3.0, s.b, 20000, 1e-10, mode=X.MODE_KEEP_NZ_LAYOUT)
    assert handle.info().spmvLayout == 1
    _check_solve(W.System(s.n, s.rowptr, s.col, s.val * 3.0, s.diag * 3.0, s.b), r)


def test_modes_and_reuse(handle):
    s = W.poisson7(16)
    rows, cols, vals = s.coo()
    # reuse modes on the first call are INVALID_VALUE (pcg.cpp:84-95, 141-152)
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 100, 1e-10, mode=X.MODE_KEEP_NZ_LAYOUT)
    assert r.status == X.INVALID_VALUE
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 100, 1e-10, mode=X.MODE_KEEP_MATRIX)
    assert r.status == X.INVALID_VALUE
    r1 = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10)
    assert r1.status == X.SUCCESS
    # KEEP_NZ_LAYOUT with NULL indices and scaled values (example.c:81-82)
    r2 = handle.coo_solve(s.n, None, None, vals * 2.0, s.diag * 2.0, s.b, 2000, 1e-10, mode=X.MODE_KEEP_NZ_LAYOUT)
    assert r2.status == X.SUCCESS, r2.message
    s2 = W.System(s.n, s.rowptr, s.col, s.val * 2.0, s.diag * 2.0, s.b)
    _check_solve(s2, r2, max_iter=2000)
    # KEEP_MATRIX with a new right-hand side
    b3 = np.random.default_rng(3).uniform(-1, 1, s.n)
    r3 = handle.coo_solve(s.n, None, None, None, s.diag * 2.0, b3, 2000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    assert r3.status == X.SUCCESS, r3.message
    s3 = W.System(s.n, s.rowptr, s.col, s.val * 2.0, s.diag * 2.0, b3)
    _check_solve(s3, r3, max_iter=2000)
    # wrong nnz on a values-only update -> INTERNAL_ERROR (checkUpdateDim)
    r4 = handle.coo_solve(s.n, None, None, vals[:-1], s.diag, s.b, 10, 1e-10, nnz=vals.size - 1,
                          mode=X.MODE_KEEP_NZ_LAYOUT)
    assert r4.status == X.INTERNAL_ERROR


def test_argument_errors(handle):
    s = W.poisson7(8)
    rows, cols, vals = s.coo()
    assert handle.coo_solve(0, rows, cols, vals, s.diag, s.b, 10, 1e-10).status == X.INVALID_VALUE
    assert handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 10, 1e-10, nnz=0).status == X.INVALID_VALUE
    assert handle.coo_solve(s.n, rows, cols, None, s.diag, s.b, 10, 1e-10).status == X.INVALID_VALUE
    assert handle.coo_solve(s.n, None, cols, vals, s.diag, s.b, 10, 1e-10).status == X.INVALID_VALUE
    bad = rows.copy()
    bad[3] = s.n
    r = handle.coo_solve(s.n, bad, cols, vals, s.diag, s.b, 10, 1e-10)
    assert r.status == X.INVALID_VALUE
    r = handle.coo_solve(s.n, rows, cols, vals, None, s.b, 10, 1e-10)
    assert r.status == X.INVALID_VALUE and "Vector is nullptr" in r.message
    assert handle.last_status() == X.INVALID_VALUE
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 10, 1e-10, mode=0x20)
    assert r.status == X.INTERNAL_ERROR


def test_maxiter_cap_and_records(handle):
    s = W.diffusion27(12, seed=9)
    rows, cols, vals = s.coo()
    for max_iter in (0, 1, 7):
        r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, max_iter, 1e-10)
        ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, max_iter, 1e-10, records=True)
        assert r.status == X.EXECUTION_FAILED
        assert r.iters == ref["iters"] == max_iter
        assert handle.info().itersRun == ref["k"] == max_iter + 1
        assert abs(r.res - ref["res"]) <= 1e-9 * ref["res"]
        recs = handle.records()
        assert len(recs) == ref["k"] + 1
        orec = ref["records"][:len(recs)]
        for f in ("id", "iter", "vecSize", "maxIter"):
            assert np.array_equal(recs[f], orec[f]), f
        for f in ("tols", "res", "rz", "alpha", "beta"):
            assert np.allclose(recs[f], orec[f], rtol=1e-9, atol=0), f


def test_records_converged(handle):
    s = W.poisson7(16)
    rows, cols, vals = s.coo()
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10)
    ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 2000, 1e-10, records=True)
    recs = handle.records()
    assert r.status == X.SUCCESS
    assert len(recs) == r.iters + 1
    assert recs["maxIter"][0] == 2001 and np.all(recs["maxIter"][1:] == 2001)
    assert np.array_equal(recs["iter"][1:], np.arange(r.iters))
    k = min(len(recs), ref["k"] + 1)
    assert np.allclose(recs["res"][:k][:20], ref["records"]["res"][:k][:20], rtol=1e-8)


def test_bitwise_determinism(handle):
    s = W.diffusion27(16, seed=2)
    rows, cols, vals = s.coo()
    a = handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 20000, 1e-10)
    b = handle.coo_solve(s.n, None, None, None, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    assert a.status == b.status == X.SUCCESS
    assert a.iters == b.iters and np.array_equal(a.x, b.x)


def test_example_known_answer(handle):
    """The reference example's three solves (pcg/sw/examples/c/example.c)."""
    n = 65536
    (r, c, d), (ri, cp, cd), diag, b1, b2, b3 = W.example_tridiagonal(n)
    res1 = handle.coo_solve(n, r, c, d, diag, b1, 100, 1e-16)
    assert res1.status == X.SUCCESS, res1.message
    rp, ci, pm = oracle.coo_to_csr(n, r, c)
    ref1 = oracle.jpcg(rp, ci, d[pm], diag, b1, 100, 1e-16)
    assert abs(res1.iters - ref1["iters"]) <= 1
    assert np.linalg.norm(res1.x - ref1["x"]) / np.linalg.norm(ref1["x"]) <= X_TOL
    res2 = handle.coo_solve(n, None, None, d, diag, b2, 100, 1e-16, mode=X.MODE_KEEP_NZ_LAYOUT)
    assert res2.status == X.SUCCESS, res2.message
    ref2 = oracle.jpcg(rp, ci, d[pm], diag, b2, 100, 1e-16)
    assert np.linalg.norm(res2.x - ref2["x"]) / np.linalg.norm(ref2["x"]) <= X_TOL
    res3 = handle.csc_sym_solve(n, ri, cp, cd, diag, b3, 100, 1e-16,
                                mode=X.MODE_DEFAULT | X.MODE_FORTRAN_INDEX)
    assert res3.status == X.SUCCESS, res3.message
    ref3 = oracle.jpcg(rp, ci, d[pm], diag, b3, 100, 1e-16)
    assert abs(res3.iters - ref3["iters"]) <= 1
    assert np.linalg.norm(res3.x - ref3["x"]) / np.linalg.norm(ref3["x"]) <= X_TOL


def test_host_loop_matches_graph_loop(gpu_lib):
    # The SpMV shape is pinned so both handles sum in the same order (the
    # tuner could otherwise pick different shapes on timing noise).
    s = W.poisson7(16)
    rows, cols, vals = s.coo()
    os.environ["XJPCG_SPMV_LANES"] = "4"
    with X.JPCG() as h:
        a = h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10)
        assert h.info().loopMode == 1
    os.environ["XJPCG_HOST_LOOP"] = "1"
    try:
        with X.JPCG() as h:
            b = h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10)
            assert h.info().loopMode == 0
    finally:
        del os.environ["XJPCG_HOST_LOOP"]
        del os.environ["XJPCG_SPMV_LANES"]
    assert a.iters == b.iters and np.array_equal(a.x, b.x)


def test_fused_and_separate_vector_kernels_agree(gpu_lib):
    """The fp64 iteration's vector work runs as one cooperative launch (the
    default) or as the update and p-update kernels (XJPCG_FUSED_UPDATE=0).
    Both meet the oracle's bar, in the graph loop and the host loop, and the
    mixed solver beside them too; the per-element arithmetic is the same,
    only the order of the r.r / r.z sums differs."""
    s = W.diffusion27(24, seed=12)
    ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
    os.environ["XJPCG_SPMV_LANES"] = "-1"
    out = {}
    try:
        for fused in ("1", "0"):
            for host in ("0", "1"):
                os.environ["XJPCG_FUSED_UPDATE"] = fused
                os.environ["XJPCG_HOST_LOOP"] = host
                with X.JPCG() as h:
                    r = h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
                    m = h.mixed_solve(s.b, s.diag, 20000, 1e-10)  # the mixed loop's FP32 update
                assert r.status == X.SUCCESS, r.message
                assert abs(r.iters - ref["iters"]) <= max(1, 0.01 * ref["iters"])
                assert np.linalg.norm(r.x - ref["x"]) / np.linalg.norm(ref["x"]) <= X_TOL
                assert m.status == X.SUCCESS, m.message
                assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, m.x) <= 1.5e-10
                assert np.linalg.norm(m.x - ref["x"]) / np.linalg.norm(ref["x"]) <= X_TOL
                out[fused, host] = r
    finally:
        for k in ("XJPCG_SPMV_LANES", "XJPCG_FUSED_UPDATE", "XJPCG_HOST_LOOP"):
            os.environ.pop(k, None)
    for fused in ("1", "0"):  # graph and host loops launch the same kernels: same bits
        a, b = out[fused, "0"], out[fused, "1"]
        assert a.iters == b.iters and np.array_equal(a.x, b.x)


@pytest.mark.parametrize("lanes", ["-3", "-2"])
def test_mixed_host_loop_matches_graph_loop(gpu_lib, lanes):
    # the mixed solver's host-driven loop (used under profilers) runs the
    # graph's kernels with self-skipping refresh kernels: same iterates
    s = W.diffusion27(14, seed=9)
    os.environ["XJPCG_SPMV_LANES"] = lanes
    try:
        with X.JPCG() as h:
            h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
            a = h.mixed_solve(s.b, s.diag, 20000, 1e-10)
            ia = h.info()
            assert ia.loopMode == 1
        os.environ["XJPCG_HOST_LOOP"] = "1"
        with X.JPCG() as h:
            h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
            b = h.mixed_solve(s.b, s.diag, 20000, 1e-10)
            ib = h.info()
            assert ib.loopMode == 0
    finally:
        os.environ.pop("XJPCG_HOST_LOOP", None)
        del os.environ["XJPCG_SPMV_LANES"]
    assert a.status == X.SUCCESS and b.status == X.SUCCESS
    assert a.iters == b.iters and ia.outerSweeps == ib.outerSweeps
    assert a.res == b.res and np.array_equal(a.x, b.x)


def test_zero_rhs_breakdown(handle):
    s = W.poisson7(8)
    rows, cols, vals = s.coo()
    r = handle.coo_solve(s.n, rows, cols, vals, s.diag, np.zeros(s.n), 50, 1e-10)
    # b = 0 makes alpha = 0/0; the loop stops at that iteration instead of
    # running to maxIter on NaN.
    assert r.status == X.EXECUTION_FAILED
    assert handle.info().itersRun == 1


def test_wait_timeout_reported_and_context_usable(handle):
    # failure detection without a fault: the library's bounded mbarrier wait
    # on a barrier that nothing completes gives up after its budget (5 ms
    # here, 2 s in the kernels), the host reports it as a timed-out solve
    # does, and the same handle then solves normally
    s = W.poisson7(16)
    r0 = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 2000, 1e-10)
    st, dev, ns = handle.diag_wait_timeout(5_000_000)
    assert st == X.INTERNAL_ERROR
    assert handle.last_message() == "INTERNAL ERROR: Run kernel failed: a device wait timed out."
    assert dev == 2  # kStatusWaitTimeout
    assert 5_000_000 <= ns < 1_000_000_000
    for bad in (0, 2_000_000_000):
        assert handle.diag_wait_timeout(bad)[0] == X.INVALID_VALUE
    r1 = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 2000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    assert r1.status == X.SUCCESS and r1.iters == r0.iters
    assert np.array_equal(r1.x, r0.x)


@pytest.mark.parametrize("fault", ["alloc", "launch"])
def test_host_fault_injection(monkeypatch, fault):
    # XJPCG_FAULT, read when a handle is created, injects on the host the
    # failures the C ABI maps to ALLOC_FAILED (a device allocation fails) and
    # INTERNAL_ERROR (a solver launch fails before anything is queued); no GPU
    # work faults.  A handle created without it then solves normally.
    s = W.poisson7(8)
    rows, cols, vals = s.coo()
    monkeypatch.setenv("XJPCG_FAULT", fault)
    h = X.JPCG()
    try:
        r = h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 100, 1e-10)
        if fault == "alloc":
            assert r.status == X.ALLOC_FAILED
            assert "device allocation failed for" in h.last_message()
        else:
            assert r.status == X.INTERNAL_ERROR
            assert "graph launch" in h.last_message() and "launch failure" in h.last_message()
            assert h.mixed_solve(s.b, s.diag, 100, 1e-10).status == X.INTERNAL_ERROR
            assert h.batch_solve([s, s], 100, 1e-10)[0] == X.INTERNAL_ERROR
    finally:
        h.close()
    monkeypatch.delenv("XJPCG_FAULT")
    h = X.JPCG()
    try:
        _check_solve(s, h.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10))
    finally:
        h.close()


def test_nan_rhs_stops_with_execution_failed(handle):
    # a NaN in b makes alpha NaN at the first iteration: the loop stops there
    # with EXECUTION_FAILED instead of running to maxIter
    s = W.poisson7(8)
    b = s.b.copy()
    b[5] = np.nan
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, b, 50, 1e-10)
    assert r.status == X.EXECUTION_FAILED
    assert handle.info().itersRun == 1


@pytest.mark.parametrize("lanes", [0, -2])
def test_power_law_rows_merge_path(handle, lanes):
    """Zipf rows (4 .. 4096+ entries): SpMV and a solve with the merge-path
    kernel against the oracle."""
    s = W.zipf_spd(60000, seed=5)
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 0, 1e-10)
    handle.set_spmv_lanes(lanes)
    x = np.random.default_rng(4).standard_normal(s.n)
    y = handle.spmv(x)
    yref = oracle.spmv(s.rowptr, s.col, s.val, x)
    scale = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
    assert np.all(np.abs(y - yref) <= 1e-13 * scale)
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    _check_solve(s, r)
    m = handle.mixed_solve(s.b, s.diag, 20000, 1e-10)
    assert m.status == X.SUCCESS, m.message
    assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, m.x) <= 1.5e-10


def test_mixed_precision_small(handle):
    s = W.zipf_spd(20000, seed=2)
    r64 = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10)
    assert r64.status == X.SUCCESS, r64.message
    m = handle.mixed_solve(s.b, s.diag, 20000, 1e-10)
    assert m.status == X.SUCCESS, m.message
    rel = oracle.true_relres(s.rowptr, s.col, s.val, s.b, m.x)
    assert rel <= 1e-10 * 1.5, rel
    tight = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 200000, 1e-14)
    err = np.linalg.norm(m.x - tight["x"]) / np.linalg.norm(tight["x"])
    err64 = np.linalg.norm(r64.x - tight["x"]) / np.linalg.norm(tight["x"])
    assert err <= max(10 * err64, 1e-8), (err, err64)
    assert handle.info().outerSweeps >= 1


@pytest.fixture(scope="module")
def zipf_small():
    # power-law rows (4 .. 1500 entries): the plain sliced layout pads too
    # much, so the length-sorted sliced layout is offered
    return W.zipf_spd(30000, hi=1500, seed=5)


def test_sorted_sliced_spmv_and_solve(handle, zipf_small):
    s = zipf_small
    handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    handle.set_spmv_lanes(-4)
    assert handle.info().spmvLayout == 4
    x = np.random.default_rng(3).standard_normal(s.n)
    y = handle.spmv(x)
    yref = oracle.spmv(s.rowptr, s.col, s.val, x)
    scale = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x))
    assert np.all(np.abs(y - yref) <= 1e-13 * scale)
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    _check_solve(s, r)
    # the mixed solver follows the forced layout for its FP32 SpMV
    m = handle.mixed_solve(s.b, s.diag, 20000, 1e-10)
    assert m.status == X.SUCCESS and handle.info().spmvLayout32 == 4
    assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, m.x) <= 1e-10


def test_sorted_sliced_deterministic_across_handles(zipf_small):
    s = zipf_small
    out = []
    for _ in range(2):
        h = X.JPCG()
        try:
            h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
            h.set_spmv_lanes(-4)
            r = h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
            out.append((r.iters, r.x.copy()))
        finally:
            h.close()
    assert out[0][0] == out[1][0]
    assert np.array_equal(out[0][1], out[1][1])


def test_sorted_sliced_not_offered_for_uniform_rows(handle):
    s = W.diffusion27(10, seed=2)
    handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    with pytest.raises(X.XJPCGError):
        handle.set_spmv_lanes(-4)
    handle.set_spmv_lanes(0)


@pytest.mark.parametrize("nx", [9, 40])
def test_shared_offset_layout_bitwise_equals_sliced(handle, nx):
    # slices whose rows share the stencil's offsets store them once; boundary
    # rows get explicit zeros in offset order, so every row sums in its CSR
    # order exactly as the plain sliced kernel does
    s = W.diffusion27(nx, seed=11)
    handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    x = np.random.default_rng(nx).standard_normal(s.n)
    handle.set_spmv_lanes(-1)
    y1 = handle.spmv(x)
    handle.set_spmv_lanes(-5)
    y5 = handle.spmv(x)
    assert handle.info().spmvLayout == 5
    assert np.array_equal(y1, y5)
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 20000, 1e-10, mode=X.MODE_KEEP_MATRIX)
    _check_solve(s, r)
    # values-only update keeps the layout and refreshes its values
    r = handle.csr_solve(s.n, s.rowptr, s.col, s.val * 2.0, s.diag * 2.0, s.b, 20000, 1e-10,
                         mode=X.MODE_KEEP_NZ_LAYOUT)
    assert handle.info().spmvLayout == 5
    _check_solve(W.System(s.n, s.rowptr, s.col, s.val * 2.0, s.diag * 2.0, s.b), r)
    m = handle.mixed_solve(s.b, s.diag * 2.0, 20000, 1e-10)
    assert m.status == X.SUCCESS and handle.info().spmvLayout32 == 5
    handle.set_spmv_lanes(0)
