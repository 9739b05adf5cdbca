"""The whole JPCG loop in the reference FPGA's arithmetic order on the GPU
(xJPCG_gbSignatureSolve, summation order 1) against the oracle's restatement
of that order (oracle/fpga_loop.py, pinned against the literal loops of the
reference source on the CPU): equal iteration counts, every per-iteration
record (r.r, r.z, alpha, beta) bit for bit, and x bit for bit.  The matrix is
the reference partitioner's layout of the system, as this library exports it
(byte-identical to the reference's own files, tests/test_gpu_signature_export.py)
and loads it back.  Cases: the reference example's tridiagonal system
(pcg/sw/examples/c/example.c, n = 65536, maxIter 100, tol 1e-16), a 7-point
12^3 system, and the 7-point 32^3 system of the first benchmark configuration
(142 iterations)."""
import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from hpc_gb300 import workloads as W
from oracle import fpga_loop, sigdecode

pytestmark = pytest.mark.gpu

X_TOL = 1e-8


def _partitioned(n, rows, cols, vals, diag, b):
    """The reference partition of the matrix, exported by the library."""
    with X.JPCG() as h:
        r = h.coo_solve(n, rows, cols, vals, diag, b, 0, 1e-10)  # stores the matrix (maxIter 0)
        assert r.status in (X.SUCCESS, X.EXECUTION_FAILED)
        return h.export_signature()


def _cases():
    n = 65536
    (r, c, d), _, diag, b1, _, _ = W.example_tridiagonal(n)
    yield "example_tridiag", n, r, c, d, diag, b1, 100, 1e-16
    s = W.poisson7(12, seed=9)
    rows, cols, vals = s.coo()
    yield "poisson7_12", s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10
    # the contract's first configuration: 7-point 32^3, shift 1e-3, b from seed 0
    s = W.poisson7(32, seed=0)
    rows, cols, vals = s.coo()
    yield "poisson7_32", s.n, rows, cols, vals, s.diag, s.b, 2000, 1e-10


@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_reference_order_loop_bit_for_bit(gpu_lib, case):
    name, n, rows, cols, vals, diag, b, max_iter, tol = case
    files = _partitioned(n, rows, cols, vals, diag, b)
    nnz_bufs = [np.frombuffer(files["nnzVal_%d" % c], np.uint8) for c in range(16)]
    par = np.frombuffer(files["parParam"], np.uint8)
    rb = np.frombuffer(files["rbParam"], np.uint8)
    dec = sigdecode.decode_bytes(files["rbParam"], files["parParam"], [files["nnzVal_%d" % c] for c in range(16)])
    ref = fpga_loop.jpcg_fpga(dec, n, diag, b, max_iter, tol)
    with X.JPCG() as h:
        h.set_signature_matrix(nnz_bufs, par, rb)
        h.set_signature_sum_order(1)
        got = h.signature_solve(b, diag, max_iter, tol)
        assert got.status == X.SUCCESS, got.message
        recs = h.records()
        k = h.info().itersRun
    assert got.iters == ref["iters"] and k == ref["k"]
    assert recs[0]["res"] == ref["bb"] and recs[0]["tols"] == ref["tols"]
    for i, want in enumerate(ref["records"]):
        rec = recs[i + 1]
        assert rec["iter"] == want["iter"]
        for f in ("res", "rz", "alpha", "beta"):
            assert rec[f] == want[f], (i, f, rec[f], want[f])
    assert got.x.tobytes() == ref["x"].tobytes()
    assert got.res == float(np.sqrt(ref["records"][-1]["res"] / ref["bb"]))
    # and the loop meets the solver bar against the oracle's plain JPCG
    rp, ci, pm = oracle.coo_to_csr(n, rows, cols)
    plain = oracle.jpcg(rp, ci, vals[pm], diag, b, max_iter, tol)
    assert abs(got.iters - plain["iters"]) <= max(1, 0.01 * plain["iters"])
    assert np.linalg.norm(got.x - plain["x"]) / np.linalg.norm(plain["x"]) <= X_TOL


def test_signature_solve_tuned_order_meets_the_bar(gpu_lib):
    s = W.poisson7(12, seed=9)
    rows, cols, vals = s.coo()
    files = _partitioned(s.n, rows, cols, vals, s.diag, s.b)
    with X.JPCG() as h:
        h.set_signature_matrix([np.frombuffer(files["nnzVal_%d" % c], np.uint8) for c in range(16)],
                               np.frombuffer(files["parParam"], np.uint8), np.frombuffer(files["rbParam"], np.uint8))
        got = h.signature_solve(s.b, s.diag, 2000, 1e-10)  # order 0: the tuned solver
        assert got.status == X.SUCCESS, got.message
    ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 2000, 1e-10)
    assert abs(got.iters - ref["iters"]) <= max(1, 0.01 * ref["iters"])
    assert np.linalg.norm(got.x - ref["x"]) / np.linalg.norm(ref["x"]) <= X_TOL


def test_signature_solve_needs_a_partitioned_matrix(handle):
    s = W.poisson7(4)
    rows, cols, vals = s.coo()
    handle.coo_solve(s.n, rows, cols, vals, s.diag, s.b, 10, 1e-10)
    got = handle.signature_solve(s.b, s.diag, 10, 1e-10)
    assert got.status == X.INVALID_VALUE
