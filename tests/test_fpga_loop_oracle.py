"""The oracle's restatement of the xJPCG loop in the reference FPGA's
arithmetic order (oracle/fpga_loop.py): the vectorised form pinned against
the literal loops of the reference source, bit for bit; and the loop checked
against the oracle's plain JPCG within the solver bar.  CPU only."""
import numpy as np
import pytest

import oracle
from hpc_gb300 import workloads as W
from oracle import fpga_loop as F
from oracle import sigdecode, sigexport


def _decoded(s):
    """The partitioned matrix of a workload system, written by the oracle's
    restatement of the reference partitioner and decoded again."""
    rows, cols, vals = s.coo()
    r, c = sigexport.coo_input(s.n, rows, cols)
    files = sigexport.export(sigexport.partition(s.n, s.n, r, c), vals)
    return sigdecode.decode_bytes(files["rbParam"], files["parParam"], [files["nnzVal_%d" % i] for i in range(16)])


@pytest.mark.parametrize("n4", [4, 8, 12, 32, 36, 100, 256, 1028])
def test_dot_matches_the_literal_delayed_adder(n4):
    rng = np.random.default_rng(n4)
    a = rng.standard_normal(n4) * 10.0 ** rng.integers(-8, 8, n4)
    b = rng.standard_normal(n4)
    assert F.dot_fpga(a, b) == F.dot_fpga_literal(a, b)
    assert F.dot_fpga(a, a) == F.dot_fpga_literal(a, a)


def test_dot_order_is_not_the_plain_sum():
    # 1 + 2^-53 + 2^-53 ... : a left-to-right sum loses every small term,
    # the 4-lane tree first pairs the small terms and keeps them.
    a = np.array([1.0, 0.0, 2.0 ** -53, 2.0 ** -53] * 2)
    b = np.ones_like(a)
    seq = 0.0
    for v in a * b:
        seq += v
    assert F.dot_fpga(a, b) == F.dot_fpga_literal(a, b) != seq


def _tridiagonal(n, seed):
    rp = np.zeros(n + 1, np.int32)
    cnt = np.full(n, 3)
    cnt[0] = cnt[-1] = 2
    rp[1:] = np.cumsum(cnt)
    col, val = [], []
    for i in range(n):
        for j in (i - 1, i, i + 1):
            if 0 <= j < n:
                col.append(j)
                val.append(2.2 if i == j else 1.0)
    b = np.random.default_rng(seed).uniform(-1, 1, n)
    return W.System(n, rp, np.array(col, np.int32), np.array(val), np.full(n, 2.2), b)


@pytest.mark.parametrize("case", ["tridiag_50", "poisson7_4"])
def test_vectorised_loop_equals_literal_loop(case):
    s = _tridiagonal(50, 3) if case == "tridiag_50" else W.poisson7(4, seed=5)
    dec = _decoded(s)
    v = F.jpcg_fpga(dec, s.n, s.diag, s.b, 200, 1e-10)
    lit = F.jpcg_fpga_literal(dec, s.n, s.diag, s.b, 200, 1e-10)
    assert v["k"] == lit["k"] and v["bb"] == lit["bb"]
    for got, want in zip(v["records"], lit["records"]):
        assert tuple(got) == tuple(want)
    assert v["x"].tobytes() == lit["x"].tobytes()


def test_fpga_order_loop_meets_the_solver_bar():
    s = W.poisson7(12, seed=6)
    dec = _decoded(s)
    v = F.jpcg_fpga(dec, s.n, s.diag, s.b, 2000, 1e-10)
    ref = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, 2000, 1e-10)
    assert abs(v["iters"] - ref["iters"]) <= max(1, 0.01 * ref["iters"])
    assert np.linalg.norm(v["x"] - ref["x"]) / np.linalg.norm(ref["x"]) <= 1e-8
    assert oracle.true_relres(s.rowptr, s.col, s.val, s.b, v["x"]) <= 1.5e-10
