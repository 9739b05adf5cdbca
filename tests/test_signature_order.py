"""The SpmvHost drop-in in the reference FPGA's summation order.

The oracle restates that order from the reference's HLS C source
(oracle/sigdecode.py fpga_order_spmv): products per group of 4 stored entries
summed left to right, runs of 8 groups summed left to right, each row's runs
in stream order, the channel sum.  On the CPU the vectorised oracle is pinned
against a literal loop restatement (bit for bit) and against the CSR SpMV
(within rounding); on the GPU the order-1 SpMV must give the oracle's bits.
The inputs are the reference partitioner's own buffers (tests/golden/) and
buffers this library exports.
"""
import glob
import os

import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from oracle import sigdecode
from hpc_gb300 import workloads as W

RAW = [p for p in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
       if "sig_raw_rbParam" in np.load(p).files]


def _load(path):
    z = np.load(path)
    nnz = [z["sig_raw_nnzVal_%d" % c] for c in range(16)]
    return z, nnz, z["sig_raw_parParam"], z["sig_raw_rbParam"]


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


@pytest.mark.parametrize("path", RAW, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_order_pinned(path):
    z, nnz, par, rb = _load(path)
    dec = sigdecode.decode_bytes(rb, par, nnz)
    n = int(z["n"])
    x = np.random.default_rng(2).standard_normal(int(dec["col"].max()) + 1)
    y = sigdecode.fpga_order_spmv(dec, x, n)
    assert np.array_equal(_bits(y), _bits(sigdecode.fpga_order_spmv_literal(dec, x, n)))
    # the same matrix in CSR order: equal within rounding
    keep = dec["val"] != 0
    m = max(n, int(dec["col"].max()) + 1)
    rp, ci, perm = oracle.coo_to_csr(m, dec["row"][keep].astype(np.uint32), dec["col"][keep].astype(np.uint32))
    vals = dec["val"][keep][perm]
    xm = np.zeros(m)
    xm[:x.size] = x
    yc = oracle.spmv(rp, ci, vals, xm)[:n]
    scale = oracle.spmv(rp, ci, np.abs(vals), np.abs(xm))[:n]
    assert np.all(np.abs(y - yc) <= 1e-13 * scale)


def test_oracle_order_is_not_csr_order():
    # cancellation that the FPGA grouping and a left-to-right row sum round
    # differently: the restatement must follow the grouping
    dec = {"val": np.zeros(32), "col": np.arange(32), "row": np.zeros(32, np.int64)}
    dec["val"][:5] = [1.0, 1e16, -1e16, 1.0, 1.0]
    x = np.ones(32)
    y = sigdecode.fpga_order_spmv(dec, x, 1)
    # group 0: ((1 + 1e16) - 1e16) + 1 = 1 (1 + 1e16 rounds to 1e16); group 1 adds 1
    assert y[0] == 2.0
    assert y[0] == sigdecode.fpga_order_spmv_literal(dec, x, 1)[0]


@pytest.mark.gpu
@pytest.mark.parametrize("path", RAW, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_reference_order_bitwise(handle, path):
    z, nnz, par, rb = _load(path)
    handle.set_signature_matrix(nnz, par, rb)
    dec = sigdecode.decode_bytes(rb, par, nnz)
    n = int(z["n"])
    npad = handle.info().n
    x = np.random.default_rng(3).standard_normal(npad)
    handle.set_signature_sum_order(1)
    y1, frame = handle.signature_spmv(x, n, start_addr=3, frame=True)
    yo = sigdecode.fpga_order_spmv(dec, x, n)
    assert np.array_equal(_bits(y1), _bits(yo))
    assert frame.tobytes() == sigdecode.transy_frame(3, n, y1)
    handle.set_signature_sum_order(0)
    y0 = handle.signature_spmv(x, n)
    scale = np.abs(yo) + 1e-300
    assert np.all(np.abs(y0 - yo) <= 1e-12 * np.maximum(scale, np.abs(x).max()))


@pytest.mark.gpu
def test_gpu_reference_order_exported(handle):
    # a larger matrix through this library's own exporter and back
    s = W.diffusion27(20, seed=21)
    handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    sig = handle.export_signature()
    u8 = lambda b: np.frombuffer(b, np.uint8)
    rb, par = u8(sig["rbParam"]), u8(sig["parParam"])
    nnz = [u8(sig["nnzVal_%d" % c]) for c in range(16)]
    h2 = X.JPCG()
    try:
        h2.set_signature_matrix(nnz, par, rb)
        h2.set_signature_sum_order(1)
        x = np.random.default_rng(4).standard_normal(h2.info().n)
        y = h2.signature_spmv(x, s.n)
        dec = sigdecode.decode_bytes(rb, par, nnz)
        assert np.array_equal(_bits(y), _bits(sigdecode.fpga_order_spmv(dec, x, s.n)))
        yref = oracle.spmv(s.rowptr, s.col, s.val, x[:s.n])
        scale = oracle.spmv(s.rowptr, s.col, np.abs(s.val), np.abs(x[:s.n]))
        assert np.all(np.abs(y - yref) <= 1e-13 * scale)
    finally:
        h2.close()


@pytest.mark.gpu
def test_gpu_reference_order_needs_signature_matrix(handle):
    s = W.poisson7(8)
    handle.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, s.b, 1, 1e-10)
    handle.set_signature_sum_order(1)
    with pytest.raises(X.XJPCGError) as e:
        handle.signature_spmv(np.ones(s.n), s.n)
    assert e.value.status == X.INVALID_VALUE
    with pytest.raises(X.XJPCGError):
        handle.set_signature_sum_order(2)
    handle.set_signature_sum_order(0)
    handle.signature_spmv(np.ones(s.n), s.n)
