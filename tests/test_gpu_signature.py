"""The SpmvHost drop-in: the reference's own partitioned-matrix buffers
(committed raw bytes from its host partitioner, tests/golden/) loaded onto the
GPU, decoded, and multiplied.  The stored matrix must hold exactly the
reference's non-padding entries in its order, y must match the oracle SpMV,
and the transY frame must match the oracle's restatement byte for byte."""
import glob
import os

import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from oracle import sigdecode

pytestmark = pytest.mark.gpu

RAW = [p for p in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
       if "sig_raw_rbParam" in np.load(p).files]


def _bufs(g, prefix="sig"):
    nnz = [g["%s_raw_nnzVal_%d" % (prefix, c)] for c in range(16)]
    return nnz, g[prefix + "_raw_parParam"], g[prefix + "_raw_rbParam"]


@pytest.mark.parametrize("path", RAW, ids=lambda p: os.path.basename(p)[:-4])
def test_signature_matrix_matches_reference(handle, path):
    z = np.load(path)
    g = {k: z[k] for k in z.files}
    nnz, par, rb = _bufs(g)
    handle.set_signature_matrix(nnz, par, rb)
    rp, ci, v, _ = handle.get_csr()
    n = int(g["n"])
    rows = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    assert np.array_equal(rows, g["sig_row"].astype(np.int64))
    assert np.array_equal(ci, g["sig_col"].astype(np.int32))
    assert np.array_equal(v, g["sig_val"])
    # y = A x for the rows the reference stores, plus the transY frame
    npad = rp.size - 1
    x = np.random.default_rng(8).standard_normal(npad)
    y, frame = handle.signature_spmv(x, n, start_addr=7, frame=True)
    yref = oracle.spmv(rp, ci, v, x)[:n]
    scale = oracle.spmv(rp, ci, np.abs(v), np.abs(x))[:n]
    assert np.all(np.abs(y - yref) <= 1e-13 * scale)
    assert frame.tobytes() == sigdecode.transy_frame(7, n, y)
    if "sig2_raw_rbParam" in g:
        nnz2, par2, rb2 = _bufs(g, "sig2")
        handle.set_signature_matrix(nnz2, par2, rb2)
        _, _, v2, _ = handle.get_csr()
        assert np.array_equal(v2, g["sig2_val"])
