"""The SpMV host classes on the GPU: tests/c/spmv_host_app.cpp replays the
reference's SpMV test sequence (L2/sparse/tests/fp64/spmv/main.cpp:71-191)
with SpmvHost<16> on the reference partitioner's own files (committed raw
bytes, tests/golden/), then the dSpmv compute -> transY frame -> store round
trip with two compute cards.  The application checks the reference test's
own tolerance and the round trip bit for bit; here y is also held against the
oracle's CSR SpMV within the SpMV bar of the other tests."""
import glob
import os
import subprocess

import numpy as np
import pytest

import oracle
from spmv_host_util import build_app, write_case

pytestmark = pytest.mark.gpu

RAW = [p for p in sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
       if "sig_raw_rbParam" in np.load(p).files]


@pytest.fixture(scope="module")
def app(tmp_path_factory, gpu_lib):
    return build_app(str(tmp_path_factory.mktemp("spmv_host")))


@pytest.mark.parametrize("path", RAW, ids=lambda p: os.path.basename(p)[:-4])
def test_spmv_host_sequence_and_dspmv_round_trip(app, path, tmp_path):
    z = np.load(path)
    g = {k: z[k] for k in z.files}
    info = np.frombuffer(np.asarray(g["sig_raw_info"], np.uint8).tobytes(), np.int32, 6)
    m, n_pad = int(info[0]), int(info[4])
    # the reference's stored entries (padding dropped), as CSR for the oracle
    rows = g["sig_row"].astype(np.uint32)
    cols = g["sig_col"].astype(np.uint32)
    vals = g["sig_val"].astype(np.float64)
    dim = max(n_pad, m, int(rows.max()) + 1, int(cols.max()) + 1)
    rp, ci, perm = oracle.coo_to_csr(dim, rows, cols)
    va = vals[perm]
    x = np.random.default_rng(11).uniform(-1.0, 1.0, n_pad)
    xf = np.zeros(dim)
    xf[:n_pad] = x
    y_ref = oracle.spmv(rp, ci, va, xf)[:m]
    scale = oracle.spmv(rp, ci, np.abs(va), np.abs(xf))[:m]
    sig_dir, vec_dir = str(tmp_path / "sig"), str(tmp_path / "vec")
    write_case(g, sig_dir, vec_dir, x, y_ref)
    out = subprocess.run([app, sig_dir, vec_dir, "0"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    assert "INFO: Test pass!" in out.stdout
    y = np.fromfile(os.path.join(vec_dir, "outVec.dat"), np.float64)
    assert y.size == m
    assert np.all(np.abs(y - y_ref) <= 1e-13 * scale)
