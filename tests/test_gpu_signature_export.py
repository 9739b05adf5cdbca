"""The device signature exporter (xJPCG_gbExportSignature) against the
reference partitioner's own files (tests/golden/, SHA-256 of every file and
raw bytes of the small cases) and against the oracle's restatement
(oracle/sigexport.py) on larger random matrices: byte for byte, after the
partition and after a values-only update."""
from __future__ import annotations

import glob
import hashlib
import os

import numpy as np
import pytest

import hpc_gb300 as X
from oracle import sigexport as S

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _same(out, want_sha, raw=None):
    assert sorted(k + ".dat" for k in out) == sorted(want_sha)
    for k, buf in out.items():
        if raw is not None and k in raw:
            ref = raw[k]
            if buf != ref:
                a, b = np.frombuffer(buf, np.uint8), np.frombuffer(ref, np.uint8)
                m = min(a.size, b.size)
                first = int(np.flatnonzero(a[:m] != b[:m])[0]) if np.any(a[:m] != b[:m]) else m
                raise AssertionError("%s: %d vs %d bytes, first difference at byte %d" % (k, a.size, b.size, first))
        assert hashlib.sha256(buf).hexdigest() == want_sha[k + ".dat"], k


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_export_matches_reference_files(handle, path):
    g = np.load(path)
    n = int(g["n"])
    base = X.MODE_FORTRAN_INDEX if int(g["base"]) else 0
    ones = np.ones(n)
    if str(g["kind"]) == "coo":
        r = handle.coo_solve(n, g["row"], g["col"], g["data"], ones, ones, 0, 1e-10, mode=base)
    else:
        r = handle.csc_sym_solve(n, g["rowidx"], g["colptr"], g["data"], ones, ones, 0, 1e-10, mode=base)
    assert r.status in (X.SUCCESS, X.EXECUTION_FAILED), r.message
    for prefix in ("sig", "sig2"):
        if prefix + "_sha256" not in g.files:
            continue
        if prefix == "sig2":
            keep = X.MODE_KEEP_NZ_LAYOUT | base
            if str(g["kind"]) == "coo":
                r = handle.coo_solve(n, None, None, g["data2"], ones, ones, 0, 1e-10, mode=keep)
            else:
                r = handle.csc_sym_solve(n, g["rowidx"], g["colptr"], g["data2"], ones, ones, 0, 1e-10, mode=keep)
            assert r.status in (X.SUCCESS, X.EXECUTION_FAILED), r.message
        out = handle.export_signature()
        want = dict(s.split("=") for s in g[prefix + "_sha256"])
        raw = {k[len(prefix) + 5:]: g[k].tobytes() for k in g.files if k.startswith(prefix + "_raw_")}
        _same(out, want, raw)


def _random_case(seed, n, extra, gap_rows=0, wide=False):
    rng = np.random.default_rng(seed)
    rows = [np.arange(n)]
    cols = [np.arange(n)]
    rr = rng.integers(0, n, extra)
    span = n if wide else min(n, 9000)
    cc = np.clip(rr + rng.integers(-span, span + 1, extra), 0, n - 1)
    rows.append(rr)
    cols.append(cc)
    dup = rng.choice(extra, extra // 20, replace=False)  # duplicates
    rows.append(rr[dup])
    cols.append(cc[dup])
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    if gap_rows:
        # empty rows: drop every entry of a band of rows (diagonal included)
        lo = n // 3
        keep = (r < lo) | (r >= lo + gap_rows)
        r, c = r[keep], c[keep]
    p = rng.permutation(r.size)
    return r[p].astype(np.uint32), c[p].astype(np.uint32)


@pytest.mark.parametrize("case", [
    dict(seed=1, n=20000, extra=60000),
    dict(seed=2, n=30000, extra=90000, gap_rows=9000),
    dict(seed=3, n=50000, extra=150000, wide=True),
    dict(seed=4, n=4097, extra=3000),
])
def test_export_matches_oracle_random(handle, case):
    r, c = _random_case(**case)
    n = case["n"]
    rng = np.random.default_rng(case["seed"] + 100)
    data = rng.standard_normal(r.size)
    data[rng.choice(r.size, 50, replace=False)] = 0.0  # stored zeros stay stored
    ones = np.ones(n)
    res = handle.coo_solve(n, r, c, data, ones, ones, 0, 1e-10)
    assert res.status in (X.SUCCESS, X.EXECUTION_FAILED), res.message
    layout = S.partition(n, n, r.astype(np.int64), c.astype(np.int64))
    want = S.export(layout, data)
    out = handle.export_signature()
    for k in want:
        assert out[k] == want[k], k
    data2 = data * -3.0 + 1.0
    res = handle.coo_solve(n, None, None, data2, ones, ones, 0, 1e-10, mode=X.MODE_KEEP_NZ_LAYOUT)
    assert res.status in (X.SUCCESS, X.EXECUTION_FAILED), res.message
    want2 = S.export(layout, data2)
    out2 = handle.export_signature()
    for k in want2:
        assert out2[k] == want2[k], k


def test_store_signature_roundtrip(handle, tmp_path):
    # files written by the exporter load back through the SpmvHost drop-in
    # and give the same products as the stored matrix
    r, c = _random_case(seed=5, n=9000, extra=30000)
    n = 9000
    data = np.random.default_rng(6).standard_normal(r.size)
    handle.coo_solve(n, r, c, data, np.ones(n), np.ones(n), 0, 1e-10)
    x = np.random.default_rng(7).standard_normal(n)
    y_ref = handle.spmv(x)
    files = handle.store_signature(str(tmp_path))
    assert sorted(os.listdir(tmp_path)) == sorted(k + ".dat" for k in files)
    h2 = X.JPCG()
    try:
        bufs = [np.fromfile(os.path.join(tmp_path, "nnzVal_%d.dat" % i), np.uint8) for i in range(16)]
        par = np.fromfile(os.path.join(tmp_path, "parParam.dat"), np.uint8)
        rb = np.fromfile(os.path.join(tmp_path, "rbParam.dat"), np.uint8)
        h2.set_signature_matrix(bufs, par, rb)
        xp = np.zeros(-(-n // 4) * 4)
        xp[:n] = x
        y = h2.signature_spmv(xp, n)
        scale = np.abs(y_ref).max() + 1.0
        assert np.max(np.abs(y - y_ref)) <= 1e-12 * scale
    finally:
        h2.close()
