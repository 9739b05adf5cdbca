"""Generates the committed golden fixtures of the format conversion.

Runs the reference's own host partitioner (compiled from the Xilinx/HPC
sources by oracle/build_ref.sh into oracle/_ref/) on small matrices and stores,
per case, the inputs and what the reference produced:

  ref_sorted_{row,col,data}  SparseMatrix::loadCoo / loadCscSym + sort_by_row
                             (L2/sparse/include/sw/fp64/matrix_params.hpp)
  sig_{row,col,val,part}     every non-padding entry of the partitioned
                             matrix written by SpmPar::partitionCooMat /
                             partitionCscSymMat, decoded with oracle/sigdecode
                             and ordered (row, partition, position)
  sig_sha256                 SHA-256 of each signature file (rbParam, parParam,
                             info, nnzVal_0..15), for a byte-level exporter
  sig_raw_<file>             the signature files' bytes, for the cases whose
                             padded size is at most RAW_MAX_PADDED entries
  sig2_*                     the same after the values-only update
                             (updateMat / updateCscSymMat) when the case has one

Values are data[k] = k + 1, so a stored value names the input position it
came from.  Usage (in a container that has the reference tree):
    python tests/golden/make_golden.py <reference-root>
(or with XJPCG_REFERENCE_ROOT set).
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import sigdecode  # noqa: E402
from hpc_gb300 import workloads as W  # noqa: E402


def _coo_cases():
    rng = np.random.default_rng(2024)
    cases = []
    # 1. shuffled 7-point 6^3 with split duplicates, C base
    s = W.poisson7(6)
    r, c, _ = s.coo()
    p = rng.permutation(r.size)
    r, c = r[p], c[p]
    d = rng.choice(r.size, 20, replace=False)
    cases.append(("coo_shuffled_dups", s.n, np.concatenate([r, r[d]]), np.concatenate([c, c[d]]), 0, True))
    # 2. 27-point 5^3, Fortran base, row-major order
    s = W.diffusion27(5, seed=8)
    r, c, _ = s.coo()
    cases.append(("coo_fortran", s.n, r + 1, c + 1, 1, False))
    # 3. the reference example's COO emission order (example.c:132-151), n = 1000
    (er, ec, _), _, _, _, _, _ = _example(1000)
    cases.append(("coo_example_tridiag", 1000, er, ec, 0, True))
    # 4. banded + long-range entries over several 4096-row blocks and
    #    4096-column partitions, shuffled
    n = 9000
    rows = [np.arange(n), np.arange(1, n), np.arange(n - 1)]
    cols = [np.arange(n), np.arange(n - 1), np.arange(1, n)]
    lr = rng.integers(0, n, 6000)
    lc = rng.integers(0, n, 6000)
    rows += [lr, lc]
    cols += [lc, lr]
    r = np.concatenate(rows).astype(np.uint32)
    c = np.concatenate(cols).astype(np.uint32)
    p = rng.permutation(r.size)
    cases.append(("coo_blocks_9000", n, r[p], c[p], 0, True))
    return cases


def _example(n):
    coo, csc, diag, b1, b2, b3 = W.example_tridiagonal(n) if n == 65536 else _small_example(n)
    return coo, csc, diag, b1, b2, b3


def _small_example(n):
    rows, cols = [], []
    for i in range(n):
        if i != 0:
            rows.append(i); cols.append(i - 1)
        if i != n - 1:
            rows.append(i); cols.append(i + 1)
        rows.append(i); cols.append(i)
    ridx, cptr = [], []
    for i in range(n):
        cptr.append(2 * i + 1)
        if i != 0:
            ridx.append(i + 1)
        ridx.append(i + 1)
    cptr.append(len(ridx) + 1)
    return ((np.array(rows, np.uint32), np.array(cols, np.uint32), None),
            (np.array(ridx, np.int64), np.array(cptr, np.int64), None), None, None, None, None)


def _csc_cases():
    cases = []
    _, (ri, cp, _), _, _, _, _ = _small_example(1000)
    cases.append(("csc_example_fortran", 1000, ri, cp, 1, True))
    s = W.poisson7(8)
    r, c, _ = s.coo()
    low = r >= c
    r, c = r[low], c[low]
    order = np.lexsort((r, c))
    r, c = r[order].astype(np.int64), c[order]
    cp = np.zeros(s.n + 1, np.int64)
    np.cumsum(np.bincount(c, minlength=s.n), out=cp[1:])
    cases.append(("csc_poisson8_c", s.n, r, cp, 0, False))
    return cases


RAW_MAX_PADDED = 40000


def _sha(path):
    out = {}
    for f in sorted(os.listdir(path)):
        with open(os.path.join(path, f), "rb") as fh:
            out[f] = hashlib.sha256(fh.read()).hexdigest()
    return out


def _store_sig(prefix, path, rec):
    dec = sigdecode.decode(path)
    so = sigdecode.stored_order(dec)
    rec[prefix + "_row"] = so["row"].astype(np.uint32)
    rec[prefix + "_col"] = so["col"].astype(np.uint32)
    rec[prefix + "_val"] = so["val"]
    rec[prefix + "_part"] = so["part"].astype(np.uint32)
    rec[prefix + "_info"] = dec["info"]
    rec[prefix + "_padded"] = np.int64(dec["val"].size)
    sha = _sha(path)
    rec[prefix + "_sha256"] = np.array(["%s=%s" % kv for kv in sorted(sha.items())])
    if dec["val"].size <= RAW_MAX_PADDED:
        # raw signature bytes of the small cases, for the device-side decoder
        # and the byte-level exporter tests
        for f in sorted(os.listdir(path)):
            with open(os.path.join(path, f), "rb") as fh:
                rec[prefix + "_raw_" + f.replace(".dat", "")] = np.frombuffer(fh.read(), np.uint8)


def run(reference_root):
    harness = oracle.build_ref(reference_root)
    if harness is None:
        raise SystemExit("reference tree not found at %s" % reference_root)
    for name, n, r, c, base, with_update in _coo_cases():
        nnz = r.size
        data = np.arange(1, nnz + 1, dtype=np.float64)
        with tempfile.TemporaryDirectory() as d:
            with open(os.path.join(d, "meta.txt"), "w") as f:
                f.write("%d %d\n" % (n, nnz))
            r.astype(np.uint32).tofile(os.path.join(d, "row.bin"))
            c.astype(np.uint32).tofile(os.path.join(d, "col.bin"))
            data.tofile(os.path.join(d, "data.bin"))
            data2 = None
            if with_update:
                data2 = data * 10.0
                data2.tofile(os.path.join(d, "data2.bin"))
            subprocess.run([harness, "coo", d, str(base)], check=True)
            rec = {"kind": np.array("coo"), "n": np.int64(n), "base": np.int64(base), "row": r.astype(np.uint32),
                   "col": c.astype(np.uint32), "data": data}
            for k in ("row", "col", "data"):
                rec["ref_sorted_" + k] = np.fromfile(os.path.join(d, "ref_sorted_%s.bin" % k), np.uint32)
            _store_sig("sig", os.path.join(d, "sig"), rec)
            if with_update:
                rec["data2"] = data2
                _store_sig("sig2", os.path.join(d, "sig2"), rec)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        print(name, n, nnz, rec["sig_padded"])
    for name, n, ri, cp, base, with_update in _csc_cases():
        nnzh = ri.size
        data = np.arange(1, nnzh + 1, dtype=np.float64)
        with tempfile.TemporaryDirectory() as d:
            with open(os.path.join(d, "meta.txt"), "w") as f:
                f.write("%d %d\n" % (n, nnzh))
            ri.astype(np.int64).tofile(os.path.join(d, "rowidx.bin"))
            cp.astype(np.int64).tofile(os.path.join(d, "colptr.bin"))
            data.tofile(os.path.join(d, "data.bin"))
            data2 = None
            if with_update:
                data2 = data * 10.0
                data2.tofile(os.path.join(d, "data2.bin"))
            subprocess.run([harness, "csc", d, str(base)], check=True)
            rec = {"kind": np.array("csc"), "n": np.int64(n), "base": np.int64(base), "rowidx": ri, "colptr": cp,
                   "data": data}
            for k in ("row", "col", "data"):
                rec["ref_sorted_" + k] = np.fromfile(os.path.join(d, "ref_sorted_%s.bin" % k), np.uint32)
            _store_sig("sig", os.path.join(d, "sig"), rec)
            if with_update:
                rec["data2"] = data2
                _store_sig("sig2", os.path.join(d, "sig2"), rec)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **rec)
        print(name, n, nnzh, rec["sig_padded"])


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("XJPCG_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_golden.py <reference-root> (or set XJPCG_REFERENCE_ROOT)")
    run(root)
