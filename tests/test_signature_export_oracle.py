"""The oracle's restatement of the signature writer (oracle/sigexport.py)
pinned against the files the reference's own partitioner wrote
(tests/golden/*.npz, made by tests/golden/make_golden.py): every file of
every case byte-identical (SHA-256), after the partition and after the
values-only update."""
from __future__ import annotations

import glob
import hashlib
import os

import numpy as np
import pytest

from oracle import sigexport as S

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def _inputs(d):
    n, base = int(d["n"]), int(d["base"])
    if str(d["kind"]) == "coo":
        r, c = S.coo_input(n, d["row"], d["col"], base)
        return n, r, c, d["data"], (d["data2"] if "data2" in d.files else None)
    r, c, v = S.cscsym_input(n, d["rowidx"], d["colptr"], d["data"], base)
    v2 = S.cscsym_input(n, d["rowidx"], d["colptr"], d["data2"], base)[2] if "data2" in d.files else None
    return n, r, c, v, v2


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_signature_bytes(path):
    d = np.load(path)
    n, r, c, v, v2 = _inputs(d)
    layout = S.partition(n, n, r, c)
    for prefix, vals in (("sig", v), ("sig2", v2)):
        if prefix + "_sha256" not in d.files:
            continue
        out = S.export(layout, vals)
        want = dict(s.split("=") for s in d[prefix + "_sha256"])
        assert sorted(k + ".dat" for k in out) == sorted(want)
        for k, buf in out.items():
            assert hashlib.sha256(buf).hexdigest() == want[k + ".dat"], (prefix, k)
            raw = prefix + "_raw_" + k
            if raw in d.files:
                assert buf == d[raw].tobytes()
