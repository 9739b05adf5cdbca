"""An unchanged C application solving through the dlopen loader on the GPU:
the relink path of the reference's pcg_userGuide (-lXilinxPcg_loader -ldl)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from loader_util import LIBDIR, build_app, fields, run_app

pytestmark = pytest.mark.gpu


def test_loader_app_solves(tmp_path):
    from hpc_gb300 import build as B
    B.build_library()
    exe = build_app(str(tmp_path))
    n = 20000
    r = run_app(exe, ["solve", str(n)], LIBDIR)
    assert r.returncode == 0, r.stdout + r.stderr
    f = fields(r.stdout)
    assert f["status"] == "0" and f["metrics"] == "0" and f["peek"] == "0"
    assert float(f["res"]) <= 1e-10
    assert float(f["true"]) <= 1.5e-10
    # same system through the oracle: iteration count within 1 %
    rows = np.concatenate([np.arange(1, n), np.arange(n), np.arange(n - 1)])
    cols = np.concatenate([np.arange(n - 1), np.arange(n), np.arange(1, n)])
    vals = np.concatenate([-np.ones(n - 1), 4.0 * np.ones(n), -np.ones(n - 1)])
    rp, cc, perm = oracle.coo_to_csr(n, rows.astype(np.uint32), cols.astype(np.uint32), 0)
    ref = oracle.jpcg(rp, cc, vals[perm], np.full(n, 4.0), np.ones(n), 1000, 1e-10)
    assert abs(int(f["iter"]) - ref["iters"]) <= max(1, ref["iters"] // 100)
