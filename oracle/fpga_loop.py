"""The xJPCG loop in the reference FPGA's arithmetic order.

TEST INFRASTRUCTURE ONLY (part of the oracle): the checker of the library's
reference-order solve (xJPCG_gbSignatureSolve with summation order 1).
Nothing in hpc_gb300 imports it.

Every operation below is one IEEE double multiply, add or divide with
round-to-nearest, in the order the reference's C source writes them (numpy
elementwise ops, no fused multiply-add), so the result is the C semantics of
that source:

  init          pcg/sw/include/impl/cgVector.hpp:101-114: over the padded
                length n4 (diag padded with 1, b with 0): r = b, J = 1/diag,
                z = J * r, p = z, x = 0; bb and rz summed sequentially from 0
                (bb += b*b, rz += r*z, in index order).  Tols = (bb*tol)*tol
                (cgVector.hpp:149-155).
  SpMV          Ap = A p over the partitioned matrix in the FPGA order
                (oracle/sigdecode.py fpga_order_spmv: multAddX, regAcc,
                rowMemAcc, accY).
  dot, nrm2s    xf::blas::DotHelper<double, 2> (L1/blas/include/hw/blas/
                helpers/funcs/dotHelper.hpp:57-70, 139-152) and nrm2s
                (L1/hpc/include/hw/cgSolver/nrm2s.hpp:41-64): the products
                (each rounded) of every 4-entry group summed as a binary
                tree, (p0 + p1) + (p2 + p3) (BinarySum, helpers/utils/
                utils.hpp:39-54, via preProcess in sum.hpp:39-58); the group
                sums padded with zeros to a multiple of 8 (padding.hpp:55-67);
                every 8 of them summed as a binary tree (the delayed adder's
                shift register, postProcess in sum.hpp:60-82, AdderDelay<double>
                = 8, utils.hpp:98-102); those block sums added one after the
                other to a sum that starts at 0.  (The shift register holds
                the eight values in reverse; IEEE addition commutes, so the
                tree over them is the tree over the values in order.)
  alpha         rz / pAp (pcg/hw/src/krnl_storeApk.cpp:70).
  x, r          axpy (L1/blas/include/hw/blas/axpy.hpp:71): x = alpha*p + x,
                r = (-alpha)*Ap + r (update_xk.hpp, update_rk_jacobi.hpp:48).
  z             z = r * J (mul, update_rk_jacobi.hpp:50).
  rr, rz', beta nrm2s(r), dot(r, z), beta = rz' / rz (update_rk_jacobi.hpp:
                51-53, 100-102).
  p             p = beta*p + z (update_pk.hpp:33).
  stop          pcg/hw/include/control.hpp:83: go on while !(rr < Tols) and
                ++k < MaxIter, MaxIter = maxIter + 1; per iteration one
                record (Iter, Res = rr, RZ = rz', Alpha, Beta).

jpcg_fpga is the vectorised form (numpy); jpcg_fpga_literal spells the same
loops out one scalar at a time and pins it on small cases.
"""
from __future__ import annotations

import numpy as np

from . import sigdecode

PAR = 4    # CG_parEntries / CG_vecParEntries (pcg/hw/Makefile:103)
DELAY = 8  # AdderDelay<double>::m_Delays


def dot_fpga(a, b) -> float:
    """DotHelper<double, 2>::dot (b may be a for nrm2s): vectorised."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.size % PAR == 0 and a.size == b.size
    prod = (a * b).reshape(-1, PAR)
    g = (prod[:, 0] + prod[:, 1]) + (prod[:, 2] + prod[:, 3])
    pad = (-g.size) % DELAY
    if pad:
        g = np.concatenate([g, np.zeros(pad)])
    g8 = g.reshape(-1, DELAY)
    t = ((g8[:, 0] + g8[:, 1]) + (g8[:, 2] + g8[:, 3])) + ((g8[:, 4] + g8[:, 5]) + (g8[:, 6] + g8[:, 7]))
    # sequential accumulation from 0 (ufunc.accumulate adds left to right)
    return float(np.add.accumulate(np.concatenate([[0.0], t]))[-1])


def dot_fpga_literal(a, b) -> float:
    """DotHelper<double, 2>::dot written as the reference's loops: mul, then
    preProcess (BinarySum over 4), padding to a multiple of 8, then
    postProcess (a shift register of 8 filled by shift(), BinarySum over it,
    added to the final sum)."""
    n = len(a)
    groups = []
    for i in range(0, n, PAR):
        p = [float(a[i + j]) * float(b[i + j]) for j in range(PAR)]
        groups.append((p[0] + p[1]) + (p[2] + p[3]))
    total = (len(groups) + DELAY - 1) // DELAY * DELAY
    padded = [groups[i] if i < len(groups) else 0.0 for i in range(total)]
    final = 0.0
    for blk in range(0, total, DELAY):
        reg = [0.0] * DELAY
        for j in range(DELAY):  # WideType::shift: every value moves up one, the new one enters at 0
            reg = [padded[blk + j]] + reg[:-1]
        tree = ((reg[0] + reg[1]) + (reg[2] + reg[3])) + ((reg[4] + reg[5]) + (reg[6] + reg[7]))
        final += tree
    return final


def _init(n, diag, b):
    n4 = (n + PAR - 1) // PAR * PAR
    d = np.ones(n4)
    d[:n] = diag
    bb_ = np.zeros(n4)
    bb_[:n] = b
    r = bb_.copy()
    J = 1.0 / d
    z = J * r
    return n4, r, J, z


def jpcg_fpga(dec, n, diag, b, max_iter, tol, dim=None):
    """The loop over a decoded signature (oracle/sigdecode.decode_bytes) of an
    n x n matrix.  Returns dict(x, iters, res, k, records) with records an
    array of (iter, res, rz, alpha, beta) rows, slot i = iteration i."""
    n4, r, J, z = _init(n, diag, b)
    rows = max(n4, int(dec["row"].max()) + 1)
    p = z.copy()
    x = np.zeros(n4)
    bb = float(np.add.accumulate(np.concatenate([[0.0], r * r]))[-1])   # cgVector.hpp:109, in index order
    rz = float(np.add.accumulate(np.concatenate([[0.0], r * z]))[-1])   # cgVector.hpp:110
    tols = (bb * tol) * tol
    max_p1 = max_iter + 1
    recs = []
    k = 0
    rr = bb
    while True:
        pfull = np.zeros(max(rows, int(dec["col"].max()) + 1))
        pfull[:n4] = p
        Ap = sigdecode.fpga_order_spmv(dec, pfull, rows)[:n4]
        pAp = dot_fpga(p, Ap)
        alpha = rz / pAp
        x = alpha * p + x
        r = (-alpha) * Ap + r
        z = r * J
        rr = dot_fpga(r, r)
        rzn = dot_fpga(r, z)
        beta = rzn / rz
        rz = rzn
        p = beta * p + z
        recs.append((k, rr, rzn, alpha, beta))
        cont = not (rr < tols)
        k += 1
        cont = cont and k < max_p1
        if not (np.isfinite(alpha) and np.isfinite(beta) and np.isfinite(rr)):
            break
        if not cont:
            break
    rec = np.array(recs, dtype=[("iter", "<u4"), ("res", "<f8"), ("rz", "<f8"), ("alpha", "<f8"), ("beta", "<f8")])
    return {"x": x[:n], "iters": min(k, max_iter), "k": k, "res": float(np.sqrt(rr / bb)), "records": rec,
            "bb": bb, "tols": tols}


def jpcg_fpga_literal(dec, n, diag, b, max_iter, tol):
    """jpcg_fpga with every vector operation as a scalar loop (small cases)."""
    n4 = (n + PAR - 1) // PAR * PAR
    d = [float(diag[i]) if i < n else 1.0 for i in range(n4)]
    bv = [float(b[i]) if i < n else 0.0 for i in range(n4)]
    r = list(bv)
    J = [1.0 / d[i] for i in range(n4)]
    z = [J[i] * r[i] for i in range(n4)]
    p = list(z)
    x = [0.0] * n4
    bb = 0.0
    rz = 0.0
    for i in range(n4):
        bb += bv[i] * bv[i]
        rz += r[i] * z[i]
    tols = (bb * tol) * tol
    rows = max(n4, int(max(dec["row"])) + 1)
    recs = []
    k = 0
    rr = bb
    while True:
        Ap = list(sigdecode.fpga_order_spmv_literal(dec, p + [0.0] * 8, rows))[:n4]
        pAp = dot_fpga_literal(p, Ap)
        alpha = rz / pAp
        for i in range(n4):
            x[i] = alpha * p[i] + x[i]
            r[i] = (-alpha) * Ap[i] + r[i]
            z[i] = r[i] * J[i]
        rr = dot_fpga_literal(r, r)
        rzn = dot_fpga_literal(r, z)
        beta = rzn / rz
        rz = rzn
        for i in range(n4):
            p[i] = beta * p[i] + z[i]
        recs.append((k, rr, rzn, alpha, beta))
        k += 1
        if (rr < tols) or k >= max_iter + 1:
            break
    return {"x": np.array(x[:n]), "iters": min(k, max_iter), "k": k, "records": recs, "bb": bb}
