"""The differentiable solve: x = A(theta)^-1 b on a 7-point diffusion matrix
with c_e = exp(theta_e), L = 0.5 ||x - x_obs||^2.  The adjoint (a second
solve, lambda = A^-1 (x - x_obs)) and the per-edge gradient kernel are
checked against fourth-order central finite differences on random unit
directions and
against an FP64 CPU reference gradient built from oracle solves; the per-nnz
dL/dA kernel against -lambda_i x_j on the host.  The solve is wrapped in a
torch.autograd.Function, as a user of the library would wrap it."""
import numpy as np
import pytest

import hpc_gb300 as X
import oracle
from hpc_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13


class Problem:
    """Fixed sparsity pattern of A(theta); only the values change with theta."""

    def __init__(self, nx, seed=4):
        self.prob = W.adjoint_problem(nx, seed=seed)
        self.n = nx ** 3
        self.ghost = W.ghost_diagonal7(self.prob.shape, self.prob.ghost)
        n, ei, ej = self.n, self.prob.edge_i.astype(np.int64), self.prob.edge_j.astype(np.int64)
        r = np.concatenate([ei, ej, np.arange(n)])
        c = np.concatenate([ej, ei, np.arange(n)])
        self.order = np.argsort(r * n + c, kind="stable")
        self.rowptr = np.zeros(n + 1, np.int64)
        np.cumsum(np.bincount(r, minlength=n), out=self.rowptr[1:])
        self.rowptr = self.rowptr.astype(np.int32)
        self.col = c[self.order].astype(np.int32)

    def system(self, theta):
        cond = np.exp(theta)
        ei, ej = self.prob.edge_i, self.prob.edge_j
        D = self.ghost + np.bincount(ei, cond, minlength=self.n) + np.bincount(ej, cond, minlength=self.n)
        v = np.concatenate([-cond, -cond, D])[self.order]
        return W.System(self.n, self.rowptr, self.col, v, D, self.prob.b)


def make_function(h, P):
    import torch

    class DiffSolve(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            th = theta.detach().cpu().numpy()
            s = P.system(th)
            r = h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, P.prob.b, 20000, TOL)
            assert r.status == X.SUCCESS, r.message
            ctx.c = np.exp(th)
            ctx.diag = s.diag
            return torch.from_numpy(r.x.copy())

        @staticmethod
        def backward(ctx, gx):
            st, lam, _, _, _ = h.adjoint(gx.detach().cpu().numpy(), ctx.diag, 20000, TOL)
            assert st == X.SUCCESS, h.last_message()
            g = h.edge_grad(P.prob.edge_i, P.prob.edge_j, ctx.c)
            return torch.from_numpy(g)

    return DiffSolve


def _loss(h, P, theta, x_obs):
    # the pattern is fixed: a values-only update (KEEP_NZ_LAYOUT) per direction
    s = P.system(theta)
    r = h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, P.prob.b, 20000, TOL, mode=X.MODE_KEEP_NZ_LAYOUT)
    assert r.status == X.SUCCESS, r.message
    return 0.5 * float(np.dot(r.x - x_obs, r.x - x_obs))


def _x_obs(h, P):
    s = P.system(P.prob.theta_obs)
    r = h.csr_solve(s.n, s.rowptr, s.col, s.val, s.diag, P.prob.b, 20000, TOL)
    assert r.status == X.SUCCESS
    return r.x.copy()


def _check(nx, ndirs, handle):
    import torch
    P = Problem(nx)
    x_obs = _x_obs(handle, P)
    F = make_function(handle, P)
    theta = torch.from_numpy(P.prob.theta.copy()).requires_grad_(True)
    x = F.apply(theta)
    loss = 0.5 * ((x - torch.from_numpy(x_obs)) ** 2).sum()
    loss.backward()
    grad = theta.grad.numpy()
    # FP64 CPU reference gradient from oracle solves
    s = P.system(P.prob.theta)
    xr = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, P.prob.b, 200000, TOL)["x"]
    lr = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, xr - x_obs, 200000, TOL)["x"]
    ei, ej = P.prob.edge_i, P.prob.edge_j
    gref = -np.exp(P.prob.theta) * (lr[ei] - lr[ej]) * (xr[ei] - xr[ej])
    assert np.linalg.norm(grad - gref) <= 1e-8 * np.linalg.norm(gref)
    # central finite differences on random unit directions
    rng = np.random.default_rng(7)
    hstep = 1e-3
    worst = 0.0
    for _ in range(ndirs):
        v = rng.standard_normal(ei.size)
        v /= np.linalg.norm(v)
        # fourth-order central difference: (8 (L(h) - L(-h)) - (L(2h) - L(-2h))) / 12h
        l1 = _loss(handle, P, P.prob.theta + hstep * v, x_obs) - _loss(handle, P, P.prob.theta - hstep * v, x_obs)
        l2 = (_loss(handle, P, P.prob.theta + 2 * hstep * v, x_obs)
              - _loss(handle, P, P.prob.theta - 2 * hstep * v, x_obs))
        fd = (8.0 * l1 - l2) / (12.0 * hstep)
        an = float(np.dot(grad, v))
        worst = max(worst, abs(fd - an) / max(abs(an), 1e-12 * np.linalg.norm(grad)))
    assert worst <= 1e-5, worst
    return worst


def test_adjoint_small_fd_and_reference(handle):
    _check(14, 16, handle)


def test_adjoint_dA_per_entry(handle):
    P = Problem(10)
    s = P.system(P.prob.theta)
    rows, cols, vals = s.coo()
    perm = np.random.default_rng(2).permutation(rows.size)  # unsorted COO input
    r = handle.coo_solve(s.n, rows[perm], cols[perm], vals[perm], s.diag, P.prob.b, 20000, TOL)
    assert r.status == X.SUCCESS
    g = np.random.default_rng(3).standard_normal(s.n)
    st, lam, ga, it, res = handle.adjoint(g, s.diag, 20000, TOL, grad_a=True)
    assert st == X.SUCCESS
    lr = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, g, 200000, TOL)["x"]
    assert np.linalg.norm(lam - lr) <= 1e-8 * np.linalg.norm(lr)
    expect = -lam[rows[perm]] * r.x[cols[perm]]
    assert np.allclose(ga, expect, rtol=1e-12, atol=0)


def test_adjoint_96_cubed_64_directions(handle):
    """The full workload: 96^3 grid, 2,626,560 edge parameters, 64 directions."""
    worst = _check(96, 64, handle)
    print("worst FD relative error over 64 directions: %.2e" % worst)
