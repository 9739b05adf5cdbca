"""Seeded synthetic systems for the xJPCG workloads.

The reference benchmarks on SuiteSparse matrices that are downloaded at run
time (pcg/sw/utils/genMat.py); none are available here, so these generators
stand in for them with the shapes, sizes and value distributions of the five
workloads this library is measured on.  Every generator uses
``numpy.random.default_rng(seed)`` and draws in the order its docstring states,
so a workload is a pure function of its parameters.

All return CSR with int32 row pointers / columns (columns ascending inside a
row), the matrix diagonal (the Jacobi diagonal handed to the solver) and b.
"""
from __future__ import annotations

import ctypes
import ctypes.util
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np


@dataclass
class System:
    n: int
    rowptr: np.ndarray  # int32[n+1]
    col: np.ndarray     # int32[nnz]
    val: np.ndarray     # float64[nnz]
    diag: np.ndarray    # float64[n]
    b: np.ndarray       # float64[n]
    name: str = ""

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])

    def coo(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Row-major COO (uint32 rows / cols) of the same matrix."""
        rows = np.repeat(np.arange(self.n, dtype=np.uint32), np.diff(self.rowptr))
        return rows, self.col.astype(np.uint32), self.val


def _grid_dirs(ndim: int) -> List[Tuple[int, ...]]:
    """All non-zero offsets in {-1,0,1}^ndim, lexicographic."""
    g = np.stack(np.meshgrid(*([np.array([-1, 0, 1])] * ndim), indexing="ij"), -1).reshape(-1, ndim)
    return [tuple(int(v) for v in d) for d in g if any(d)]


def _slices(shape, d):
    """(source, destination) slices of the sub-box where p and p+d are both in the grid."""
    src, dst = [], []
    for L, o in zip(shape, d):
        src.append(slice(max(0, -o), L - max(0, o)))
        dst.append(slice(max(0, o), L - max(0, -o)))
    return tuple(src), tuple(dst)


def stencil_system(shape, offsets, pair_cond, ghost_cond, diag_shift=0.0, rng=None, b=None, name="") -> System:
    """Assembles A = sum_e c_e (e_i - e_j)(e_i - e_j)^T + diag(ghost + shift).

    shape      grid extents, slowest first (z, y, x)
    offsets    the stencil's neighbour offsets (each d and -d present)
    pair_cond  dict d -> conductance array over the valid sub-box of d, for the
               "forward" half of the offsets (d > 0 lexicographically)
    ghost_cond array over the grid added to the diagonal (Dirichlet ghosts)
    """
    ndim = len(shape)
    n = int(np.prod(shape))
    strides = [int(np.prod(shape[i + 1:])) for i in range(ndim)]
    offs = sorted(offsets, key=lambda d: sum(o * s for o, s in zip(d, strides)))
    zero = tuple([0] * ndim)
    offs_all = sorted(offs + [zero], key=lambda d: sum(o * s for o, s in zip(d, strides)))
    S = len(offs_all)
    slot = {d: i for i, d in enumerate(offs_all)}
    vals = np.zeros(shape + (S,), np.float64)
    valid = np.zeros(shape + (S,), bool)
    D = np.asarray(ghost_cond, np.float64).reshape(shape).copy() + diag_shift
    for d, c in pair_cond.items():
        src, dst = _slices(shape, d)
        nd = tuple(-o for o in d)
        vals[src + (slot[d],)] = -c
        valid[src + (slot[d],)] = True
        vals[dst + (slot[nd],)] = -c
        valid[dst + (slot[nd],)] = True
        D[src] += c
        D[dst] += c
    vals[..., slot[zero]] = D
    valid[..., slot[zero]] = True
    vals = vals.reshape(n, S)
    valid = valid.reshape(n, S)
    lin = np.array([sum(o * s for o, s in zip(d, strides)) for d in offs_all], np.int64)
    counts = valid.sum(1)
    rowptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=rowptr[1:])
    cols = (np.arange(n, dtype=np.int64)[:, None] + lin[None, :])[valid].astype(np.int32)
    v = vals[valid]
    return System(n, rowptr.astype(np.int32), cols, v, D.reshape(n).copy(), b, name)


def poisson7(nx: int = 32, shift: float = 1e-3, seed: int = 0) -> System:
    """3D 7-point Dirichlet Laplacian (diag 6, off -1) + shift*I on nx^3.

    Draws: b ~ U[-1, 1] (n values).  32^3 gives n = 32768, nnz = 223232.
    """
    rng = np.random.default_rng(seed)
    shape = (nx, nx, nx)
    offs = [d for d in _grid_dirs(3) if sum(abs(o) for o in d) == 1]
    fwd = [d for d in offs if d > (0, 0, 0)]
    pair = {}
    for d in fwd:
        src, _ = _slices(shape, d)
        pair[d] = np.ones(tuple(s.stop - s.start for s in src))
    # Dirichlet ghosts with conductance 1 make every diagonal exactly 6.
    ghost = np.zeros(shape)
    for d in offs:
        src, _ = _slices(shape, d)
        m = np.ones(shape, bool)
        m[src] = False
        ghost[m] += 1.0
    sysm = stencil_system(shape, offs, pair, ghost, diag_shift=shift, name="poisson7_%d" % nx)
    sysm.b = rng.uniform(-1.0, 1.0, sysm.n)
    return sysm


def diffusion27(nx: int = 160, sigma: float = 1.5, seed: int = 1) -> System:
    """3D 27-point variable-coefficient diffusion on nx^3.

    Draws, in order: for each of the 13 forward directions d (lexicographic
    (dz,dy,dx) > 0), one log-normal(0, sigma) conductance per pair (p, p+d),
    pairs in lexicographic order of p; then, for each of the 26 directions
    (lexicographic), one log-normal(0, sigma) Dirichlet ghost conductance per
    point p whose neighbour p+d lies outside the grid, points in lexicographic
    order; then b ~ U[-1, 1].  160^3 gives n = 4096000, nnz = 478^3.
    """
    rng = np.random.default_rng(seed)
    shape = (nx, nx, nx)
    offs = _grid_dirs(3)
    fwd = [d for d in offs if d > (0, 0, 0)]
    pair = {}
    for d in fwd:
        src, _ = _slices(shape, d)
        pair[d] = rng.lognormal(0.0, sigma, tuple(s.stop - s.start for s in src))
    ghost = np.zeros(shape)
    for d in offs:
        src, _ = _slices(shape, d)
        m = np.ones(shape, bool)
        m[src] = False
        cnt = int(m.sum())
        ghost[m] += rng.lognormal(0.0, sigma, cnt)
    sysm = stencil_system(shape, offs, pair, ghost, name="diffusion27_%d" % nx)
    sysm.b = rng.uniform(-1.0, 1.0, sysm.n)
    return sysm


def zipf_spd(n: int = 2_000_000, alpha: float = 1.8, lo: int = 4, hi: int = 4096, seed: int = 2) -> System:
    """Random SPD matrix with Zipf row lengths, symmetrically scaled.

    Draws, in order: row lengths L ~ Zipf(alpha) clipped to [lo, hi]; sum(L)
    uniform columns; one N(0,1) value per distinct unordered off-diagonal pair
    (pairs in ascending (min, max) order; self pairs and repeats dropped);
    d_i = 10^U(-3, 3); b ~ U[-1, 1].  A0 = W + diag(1.01 sum_j |w_ij|),
    A = D A0 D with D = diag(d).
    """
    import scipy.sparse as sps

    rng = np.random.default_rng(seed)
    L = np.clip(rng.zipf(alpha, n), lo, hi).astype(np.int64)
    rows = np.repeat(np.arange(n, dtype=np.int64), L)
    cols = rng.integers(0, n, size=int(L.sum()), dtype=np.int64)
    keep = rows != cols
    key = np.minimum(rows, cols)[keep] * n + np.maximum(rows, cols)[keep]
    del rows, cols, keep
    key = np.sort(key)  # sorted distinct pairs (np.unique is much slower here)
    first = np.empty(key.size, bool)
    first[:1] = True
    np.not_equal(key[1:], key[:-1], out=first[1:])
    key = key[first]
    del first
    pa = key // n
    pb = key - pa * n
    del key
    w = rng.standard_normal(pa.size)
    d = 10.0 ** rng.uniform(-3.0, 3.0, n)
    absw = np.abs(w)
    diag0 = 1.01 * (np.bincount(pa, absw, minlength=n) + np.bincount(pb, absw, minlength=n))
    diag0[diag0 == 0] = 1.0
    ar = np.arange(n, dtype=np.int64)
    A = sps.csr_matrix((np.concatenate([w, w, diag0]),
                        (np.concatenate([pa, pb, ar]), np.concatenate([pb, pa, ar]))), shape=(n, n))
    del pa, pb, w
    A.sort_indices()
    rowptr = A.indptr.astype(np.int64)
    c = A.indices.astype(np.int64)
    r = np.repeat(ar, np.diff(rowptr))
    v = A.data * d[r] * d[c]
    del A, r
    diag = diag0 * d * d
    b = rng.uniform(-1.0, 1.0, n)
    return System(n, rowptr.astype(np.int32), c.astype(np.int32), v, diag, b, "zipf_spd_%d" % n)


def _near_grid(n: int, ndim: int) -> Tuple[int, ...]:
    if ndim == 2:
        nx = max(2, int(round(np.sqrt(n))))
        ny = max(2, int(round(n / nx)))
        return (ny, nx)
    nx = max(2, int(round(n ** (1.0 / 3.0))))
    ny = max(2, int(round(np.sqrt(n / nx))))
    nz = max(2, int(round(n / (nx * ny))))
    return (nz, ny, nx)


def variable_stencil(shape, sigma: float, rng) -> System:
    """5-point (2D) or 7-point (3D) stencil with log-normal(0, sigma) edge and
    Dirichlet ghost conductances; draws edges (forward directions, each in
    lexicographic order), then ghosts (all directions), then b ~ U[-1, 1]."""
    ndim = len(shape)
    offs = [d for d in _grid_dirs(ndim) if sum(abs(o) for o in d) == 1]
    fwd = [d for d in offs if d > tuple([0] * ndim)]
    pair = {}
    for d in fwd:
        src, _ = _slices(shape, d)
        pair[d] = rng.lognormal(0.0, sigma, tuple(s.stop - s.start for s in src))
    ghost = np.zeros(shape)
    for d in offs:
        src, _ = _slices(shape, d)
        m = np.ones(shape, bool)
        m[src] = False
        ghost[m] += rng.lognormal(0.0, sigma, int(m.sum()))
    sysm = stencil_system(tuple(shape), offs, pair, ghost)
    sysm.b = rng.uniform(-1.0, 1.0, sysm.n)
    return sysm


def batched_stencils(count: int = 4096, lo: int = 200, hi: int = 20000, sigma: float = 1.0,
                     seed: int = 3) -> List[System]:
    """Independent systems for the batched solver.

    Draws, per system in order: target size n ~ log-uniform[lo, hi]; a fair
    coin (2D 5-point or 3D 7-point); then the stencil draws of
    ``variable_stencil`` on the near-square / near-cubic grid for n.
    """
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        nt = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        ndim = 2 if rng.random() < 0.5 else 3
        shape = _near_grid(nt, ndim)
        sysm = variable_stencil(shape, sigma, rng)
        sysm.name = "batch_%d_%s" % (s, "x".join(map(str, shape)))
        out.append(sysm)
    return out


@dataclass
class AdjointProblem:
    shape: Tuple[int, int, int]
    theta: np.ndarray        # per-edge log conductance
    edge_i: np.ndarray       # int32, lower endpoint (row index)
    edge_j: np.ndarray       # int32, upper endpoint
    b: np.ndarray
    x_obs: np.ndarray
    ghost: float


def diffusion7_edges(shape):
    """Interior edges of the 7-point stencil: for each forward direction
    (lexicographic), the pairs (p, p+d) in lexicographic order of p."""
    n = int(np.prod(shape))
    idx = np.arange(n, dtype=np.int64).reshape(shape)
    ei, ej = [], []
    offs = [d for d in _grid_dirs(3) if sum(abs(o) for o in d) == 1 and d > (0, 0, 0)]
    for d in offs:
        src, dst = _slices(shape, d)
        ei.append(idx[src].ravel())
        ej.append(idx[dst].ravel())
    return np.concatenate(ei).astype(np.int32), np.concatenate(ej).astype(np.int32)


def assemble_edges(n: int, ei: np.ndarray, ej: np.ndarray, c: np.ndarray, ghost_diag: np.ndarray) -> System:
    """CSR of sum_e c_e (e_i - e_j)(e_i - e_j)^T + diag(ghost_diag)."""
    r = np.concatenate([ei, ej, np.arange(n)]).astype(np.int64)
    cc = np.concatenate([ej, ei, np.arange(n)]).astype(np.int64)
    D = ghost_diag + np.bincount(ei, c, minlength=n) + np.bincount(ej, c, minlength=n)
    v = np.concatenate([-c, -c, D])
    order = np.argsort(r * n + cc, kind="stable")
    r, cc, v = r[order], cc[order], v[order]
    rowptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=rowptr[1:])
    return System(n, rowptr.astype(np.int32), cc.astype(np.int32), v, D, np.zeros(n))


def ghost_diagonal7(shape, g: float) -> np.ndarray:
    ghost = np.zeros(shape)
    for d in [d for d in _grid_dirs(3) if sum(abs(o) for o in d) == 1]:
        src, _ = _slices(shape, d)
        m = np.ones(shape, bool)
        m[src] = False
        ghost[m] += g
    return ghost.ravel()


def adjoint_problem(nx: int = 96, seed: int = 4, ghost: float = 1.0) -> AdjointProblem:
    """Differentiable-solve workload on a 7-point grid nx^3.

    Draws, in order: theta ~ N(0, 1) per interior edge (edge order of
    ``diffusion7_edges``); theta_obs = theta + 0.1 N(0, 1); b ~ U[-1, 1].
    x_obs is the solution with conductances exp(theta_obs), computed by the
    caller's solver (``x_obs`` is filled with NaN here until then).
    """
    rng = np.random.default_rng(seed)
    shape = (nx, nx, nx)
    ei, ej = diffusion7_edges(shape)
    theta = rng.standard_normal(ei.size)
    theta_obs = theta + 0.1 * rng.standard_normal(ei.size)
    n = nx ** 3
    b = rng.uniform(-1.0, 1.0, n)
    prob = AdjointProblem(shape, theta, ei, ej, b, np.full(n, np.nan), ghost)
    prob.theta_obs = theta_obs
    return prob


def example_tridiagonal(n: int = 65536):
    """The reference example's known-answer systems (pcg/sw/examples/c/
    example.c:132-176): tridiagonal, diagonal 2.2, off-diagonal 1.0, in the
    example's COO emission order and as a 1-based lower-triangle CSC, with b
    from glibc rand() after srand(1) (the default seed): b_i =
    (rand() % n - n/2) / 97.0.  Returns (coo, csc, diag, b1, b2, b3) where the
    three right-hand sides are the example's three successive genVec calls.
    """
    rows, cols, data = [], [], []
    for i in range(n):
        if i != 0:
            rows.append(i); cols.append(i - 1); data.append(1.0)
        if i != n - 1:
            rows.append(i); cols.append(i + 1); data.append(1.0)
        rows.append(i); cols.append(i); data.append(2.2)
    coo = (np.array(rows, np.uint32), np.array(cols, np.uint32), np.array(data, np.float64))
    half = (len(data) + n) // 2
    ridx, cptr, cdat = [], [], []
    for i in range(n):
        cptr.append(i * 2 + 1)
        if i != 0:
            ridx.append(i + 1); cdat.append(1.0)
        ridx.append(i + 1); cdat.append(2.2)
    assert len(ridx) == half
    cptr.append(half + 1)
    csc = (np.array(ridx, np.int64), np.array(cptr, np.int64), np.array(cdat, np.float64))
    diag = np.full(n, 2.2)
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(1)
    bs = []
    for _ in range(3):
        v = np.empty(n)
        for i in range(n):
            val = libc.rand() % n - n // 2
            v[i] = val / 97.0
        bs.append(v)
    return coo, csc, diag, bs[0], bs[1], bs[2]
