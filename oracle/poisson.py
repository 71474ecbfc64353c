"""FP64 restatement of the demag Poisson solve: SA-AMG setup, V-cycles, PCG and ``solve_U``.

Test infrastructure (see ``oracle/__init__.py``).

The reference builds its hierarchy with PyAMG (``src/poisson_solve.py:596-598``), which is absent.
The hierarchy here is the project's own smoothed aggregation, the same algorithm the product's C++
setup implements; integer aggregation must match it bit for bit:

* symmetric strength: off-diagonal a_ij is strong when a_ij^2 > theta^2 |a_ii a_jj|, theta = 0.115
  on the finest level (0.1 when 0.115 gives more than four levels), times 0.35 on every coarser level;
* standard three-pass greedy aggregation in node order (Vanek, Mandel and Brezina 1996): (1) a node
  whose strong neighbours are all free seeds an aggregate with them; (2) a free node joins the
  aggregate of its first aggregated strong neighbour (aggregates as they stood after pass 1);
  (3) a node still free seeds an aggregate with its free strong neighbours; nodes with no strong
  neighbour (Dirichlet rows) stay unaggregated and get an empty prolongation row;
* tentative prolongation 1/sqrt(|aggregate|), damped-Jacobi smoothing
  P = (I - omega D^-1 A) P_tent with omega = (4/3)/rho and rho = 1.05 x the power-method estimate of
  rho(D^-1 A) after 20 steps from a fixed pseudo-random start (Knuth's multiplicative hash of the row
  index), every norm a left-to-right sum so that the C++ setup reproduces it;
* Galerkin A_c = P^T A P, R = P^T; stop at ``max_coarse`` unknowns or ``max_levels`` levels; dense
  inverse on the coarsest level;
* the level-1 Galerkin operator without its weak couplings (|a_ij| + |a_ji| < 2 * 0.002 *
  sqrt(|a_ii a_jj|)), which are added to the diagonal of their row before level 2 is built from it.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

from .fem import spai0_diagonal

THETA0 = 0.115
THETA0_FALLBACK = 0.1  # when THETA0 gives more than four levels
THETA_FACTOR = 0.35    # each coarser level's threshold relative to the finer one
FILTER_EPS = 0.002     # weak couplings of the level-1 operator moved into its diagonal
RHO_STEPS = 20
RHO_SAFETY = 1.05


def strength(A: sp.csr_matrix, theta: float) -> sp.csr_matrix:
    """Boolean strength pattern (no diagonal)."""
    A = A.tocsr()
    d = A.diagonal()
    rows = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    cols = A.indices
    v = A.data
    keep = (rows != cols) & (v * v > (theta * theta) * np.abs(d[rows] * d[cols]))
    S = sp.csr_matrix((np.ones(int(keep.sum()), dtype=np.int8), (rows[keep], cols[keep])), shape=A.shape)
    S.sort_indices()
    return S


def standard_aggregation(S: sp.csr_matrix) -> tuple[np.ndarray, int]:
    """Greedy three-pass aggregation; returns (aggregate id per node or -1, number of aggregates)."""
    n = S.shape[0]
    ptr, idx = S.indptr, S.indices
    agg = np.full(n, -1, dtype=np.int64)
    nagg = 0
    # pass 1
    for i in range(n):
        if agg[i] >= 0:
            continue
        nb = idx[ptr[i]:ptr[i + 1]]
        if nb.size == 0:
            continue
        if np.any(agg[nb] >= 0):
            continue
        agg[i] = nagg
        agg[nb] = nagg
        nagg += 1
    # pass 2: attach to aggregates as they stood after pass 1
    after1 = agg.copy()
    for i in range(n):
        if after1[i] >= 0:
            continue
        nb = idx[ptr[i]:ptr[i + 1]]
        for j in nb:
            if after1[j] >= 0:
                agg[i] = after1[j]
                break
    # pass 3
    for i in range(n):
        if agg[i] >= 0:
            continue
        nb = idx[ptr[i]:ptr[i + 1]]
        if nb.size == 0:
            continue
        agg[i] = nagg
        for j in nb:
            if agg[j] < 0:
                agg[j] = nagg
        nagg += 1
    return agg, nagg


def tentative_prolongator(agg: np.ndarray, nagg: int) -> sp.csr_matrix:
    n = agg.shape[0]
    has = agg >= 0
    size = np.bincount(agg[has], minlength=nagg).astype(np.float64)
    rows = np.nonzero(has)[0]
    vals = 1.0 / np.sqrt(size[agg[has]])
    P = sp.csr_matrix((vals, (rows, agg[has])), shape=(n, nagg))
    P.sort_indices()
    return P


def gershgorin_rho(A: sp.csr_matrix) -> float:
    d = np.abs(A.diagonal())
    rs = np.asarray(abs(A).sum(axis=1)).ravel()
    ok = d > 0
    return float(np.max(rs[ok] / d[ok])) if np.any(ok) else 1.0


def power_rho(A: sp.csr_matrix, steps: int = RHO_STEPS, safety: float = RHO_SAFETY) -> float:
    """rho(D^-1 A) by the power method (the spectral-radius estimate of the prolongation smoothing)."""
    n = A.shape[0]
    d = A.diagonal()
    dinv = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 0.0)
    x = ((np.arange(n, dtype=np.uint64) * np.uint64(2654435761)) % np.uint64(1 << 32)).astype(np.float64)
    x = x / 4294967296.0 - 0.5
    nx = float(np.sqrt(np.cumsum(x * x)[-1])) if n else 0.0
    lam = 1.0
    for _ in range(steps):
        y = dinv * (A @ x)
        ny = float(np.sqrt(np.cumsum(y * y)[-1]))
        if not (ny > 0.0 and nx > 0.0):
            break
        lam = ny / nx
        x = y / ny
        nx = 1.0
    return safety * lam


def smooth_prolongator(A: sp.csr_matrix, T: sp.csr_matrix) -> sp.csr_matrix:
    rho = power_rho(A)
    omega = (4.0 / 3.0) / rho
    d = A.diagonal()
    dinv = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 0.0)
    P = (T - omega * (sp.diags(dinv) @ (A @ T))).tocsr()
    P.sort_indices()
    return P


def filter_weak(A: sp.csr_matrix, eps: float) -> sp.csr_matrix:
    """A without its weak off-diagonal couplings, |a_ij| + |a_ji| < 2 eps sqrt(|a_ii a_jj|) (a_ji = 0
    when not stored), each row's weak values summed from zero in column order and added to its
    diagonal (row sums kept)."""
    A = A.tocsr()
    A.sort_indices()
    n = A.shape[0]
    rows = np.repeat(np.arange(n), np.diff(A.indptr))
    cols = A.indices
    d = A.diagonal()
    At = A.T.tocsr()
    At.sort_indices()
    if np.array_equal(At.indptr, A.indptr) and np.array_equal(At.indices, A.indices):
        aji = At.data
    else:
        aji = np.asarray(A[cols, rows]).ravel()
    weak = (rows != cols) & (np.abs(A.data) + np.abs(aji) < 2.0 * eps * np.sqrt(np.abs(d[rows] * d[cols])))
    lump = np.bincount(rows[weak], weights=A.data[weak], minlength=n)
    keep = ~weak
    data, r, c = A.data[keep].copy(), rows[keep], cols[keep]
    on_diag = r == c
    data[on_diag] = data[on_diag] + lump[r[on_diag]]
    indptr = np.concatenate([[0], np.cumsum(np.bincount(r, minlength=n))]).astype(A.indptr.dtype)
    return sp.csr_matrix((data, c.copy(), indptr), shape=A.shape)


@dataclass
class Level:
    A: sp.csr_matrix
    spai0: np.ndarray
    diag: np.ndarray
    P: sp.csr_matrix | None = None
    R: sp.csr_matrix | None = None
    agg: np.ndarray | None = None
    A_inv: np.ndarray | None = None


@dataclass
class Hierarchy:
    levels: list[Level] = field(default_factory=list)


def build_hierarchy(A: sp.csr_matrix, max_levels: int = 10, max_coarse: int = 1000,
                    theta0: float | None = None) -> Hierarchy:
    """SA-AMG setup (the project's own restatement; the reference calls PyAMG here).  Without theta0:
    THETA0, or THETA0_FALLBACK when THETA0 gives more than four levels."""
    if theta0 is None:
        H = build_hierarchy(A, max_levels, max_coarse, THETA0)
        return H if len(H.levels) <= 4 else build_hierarchy(A, max_levels, max_coarse, THETA0_FALLBACK)
    H = Hierarchy()
    Acur = A.tocsr()
    Acur.sort_indices()
    theta = theta0
    while True:
        lvl = Level(A=Acur, spai0=spai0_diagonal(Acur), diag=Acur.diagonal().copy())
        H.levels.append(lvl)
        n = Acur.shape[0]
        if n <= max_coarse or len(H.levels) >= max_levels:
            break
        S = strength(Acur, theta)
        agg, nagg = standard_aggregation(S)
        if nagg == 0 or nagg >= n:
            break
        T = tentative_prolongator(agg, nagg)
        P = smooth_prolongator(Acur, T)
        R = P.T.tocsr()
        R.sort_indices()
        Ac = (R @ Acur @ P).tocsr()
        Ac.sort_indices()
        if len(H.levels) == 1 and FILTER_EPS > 0:
            Ac = filter_weak(Ac, FILTER_EPS)
        lvl.P, lvl.R, lvl.agg = P, R, agg
        Acur = Ac
        theta *= THETA_FACTOR
    last = H.levels[-1]
    last.A_inv = np.linalg.inv(last.A.toarray())
    return H


def vcycle_spai0(H: Hierarchy, apply_A0, b: np.ndarray) -> np.ndarray:
    """SPAI0-smoothed V(1,1) cycle, ``src/amg_utils.py:557-623``."""

    def rec(l, bl):
        lvl = H.levels[l]
        if l == len(H.levels) - 1:
            return lvl.A_inv @ bl
        Aop = apply_A0 if l == 0 else (lambda v: lvl.A @ v)
        x = np.zeros_like(bl)
        x = x + lvl.spai0 * (bl - Aop(x))
        r = bl - Aop(x)
        e = rec(l + 1, lvl.R @ r)
        x = x + lvl.P @ e
        x = x + lvl.spai0 * (bl - Aop(x))
        return x

    return rec(0, b)


def vcycle_jacobi(H: Hierarchy, apply_A0, b: np.ndarray, omega: float = 0.6667) -> np.ndarray:
    """Jacobi-smoothed V(1,1) cycle, ``src/amg_utils.py:491-554`` with ``:377-404``."""

    def rec(l, bl):
        lvl = H.levels[l]
        if l == len(H.levels) - 1:
            return lvl.A_inv @ bl
        Aop = apply_A0 if l == 0 else (lambda v: lvl.A @ v)
        x = np.zeros_like(bl)
        x = x + omega * ((bl - Aop(x)) / (lvl.diag + 1e-30))
        r = bl - Aop(x)
        e = rec(l + 1, lvl.R @ r)
        x = x + lvl.P @ e
        x = x + omega * ((bl - Aop(x)) / (lvl.diag + 1e-30))
        return x

    return rec(0, b)


def pcg(apply_A, apply_Minv, b, x0, tol, maxiter, mask=None):
    """Preconditioned CG with the reference's stopping rule, ``src/poisson_solve.py:422-478``.

    Returns (x, iterations, r.r) with r the recursively updated residual.
    """
    eps = 1e-30
    if mask is not None:
        b = b * mask
        x = x0 * mask
    else:
        x = x0.copy()
    r = b - apply_A(x)
    if mask is not None:
        r = r * mask
    z = apply_Minv(r)
    p = z.copy()
    rz = float(r @ z)
    r2 = float(r @ r)
    tol2 = tol * tol * float(b @ b)
    it = 0
    while it < maxiter and r2 > tol2:
        Ap = apply_A(p)
        if mask is not None:
            Ap = Ap * mask
        alpha = rz / (float(p @ Ap) + eps)
        x = x + alpha * p
        r = r - alpha * Ap
        z = apply_Minv(r)
        rz_new = float(r @ z)
        beta = rz_new / (rz + eps)
        p = z + beta * p
        r2 = float(r @ r)
        rz = rz_new
        it += 1
    return x, it, r2


class SolveU:
    """``make_solve_U`` / ``solve_U`` in assembled or matrix-free mode, ``src/poisson_solve.py:483-776``.

    The operator honours the reference's semantics: in assembled mode A already carries the
    Dirichlet identity rows and no mask is applied at call time; in matrix-free mode the Poisson
    operator is the regularised Neumann one unless ``mask`` is given at call time (the reference
    reads it from ``sparse_ops["boundary_mask"]``).  Zero-mean projection is applied only when the
    problem was built without a boundary mask (``:535-536``).
    """

    def __init__(self, p, ops=None, mode="assembled", precond_type="amgcl", cg_tol=1e-8, cg_maxiter=2000,
                 reg=1e-12, hierarchy=None, max_levels=10, max_coarse=1000):
        from . import fem

        self.p, self.mode, self.precond_type = p, mode, precond_type
        self.cg_tol, self.cg_maxiter, self.reg = cg_tol, cg_maxiter, reg
        self.enforce_zero_mean = p.boundary_mask is None
        self.ops = ops if ops is not None else fem.assembled_operators(p, reg=reg)
        self.H = hierarchy if hierarchy is not None else build_hierarchy(self.ops["A"], max_levels, max_coarse)

    def apply_A(self, U, mask=None):
        from . import fem

        if self.mode == "assembled":
            return fem.apply_A_asm(self.ops, U, mask)
        return fem.apply_A_mf(self.p, U, self.reg, mask)

    def rhs(self, m, mask=None):
        from . import fem

        if self.mode == "assembled":
            return fem.rhs_from_m_asm(self.ops, m, mask)
        return fem.rhs_from_m_mf(self.p, m) * (1.0 if mask is None else mask)

    def __call__(self, m, x0, tol=None, return_info=False, mask=None):
        tol = self.cg_tol if tol is None else tol
        b = self.rhs(m, mask if self.mode == "assembled" else None)
        bnorm2 = float(b @ b)
        x0 = np.asarray(x0, np.float64)
        if self.enforce_zero_mean:
            b = b - b.mean()
            x0 = x0 - x0.mean()
        A0 = lambda v: self.apply_A(v, mask)  # noqa: E731
        if self.precond_type == "amgcl":
            M = lambda r: vcycle_spai0(self.H, A0, r)  # noqa: E731
        elif self.precond_type == "amg":
            M = lambda r: vcycle_jacobi(self.H, A0, r)  # noqa: E731
        elif self.precond_type == "jacobi":
            d = self.ops["A"].diagonal()
            M = lambda r: r / (d + 1e-30) * (1.0 if mask is None else mask)  # noqa: E731
        else:
            M = lambda r: r * (1.0 if mask is None else mask)  # noqa: E731
        U, it, r2 = pcg(A0, M, b, x0, tol, self.cg_maxiter, mask)
        if self.enforce_zero_mean:
            U = U - U.mean()
        if return_info:
            return U, it, float(np.sqrt(r2 / (bnorm2 + 1e-30)))
        return U
