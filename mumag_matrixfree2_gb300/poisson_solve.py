"""``make_solve_U`` with the reference's signature (``src/poisson_solve.py:483-533``), on the GPU."""

from __future__ import annotations

import numpy as np

from .cuda_backend import problem_for_geom


def make_solve_U(geom, Js_lookup, *, precond_type: str = "jacobi", order: int = 3, chunk_elems: int = 200_000,
                 cg_maxiter: int = 2000, cg_tol: float = 1e-8, poisson_reg: float = 1e-12,
                 grad_backend: str = "stored_grad_phi", enforce_zero_mean=None, boundary_mask=None,
                 assembly: str = "scatter", mode: str = "matrix_free", A_sparse=None, Dx_sparse=None,
                 Dy_sparse=None, Dz_sparse=None, A_diag=None, cpu_spmv_backend: str = "scipy",
                 poisson_solver: str = "jax", precision: str = "fp64", problem=None, max_levels: int = 10,
                 max_coarse: int = 1000):
    """Return solve_U(m, x0, tol=None, return_info=False, sparse_ops=None) -> U or (U, it, rel_res).

    The demag right-hand side is b = D m; PCG with the chosen preconditioner ("amgcl": SA-AMG V-cycle
    with SPAI0 smoothing, "amg": with damped Jacobi, "jacobi", "none") runs from x0 until the
    recursive residual satisfies |r| <= tol |b| (``:422-478``).  Without a boundary mask the mean of b,
    x0 and U is projected out (``:535-536``).  precision="mixed" solves the same system with FP32
    corrections inside FP64 iterative refinement (the true FP64 residual meets the tolerance).
    ``problem``: share an existing device problem (e.g. the minimizer's).
    """
    if precond_type == "chebyshev":
        raise NotImplementedError("the chebyshev preconditioner is not part of the cuda backend")
    if enforce_zero_mean is not None and enforce_zero_mean != (boundary_mask is None):
        raise NotImplementedError("zero-mean projection follows the boundary mask in the cuda backend")
    Js = np.asarray(Js_lookup, np.float64).ravel()
    G = len(Js)
    if problem is None:
        problem = problem_for_geom(geom, np.zeros(G), np.zeros(G), Js, np.tile([0.0, 0.0, 1.0], (G, 1)),
                                   boundary_mask=boundary_mask)
    prob = problem
    if not prob.poisson_built:
        if precision != "fp64":
            prob.set_precision(precision)
        prob.build_poisson(poisson_reg, precond_type, max_levels, max_coarse)
    default_tol = float(cg_tol)

    def solve_U(m, x0, tol=None, return_info=False, sparse_ops=None):
        U, it, rr, rc = prob.solve_u(m, x0, default_tol if tol is None else float(tol), cg_maxiter)
        if return_info:
            return U, it, rr
        return U

    solve_U.problem = prob
    return solve_U
