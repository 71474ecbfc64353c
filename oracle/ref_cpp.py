"""ctypes driver of the reference's CPU minimizer library (test infrastructure).

``oracle/_ref/libcpp_mkl_minimizer.so`` is the reference's ``src/cpp/cpp_mkl_minimizer.cpp``
compiled unchanged against the MKL-API shim (``oracle/build_ref.py``); ``oracle/_build/libref_port.so``
restates its demag solve and energy/gradient entry points for hosts without the reference source.
This module binds either library the way the reference's Python side does
(``src/cpp_minimizer.py:31-175``, ``src/amg_utils.py:792-881``) and builds the interleaved operators
that its ``--cpp-mkl`` path passes (``src/loop.py:1133-1166``):

* ``K_eff`` (3N x 3N): exchange + anisotropy, rows/columns ``3 i + c``;
* ``G`` (3N x N): 2 D^T with rows ``3 i + c``;
* ``D`` (N x 3N): the divergence operator with columns ``3 j + c``;
* PARDISO is given the upper triangle of the Dirichlet Poisson matrix (``src/amg_utils.py:825-829``).

Only ``tests/``, ``bench.py``'s reference / ``cpu_baseline`` legs and the fixture scripts under
``tests/golden/`` use it.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np
import scipy.sparse as sp

from . import fem
from . import minimize as omin

ORACLE = Path(__file__).resolve().parent
REF_LIB = ORACLE / "_ref" / "libcpp_mkl_minimizer.so"
PORT_LIB = ORACLE / "_build" / "libref_port.so"

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray):
    return a.ctypes.data_as(_ip)


class RefLib:
    """One loaded library; ``kind`` is "reference" (the reference's own C++) or "port"."""

    def __init__(self, path: Path, kind: str):
        self.path, self.kind = Path(path), kind
        L = self.lib = ctypes.CDLL(str(path))
        L.mkl_sparse_d_create_csr.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, _ip, _ip, _ip, _dp]
        L.mkl_sparse_d_create_csr.restype = ctypes.c_int
        L.mkl_sparse_destroy.argtypes = [ctypes.c_void_p]
        L.mkl_sparse_destroy.restype = ctypes.c_int
        L.init_pardiso.argtypes = [ctypes.c_int, _dp, _ip, _ip]
        L.init_pardiso.restype = ctypes.c_int64
        L.free_pardiso.argtypes = [ctypes.c_int64]
        L.free_pardiso.restype = None
        L.pardiso_solve_direct.argtypes = [ctypes.c_int64, _dp, _dp]
        L.pardiso_solve_direct.restype = ctypes.c_int
        L.evaluate_energy_and_grad.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_void_p, ctypes.c_void_p,
                                               _dp, _dp, ctypes.c_double]
        L.evaluate_energy_and_grad.restype = None
        L.solve_poisson.argtypes = [ctypes.c_int, _dp, ctypes.c_int64, ctypes.c_void_p, _dp, _dp]
        L.solve_poisson.restype = None
        L.mkl_shim_set_pardiso_tol.argtypes = [ctypes.c_double]
        L.mkl_shim_set_pardiso_tol.restype = None
        L.mkl_shim_last_iterations.restype = ctypes.c_int
        L.mkl_shim_last_relres.restype = ctypes.c_double
        L.mkl_shim_max_threads.restype = ctypes.c_int
        self.full = kind == "reference"
        if self.full:
            L.solve_Py_g.argtypes = [ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _ip]
            L.solve_Py_g.restype = None
            # src/cpp_minimizer.py:31-75
            L.run_cpp_pcohen_hs_minimization.argtypes = (
                [ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6 + [ctypes.c_int, ctypes.c_double, ctypes.c_int64]
                + [_dp] * 5 + [_dp, _ip, _ip] * 3 + [_dp, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_int, ctypes.c_int] + [_ip] * 4 + [_dp] * 2)
            L.run_cpp_pcohen_hs_minimization.restype = ctypes.c_int

    def set_pardiso_tol(self, tol: float) -> None:
        self.lib.mkl_shim_set_pardiso_tol(float(tol))

    def threads(self) -> int:
        """OpenMP threads of the library's parallel regions."""
        return int(self.lib.mkl_shim_max_threads())

    def last_solve(self) -> tuple[int, float]:
        return int(self.lib.mkl_shim_last_iterations()), float(self.lib.mkl_shim_last_relres())


def load(kind: str = "any") -> RefLib | None:
    """The reference library when built (``kind`` "reference" or "any"), else the port ("port" or "any")."""
    if kind in ("reference", "any") and REF_LIB.exists():
        return RefLib(REF_LIB, "reference")
    if kind in ("port", "any") and PORT_LIB.exists():
        return RefLib(PORT_LIB, "port")
    return None


class Csr:
    """A CSR matrix registered with the library (the arrays are kept alive here)."""

    def __init__(self, lib: RefLib, M: sp.csr_matrix):
        M = sp.csr_matrix(M)
        M.sort_indices()
        self.lib = lib
        self.shape = M.shape
        self.val = np.ascontiguousarray(M.data, np.float64)
        self.col = np.ascontiguousarray(M.indices, np.int32)
        self.ptr = np.ascontiguousarray(M.indptr, np.int32)
        h = ctypes.c_void_p()
        st = lib.lib.mkl_sparse_d_create_csr(ctypes.byref(h), 0, M.shape[0], M.shape[1], _i(self.ptr[:-1]),
                                             _i(self.ptr[1:]), _i(self.col), _d(self.val))
        if st != 0:
            raise RuntimeError(f"mkl_sparse_d_create_csr failed ({st})")
        self.handle = h

    def __del__(self):
        try:
            self.lib.lib.mkl_sparse_destroy(self.handle)
        except Exception:  # noqa: BLE001 - interpreter teardown
            pass


def _pair_pattern(conn: np.ndarray, N: int):
    """Node pairs that share an element, sorted row-major: (rows, cols, row pointer, map from the
    (E,4,4) element pairs to their pattern index, map from each pair (i,j) to the index of (j,i))."""
    conn = np.asarray(conn, np.int64)
    keys = (np.repeat(conn, 4, axis=1) * N + np.tile(conn, (1, 4))).reshape(-1)
    uk, inv = np.unique(keys, return_inverse=True)
    pr, pc = uk // N, uk % N
    ptr = np.zeros(N + 1, np.int64)
    np.cumsum(np.bincount(pr, minlength=N), out=ptr[1:])
    tperm = np.searchsorted(uk, pc * N + pr)
    return pr, pc, ptr, inv.reshape(-1), tperm


def interleaved_operators(p: fem.Problem, reg: float = 1e-12) -> dict:
    """K_eff, G, D in the C++ path's interleaved layout and the Dirichlet Poisson matrix A.

    Every node pair that shares an element carries a full 3x3 block in K_eff, three entries in D and
    G, explicit zeros included, as the reference's COO assembly leaves them
    (``src/amg_utils.py:660-702,741-789``, ``src/loop.py:1133-1154``).  The entries are summed per
    pair with one pass over the element pairs instead of a 9x larger COO array.
    """
    N = p.N
    pr, pc, ptr, inv, tperm = _pair_pattern(p.conn, N)
    nnz = len(pr)
    gp = p.grad_phi
    grp = p.mat_id - 1
    # exchange 2 A Ve grad phi_a . grad phi_b (x I3) and anisotropy -2 K1 Ve / 20 (1 + delta_ab) (x k k^T)
    exch = (2.0 * p.A_lookup[grp] * p.volume)[:, None, None] * np.einsum("eai,ebi->eab", gp, gp)
    blocks = np.zeros((nnz, 3, 3))
    blocks[:, [0, 1, 2], [0, 1, 2]] = np.bincount(inv, weights=exch.reshape(-1), minlength=nnz)[:, None]
    del exch
    base = np.ones((4, 4)) + np.eye(4)
    for g in range(len(p.K1_lookup)):
        if p.K1_lookup[g] == 0.0:
            continue
        sel = grp == g
        w = np.zeros((len(grp), 4, 4))
        w[sel] = (-2.0 * p.K1_lookup[g] * p.volume[sel] / 20.0)[:, None, None] * base
        k = p.k_easy[g]
        blocks += np.bincount(inv, weights=w.reshape(-1), minlength=nnz)[:, None, None] * np.outer(k, k)
    cnt = np.diff(ptr)
    row = np.repeat(np.arange(N), cnt)
    off = np.arange(nnz) - ptr[row]
    # K_eff: row 3i+c holds, pair by pair (ascending j), the columns 3j, 3j+1, 3j+2
    kpos = (9 * ptr[row] + 3 * off)[:, None, None] + (3 * cnt[row])[:, None, None] * np.arange(3)[None, :, None] \
        + np.arange(3)[None, None, :]
    kval = np.empty(9 * nnz)
    kval[kpos.reshape(-1)] = blocks.reshape(-1)
    kcol = np.empty(9 * nnz, np.int64)
    kcol[kpos.reshape(-1)] = np.broadcast_to(3 * pc[:, None, None] + np.arange(3)[None, None, :], kpos.shape).reshape(-1)
    kptr = np.zeros(3 * N + 1, np.int64)
    kptr[1:] = np.cumsum(np.repeat(3 * cnt, 3))
    K = sp.csr_matrix((kval, kcol, kptr), shape=(3 * N, 3 * N))
    del blocks, kpos, kval, kcol
    # D (N x 3N): D_c(a,b) = Js Ve / 4 (grad phi_a)_c, columns 3b+c; G = 2 D^T with rows 3b+c
    f = p.Js_lookup[grp] * p.volume / 4.0
    dv = np.empty((nnz, 3))
    for c in range(3):
        w = np.repeat((f[:, None] * gp[:, :, c])[:, :, None], 4, axis=2)
        dv[:, c] = np.bincount(inv, weights=w.reshape(-1), minlength=nnz)
    D = sp.csr_matrix((dv.reshape(-1), (3 * pc[:, None] + np.arange(3)).reshape(-1), 3 * ptr), shape=(N, 3 * N))
    gpos = (3 * ptr[row] + off)[:, None] + cnt[row][:, None] * np.arange(3)[None, :]
    gval = np.empty(3 * nnz)
    gval[gpos.reshape(-1)] = (2.0 * dv[tperm]).reshape(-1)
    gcol = np.empty(3 * nnz, np.int64)
    gcol[gpos.reshape(-1)] = np.repeat(pc, 3)
    gptr = np.zeros(3 * N + 1, np.int64)
    gptr[1:] = np.cumsum(np.repeat(cnt, 3))
    G = sp.csr_matrix((gval, gcol, gptr), shape=(3 * N, N))
    A = fem.assemble_poisson(p, reg=reg, with_boundary=p.boundary_mask is not None)
    return {"A": A, "K_eff": K, "D": D, "G": G}


class CppProblem:
    """A problem set up for the C++ path: registered operators, the factorised Poisson matrix and the
    node weights that ``src/cpp_minimizer.py:89-94`` and ``src/hysteresis_loop.py:473-474`` pass."""

    def __init__(self, lib: RefLib, p: fem.Problem, reg: float = 1e-12, pardiso_tol: float = 1e-12):
        self.lib, self.p, self.N = lib, p, p.N
        ops = interleaved_operators(p, reg)
        self.K = Csr(lib, ops["K_eff"])
        self.G = Csr(lib, ops["G"])
        self.D = Csr(lib, ops["D"])
        del ops["K_eff"], ops["G"]
        lib.set_pardiso_tol(pardiso_tol)
        Au = sp.triu(ops["A"], format="csr")
        Au.sort_indices()
        self._a = np.ascontiguousarray(Au.data, np.float64)
        self._ia = np.ascontiguousarray(Au.indptr, np.int32)
        self._ja = np.ascontiguousarray(Au.indices, np.int32)
        self.pardiso = int(lib.lib.init_pardiso(p.N, _d(self._a), _i(self._ia), _i(self._ja)))
        if self.pardiso <= 0:
            raise RuntimeError(f"init_pardiso failed ({self.pardiso})")
        self.mask = None if p.boundary_mask is None else np.ascontiguousarray(p.boundary_mask, np.float64)
        self.M_nodal = np.ascontiguousarray(p.M_nodal, np.float64)
        self.inv_Vmag = 1.0 / p.V_mag
        self.inv_M_rel = np.ascontiguousarray(
            np.divide(p.V_mag, p.M_nodal, out=np.zeros(p.N), where=p.M_nodal > 1e-20))
        self.inv_M_prec = np.ascontiguousarray(1.0 / (fem.exchange_diagonal(p) + 1e-30))

    def __del__(self):
        try:
            self.lib.lib.free_pardiso(self.pardiso)
        except Exception:  # noqa: BLE001
            pass

    # --- the library's entry points --------------------------------------------------------
    def energy_and_grad(self, m, U, B):
        """``evaluate_energy_and_grad`` (cpp_mkl_minimizer.cpp:178-206): (E, g (N,3))."""
        m = np.ascontiguousarray(np.asarray(m, np.float64).reshape(-1))
        U = np.ascontiguousarray(U, np.float64)
        B = np.ascontiguousarray(B, np.float64)
        g = np.zeros(3 * self.N)
        E = ctypes.c_double()
        self.lib.lib.evaluate_energy_and_grad(self.N, _d(m), _d(U), _d(B), _d(self.M_nodal), self.K.handle,
                                              self.G.handle, ctypes.byref(E), _d(g), self.inv_Vmag)
        return float(E.value), g.reshape(self.N, 3)

    def solve_poisson(self, m):
        """``solve_poisson`` (cpp_mkl_minimizer.cpp:208-231): U = mask A^-1 (mask D m)."""
        m = np.ascontiguousarray(np.asarray(m, np.float64).reshape(-1))
        U = np.zeros(self.N)
        mp = None if self.mask is None else _d(self.mask)
        self.lib.lib.solve_poisson(self.N, _d(m), self.pardiso, self.D.handle, _d(U), mp)
        return U

    def solve_Py_g(self, m, g_ext, g_tan_ext, max_iter, tol=0.0, reg=0.0, nu=1e-3):
        """``solve_Py_g`` (cpp_mkl_minimizer.cpp:233-359): (y (N,3), inner iterations)."""
        if not self.lib.full:
            raise RuntimeError("solve_Py_g needs the reference library")
        arr = [np.ascontiguousarray(np.asarray(a, np.float64).reshape(-1)) for a in (m, g_ext, g_tan_ext)]
        y = np.zeros(3 * self.N)
        it = ctypes.c_int()
        self.lib.lib.solve_Py_g(self.N, _d(arr[0]), _d(arr[1]), _d(arr[2]), _d(self.inv_M_prec), self.K.handle,
                                int(max_iter), float(tol), float(reg), float(nu), self.inv_Vmag, _d(y),
                                ctypes.byref(it))
        return y.reshape(self.N, 3), int(it.value)

    def minimize(self, m0, B, U0, prm: omin.Params, method: str = "pcohen_hs"):
        """``run_cpp_pcohen_hs_minimization`` with the arguments of ``src/cpp_minimizer.py:79-175``
        (Hestenes-Stiefel beta when "hs" is in the method name, else Polak-Ribiere, ``:125-126``).

        Returns (m, U, info) with info keys iters, evals, demag, preco_iters, E, gnorm.
        """
        if not self.lib.full:
            raise RuntimeError("the minimizer needs the reference library")
        N = self.N
        m = np.ascontiguousarray(np.asarray(m0, np.float64).reshape(-1)).copy()
        U = np.ascontiguousarray(np.asarray(U0, np.float64)).copy()
        B = np.ascontiguousarray(B, np.float64)
        out_i = [ctypes.c_int() for _ in range(4)]
        out_d = [ctypes.c_double() for _ in range(2)]
        mp = None if self.mask is None else _d(self.mask)
        K, G, D = self.K, self.G, self.D
        self.lib.lib.run_cpp_pcohen_hs_minimization(
            N, int(prm.max_iter), float(prm.tau_f), float(prm.eps_a), float(prm.ls_eta1), float(prm.ls_eta2),
            float(prm.ls_C), float(prm.ls_c), 15, self.inv_Vmag, self.pardiso,
            _d(m), _d(B), _d(U), _d(self.M_nodal), mp,
            _d(K.val), _i(K.col), _i(K.ptr), _d(G.val), _i(G.col), _i(G.ptr), _d(D.val), _i(D.col), _i(D.ptr),
            _d(self.inv_M_rel), _d(self.inv_M_prec),
            1 if prm.pc_auto else 0, float(prm.pc_force_eta), float(prm.pc_force_alpha),
            float(prm.cg_tol), int(prm.pc_iters), float(prm.pc_reg), float(prm.pc_stagnation_nu),
            int(prm.L) if prm.L is not None else N, 1 if "hs" in method else 0,
            *[ctypes.byref(o) for o in out_i], *[ctypes.byref(o) for o in out_d])
        info = dict(iters=out_i[0].value, evals=out_i[1].value, demag=out_i[2].value, preco_iters=out_i[3].value,
                    E=out_d[0].value, gnorm=out_d[1].value)
        return m.reshape(N, 3), U, info


def run_sweep(cp: CppProblem, m0, h_dir, B_vals, prm: omin.Params, Js_ref=1.0, method="pcohen_hs"):
    """The ``--cpp-mkl`` branch of the field loop (``src/hysteresis_loop.py:457-495,566-580``).

    Returns rows (B_tesla, J_tesla, E, iters, evals, demag, preco) and the final (m, U).
    """
    p = cp.p
    m = m0 / np.linalg.norm(m0, axis=1, keepdims=True)
    U = np.zeros(p.N)
    rows = []
    for Bmag in B_vals:
        m, U, info = cp.minimize(m, Bmag * h_dir, U, prm, method)
        J = omin.volume_averaged_J_parallel(m, p.conn, p.volume, p.mat_id, p.Js_lookup, h_dir)
        rows.append((Bmag * Js_ref, J * Js_ref, info["E"], info["iters"], info["evals"], info["demag"],
                     info["preco_iters"]))
    return rows, m, U
