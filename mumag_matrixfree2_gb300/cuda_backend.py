"""Device problem: one mesh with its materials resident on the GPU behind libmumag_cuda.

``Problem`` is the thin object every factory of this package (``make_energy_kernels``,
``make_solve_U``, ``make_minimizer``) shares, so the mesh and operators are uploaded once.  Host
arrays (numpy) go through the host-pointer entry points; CUDA torch tensors go through the ``_dev``
entry points without a copy.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import check, dptr, f64, i32, lib


def _is_torch_cuda(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


@dataclass
class MinimizerParams:
    """Defaults of the reference's CLI (``src/loop.py:578-700``) for the minimizer parameters."""

    method: str = "pcohen_hs"
    max_iter: int = 2000
    tau_f: float = 1e-8
    eps_a: float = 1e-12
    tau0: float = 1e-2
    ls_eta1: float = 0.1
    ls_eta2: float = 0.1
    ls_C: float = 2.0
    ls_c: float = 0.5
    ls_max_evals: int = 15
    pc_iters: int = 10
    pc_auto: bool = True
    pc_force_eta: float = 0.5
    pc_force_alpha: float = 0.5
    pc_stagnation_nu: float = 0.01
    pc_reg: float = 0.0
    memory: int = 5
    wg_gamma: int = 5
    L: int | None = None
    cg_tol: float = 1e-8
    phi_tol: float | None = None
    cg_maxiter: int = 2000
    tn_iters: int = 5
    lr: float = 0.1
    mu: float = 0.9
    phi_extrapolate: bool = True
    cpp_semantics: bool = False  # the reference's C++ minimizer conventions (pcohen_hs / pcohen)

    def to_c(self) -> _abi.MinParams:
        if self.method not in _abi.METHODS:
            raise ValueError(f"method {self.method!r} is not available in the cuda backend "
                             f"(available: {sorted(_abi.METHODS)})")
        return _abi.MinParams(
            method=_abi.METHODS[self.method], max_iter=int(self.max_iter), pc_iters=int(self.pc_iters),
            pc_auto=1 if self.pc_auto else 0, ls_max_evals=int(self.ls_max_evals), L=int(self.L or 0),
            memory=int(self.memory), wg_gamma=int(self.wg_gamma), tau_f=self.tau_f, eps_a=self.eps_a,
            tau0=self.tau0, ls_eta1=self.ls_eta1, ls_eta2=self.ls_eta2, ls_C=self.ls_C, ls_c=self.ls_c,
            pc_force_eta=self.pc_force_eta, pc_force_alpha=self.pc_force_alpha,
            pc_stagnation_nu=self.pc_stagnation_nu, pc_reg=self.pc_reg, cg_tol=self.cg_tol,
            phi_tol=-1.0 if self.phi_tol is None else float(self.phi_tol), cg_maxiter=int(self.cg_maxiter),
            tn_iters=int(self.tn_iters), lr=float(self.lr), mu=float(self.mu),
            phi_extrapolate=1 if self.phi_extrapolate else 0, cpp_semantics=1 if self.cpp_semantics else 0)


class Problem:
    """A mesh, its materials and (after ``build_poisson``) the demag solver, resident on the GPU."""

    def __init__(self, conn, volume, grad_phi, mat_id, A_lookup, K1_lookup, Js_lookup, k_easy, V_mag, M_nodal,
                 boundary_mask=None, n_nodes: int | None = None):
        self.conn = i32(np.asarray(conn)[:, :4])
        self.N = int(n_nodes if n_nodes is not None else self.conn.max() + 1)
        self.E = int(self.conn.shape[0])
        volume, grad_phi = f64(volume), f64(grad_phi, (self.E, 4, 3))
        mat_id = i32(mat_id)
        A, K1, Js = f64(np.ravel(A_lookup)), f64(np.ravel(K1_lookup)), f64(np.ravel(Js_lookup))
        k = f64(k_easy, (len(A), 3))
        M = f64(M_nodal).reshape(-1)
        mask = None if boundary_mask is None else f64(boundary_mask).reshape(-1)
        self.V_mag = float(V_mag)
        self.has_mask = mask is not None
        self.mask_host = mask
        self.precision = "fp64"
        self.reg, self.precond_type, self.max_levels, self.max_coarse = 1e-12, "amgcl", 10, 1000
        h = C.c_void_p()
        check("mm_create", lib().mm_create(
            self.N, self.E, _abi.iptr(self.conn), dptr(volume), dptr(grad_phi), _abi.iptr(mat_id), len(A), dptr(A),
            dptr(K1), dptr(Js), dptr(k), self.V_mag, dptr(M), dptr(mask), C.byref(h)))
        self.h = h
        self.poisson_built = False
        self.n_levels = 0

    # -- lifetime --------------------------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            lib().mm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, fn, rc):
        return check(fn, rc, self.h)

    # -- Poisson ---------------------------------------------------------------------------------
    def build_poisson(self, reg=1e-12, precond_type="amgcl", max_levels=10, max_coarse=1000) -> int:
        if precond_type == "chebyshev":
            raise ValueError("the chebyshev preconditioner is not part of the cuda backend; use amgcl")
        self.reg, self.precond_type, self.max_levels, self.max_coarse = reg, precond_type, max_levels, max_coarse
        nl = C.c_int()
        self._check("mm_build_poisson", lib().mm_build_poisson(self.h, float(reg), _abi.PRECOND[precond_type],
                                                               int(max_levels), int(max_coarse), C.byref(nl)))
        self.poisson_built = True
        self.n_levels = nl.value
        return nl.value

    def amg_levels(self) -> list[dict]:
        import scipy.sparse as sp

        out = []
        for lvl in range(self.n_levels):
            n, nA, nP = C.c_int(), C.c_int64(), C.c_int64()
            self._check("mm_amg_level_info", lib().mm_amg_level_info(self.h, lvl, C.byref(n), C.byref(nA), C.byref(nP)))
            ptr, col, val = np.empty(n.value + 1, np.int32), np.empty(nA.value, np.int32), np.empty(nA.value)
            agg = np.empty(n.value, np.int32)
            self._check("mm_amg_export_level", lib().mm_amg_export_level(self.h, lvl, _abi.iptr(ptr), _abi.iptr(col),
                                                                         dptr(val), _abi.iptr(agg)))
            out.append(dict(A=sp.csr_matrix((val, col, ptr), shape=(n.value, n.value)), agg=agg,
                            nnz_P=int(nP.value)))
        return out

    def apply_A(self, U):
        U = f64(U)
        y = np.empty(self.N)
        self._check("mm_apply_A", lib().mm_apply_A(self.h, dptr(U), dptr(y)))
        return y

    def precond(self, r):
        r = f64(r)
        z = np.empty(self.N)
        self._check("mm_precond", lib().mm_precond(self.h, dptr(r), dptr(z)))
        return z

    def rhs(self, m):
        m = f64(m, (self.N, 3))
        b = np.empty(self.N)
        bb = C.c_double()
        self._check("mm_rhs", lib().mm_rhs(self.h, dptr(m), dptr(b), C.byref(bb)))
        return b, bb.value

    def solve_u(self, m, x0, tol, maxiter=2000, out=None):
        """(U, iterations, rel_res, status).  Torch CUDA tensors are solved in place, without copies.
        Host arrays: `out` (a float64 (N,) array, e.g. in pinned memory) receives U, starting from x0."""
        it, rr = C.c_int(), C.c_double()
        if _is_torch_cuda(m):
            U = x0 if _is_torch_cuda(x0) else None
            if U is None:
                raise TypeError("x0 must be a CUDA tensor when m is one")
            rc = self._check("mm_solve_u_dev", lib().mm_solve_u_dev(self.h, C.c_void_p(m.data_ptr()),
                                                                    C.c_void_p(U.data_ptr()), float(tol), int(maxiter),
                                                                    C.byref(it), C.byref(rr)))
            return U, it.value, rr.value, rc
        m = f64(m, (self.N, 3))
        if out is None:
            U = f64(x0).reshape(-1).copy()
        else:
            if out.dtype != np.float64 or out.shape != (self.N,) or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous float64 array of shape (N,)")
            U = out
            if x0 is not out:  # x0 goes to the device as it is; U lands in `out`
                x0 = f64(x0).reshape(-1)
                if x0.shape != (self.N,):
                    raise ValueError("x0 must have N entries")
                rc = self._check("mm_solve_u_x0", lib().mm_solve_u_x0(self.h, dptr(m), dptr(x0), dptr(U), float(tol),
                                                                      int(maxiter), C.byref(it), C.byref(rr)))
                return U, it.value, rr.value, rc
        rc = self._check("mm_solve_u", lib().mm_solve_u(self.h, dptr(m), dptr(U), float(tol), int(maxiter),
                                                        C.byref(it), C.byref(rr)))
        return U, it.value, rr.value, rc

    # -- energy ------------------------------------------------------------------------------------
    def energy_and_grad(self, m, U, B_ext, B_bias=None):
        B = f64(B_ext).reshape(3)
        E = C.c_double()
        if _is_torch_cuda(m):
            import torch

            g = torch.empty_like(m)
            bias = None if B_bias is None else C.c_void_p(B_bias.data_ptr())
            self._check("mm_energy_grad_dev", lib().mm_energy_grad_dev(self.h, C.c_void_p(m.data_ptr()),
                                                                       C.c_void_p(U.data_ptr()), dptr(B), bias,
                                                                       C.byref(E), C.c_void_p(g.data_ptr())))
            return E.value, g
        m = f64(m, (self.N, 3))
        U = f64(U).reshape(-1)
        bias = None if B_bias is None else f64(B_bias, (self.N, 3))
        g = np.empty((self.N, 3))
        self._check("mm_energy_grad", lib().mm_energy_grad(self.h, dptr(m), dptr(U), dptr(B), dptr(bias),
                                                           C.byref(E), dptr(g)))
        return E.value, g

    def local_grad(self, v):
        v = f64(v, (self.N, 3))
        out = np.empty((self.N, 3))
        self._check("mm_local_grad", lib().mm_local_grad(self.h, dptr(v), dptr(out)))
        return out

    def solve_py_g(self, m, g_ext, g_tan_ext, max_iter, tol=0.0, reg=0.0, stagnation_nu=1e-3):
        """Inner Steihaug PCG of the preconditioned minimizers (the reference's exported
        ``solve_Py_g``, src/cpp/cpp_mkl_minimizer.cpp:233-359): (y (N,3), iterations)."""
        m, ge, gt = f64(m, (self.N, 3)), f64(g_ext, (self.N, 3)), f64(g_tan_ext, (self.N, 3))
        y = np.empty((self.N, 3))
        it = C.c_int()
        self._check("mm_solve_py_g", lib().mm_solve_py_g(self.h, dptr(m), dptr(ge), dptr(gt), int(max_iter),
                                                         float(tol), float(reg), float(stagnation_nu), dptr(y),
                                                         C.byref(it)))
        return y, it.value

    def exchange_diagonal(self):
        d = np.empty(self.N)
        self._check("mm_exchange_diagonal", lib().mm_exchange_diagonal(self.h, dptr(d)))
        return d

    # -- minimizer ---------------------------------------------------------------------------------
    def set_magnetoelastic(self, k1me=None, k1me_p=None):
        """Per-element magnetoelastic constants (reduced units) as make_energy_kernels takes them
        (``src/energy_kernels.py:92-93,212-224``); None removes the term."""
        if k1me is None:
            self._check("mm_set_magnetoelastic", lib().mm_set_magnetoelastic(self.h, 0, None, None))
            return
        a = f64(k1me).reshape(-1)
        b = None if k1me_p is None else f64(k1me_p).reshape(-1)
        if b is not None and b.size < a.size:
            b = np.concatenate([b, np.zeros(a.size - b.size)])
        n = a.size
        if b is not None and b.size > n:
            a = np.concatenate([a, np.zeros(b.size - n)])
            n = b.size
        self._check("mm_set_magnetoelastic", lib().mm_set_magnetoelastic(self.h, n, dptr(a), dptr(b)))

    def set_node_weights(self, inv_M_rel=None, inv_M_prec=None):
        a = None if inv_M_rel is None else f64(inv_M_rel).reshape(-1)
        b = None if inv_M_prec is None else f64(inv_M_prec).reshape(-1)
        self._check("mm_set_node_weights", lib().mm_set_node_weights(self.h, dptr(a), dptr(b)))

    def set_bias_field(self, B_bias=None):
        """Per-node bias field (N,3) added to B_ext in every energy evaluation of minimize (the
        reference's sparse_ops["B_bias"]); None removes it."""
        b = None if B_bias is None else f64(B_bias, (self.N, 3))
        self._check("mm_set_bias_field", lib().mm_set_bias_field(self.h, dptr(b)))

    def minimize(self, B_ext, m0, U0, params: MinimizerParams):
        """Minimize for one applied field: (m, U, info).  Host arrays are copied (the inputs stay
        untouched); float64 CUDA tensors are the state itself, updated in place and returned, so a
        field sweep keeps m and U on the GPU (make_minimizer's minimize copies them first unless it is
        called with inplace=True)."""
        if not self.poisson_built:
            raise RuntimeError("build_poisson() must be called before minimize()")
        B = f64(B_ext).reshape(3)
        info = _abi.MinInfo()
        prm = params.to_c()
        if _is_torch_cuda(m0):
            # device-resident state (a field sweep keeps m and U on the GPU): updated in place
            import torch

            m, U = m0, U0
            if not _is_torch_cuda(U):
                raise TypeError("U0 must be a CUDA tensor when m0 is one")
            if (m.dtype != torch.float64 or U.dtype != torch.float64 or not m.is_contiguous()
                    or not U.is_contiguous() or m.numel() != 3 * self.N or U.numel() != self.N):
                raise ValueError("m0 (N,3) and U0 (N,) must be contiguous float64 CUDA tensors")
            torch.cuda.current_stream().synchronize()  # the caller's writes are complete
            self._check("mm_minimize_dev", lib().mm_minimize_dev(self.h, dptr(B), C.c_void_p(m.data_ptr()),
                                                                 C.c_void_p(U.data_ptr()), C.byref(prm),
                                                                 C.byref(info)))
        else:
            m = f64(m0, (self.N, 3)).copy()
            U = f64(U0).reshape(-1).copy()
            self._check("mm_minimize", lib().mm_minimize(self.h, dptr(B), dptr(m), dptr(U), C.byref(prm),
                                                         C.byref(info)))
        return m, U, dict(iters=info.iters, evals=info.evals, preco_iters=info.preco_iters,
                          demag_iters=info.demag_iters, E=info.E, gnorm=info.gnorm, time=info.seconds,
                          status=info.status, demag_time=info.demag_seconds,
                          demag_wall_time=info.demag_wall_seconds, device_loop=bool(info.device_loop))

    def time_kernel(self, kernel: str, reps: int = 20):
        """(mean ms per launch with L2 flushed before each, algorithmic bytes per launch)."""
        ms, nb = C.c_double(), C.c_double()
        self._check("mm_time_kernel", lib().mm_time_kernel(self.h, _abi.KERNELS[kernel], int(reps), C.byref(ms),
                                                           C.byref(nb)))
        return ms.value, nb.value

    OPTIONS = {"graph": 1, "precision": 2, "mixed_eta_e6": 3, "grid_cap": 4, "profile": 5, "pdl": 8,
               "coarse_fuse": 9, "min_fp32": 10, "split_a0": 11, "fuse_restrict": 12, "energy_ff": 13,
               "min_graph": 14, "energy_ff_lanes": 15, "coarse_cycle": 16, "csr_lanes": 17, "sa_theta_e3": 18,
               "sa_factor_e3": 19, "sa_filter_e6": 20}

    def set_option(self, name: str, value: int):
        self._check("mm_set_option", lib().mm_set_option(self.h, self.OPTIONS[name], int(value)))

    def get_option(self, name: str) -> int:
        """coarse_cycle, fuse_restrict, coarse_fuse, energy_ff_lanes or min_graph as now in effect."""
        v = C.c_int()
        self._check("mm_get_option", lib().mm_get_option(self.h, self.OPTIONS[name], C.byref(v)))
        return v.value

    def autotune(self, reps: int = 20) -> dict:
        """Time the launch shapes of the hierarchy's operators and the fused coarse correction on this
        GPU and keep the fastest (mm_autotune); returns the report."""
        import json

        buf = C.create_string_buffer(1 << 16)
        self._check("mm_autotune", lib().mm_autotune(self.h, int(reps), buf, len(buf)))
        return json.loads(buf.value.decode())

    def set_precision(self, precision: str):
        """"fp64" (the reference's plain method), "mixed" (FP32 correction solves inside FP64 iterative
        refinement) or "fp32_precond" (the FP64 PCG with the V-cycle applied in FP32); call before
        build_poisson()."""
        self.set_option("precision", {"fp64": 0, "mixed": 1, "fp32_precond": 2}[precision])
        self.precision = precision

    def set_inner_precision(self, precision: str):
        """Precision of the minimizer's inner preconditioner solve: "auto" (FP32 when the demag solve
        is not plain FP64), "fp64" or "fp32"."""
        self.set_option("min_fp32", {"auto": -1, "fp64": 0, "fp32": 1}[precision])

    def profile(self, reset: bool = False) -> list[dict]:
        """In-solve kernel profile (set_option("profile", 1) first): one row per used slot with the
        kernel kind, AMG level, precision, launches, total and mean device time and algorithmic bytes
        per launch."""
        n = np.zeros(_abi.PROF_SLOTS, np.int64)
        ms = np.zeros(_abi.PROF_SLOTS)
        nb = np.zeros(_abi.PROF_SLOTS)
        self._check("mm_profile_read", lib().mm_profile_read(self.h, n.ctypes.data_as(_abi._lp), _abi.dptr(ms),
                                                             _abi.dptr(nb)))
        if reset:
            self._check("mm_profile_reset", lib().mm_profile_reset(self.h))
        nk = len(_abi.PROF_KINDS)
        rows = []
        for slot in np.nonzero(n)[0]:
            kind, rest = int(slot) % nk, int(slot) // nk
            level, f32 = rest % _abi.PROF_LEVELS, rest // _abi.PROF_LEVELS
            rows.append({"kernel": _abi.PROF_KINDS[kind], "level": level, "precision": "fp32" if f32 else "fp64",
                         "launches": int(n[slot]), "total_ms": float(ms[slot]),
                         "ms_per_launch": float(ms[slot] / n[slot]), "bytes_per_launch": float(nb[slot])})
        return sorted(rows, key=lambda r: -r["total_ms"])

    def last_refinements(self) -> int:
        n = C.c_int()
        self._check("mm_last_refinements", lib().mm_last_refinements(self.h, C.byref(n)))
        return n.value

    def last_solve_ms(self) -> float:
        ms = C.c_double()
        self._check("mm_last_solve_ms", lib().mm_last_solve_ms(self.h, C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        n = C.c_int64()
        self._check("mm_launch_count", lib().mm_launch_count(self.h, C.byref(n)))
        return n.value

    def sync(self):
        self._check("mm_sync", lib().mm_sync(self.h))


# ------------------------------------------------------------------------------------------------
# one device problem per (mesh, materials), shared by the factories of this package
# ------------------------------------------------------------------------------------------------
def _digest(*arrays) -> str:
    import hashlib

    h = hashlib.sha1()
    for a in arrays:
        if a is None:
            h.update(b"none")
            continue
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64) if not isinstance(a, np.ndarray) else a)
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def problem_for_geom(geom, A_lookup, K1_lookup, Js_lookup, k_easy, V_mag=None, M_nodal=None, boundary_mask=None,
                     n_nodes=None, k1me=None, k1me_p=None) -> Problem:
    """The device problem of a reference-style ``TetGeom`` and material tables (created once).

    V_mag and M_nodal default to the reference's definitions (``src/loop.py:864-939``).
    """
    conn = np.asarray(geom.conn)
    volume = np.asarray(geom.volume, np.float64)
    mat_id = np.asarray(geom.mat_id, np.int32)
    Js = np.asarray(Js_lookup, np.float64).ravel()
    N = int(n_nodes if n_nodes is not None else (geom.x_nodes.shape[0] if getattr(geom, "x_nodes", None) is not None
                                                 else conn.max() + 1))
    if V_mag is None:
        is_mag = np.isin(mat_id, np.where(Js > 0)[0] + 1)
        V_mag = float(np.sum(volume[is_mag])) or 1.0
    if M_nodal is None:
        M_nodal = np.bincount(conn.reshape(-1), weights=np.repeat(0.25 * volume * Js[mat_id - 1], 4), minlength=N)
    M_nodal = np.asarray(M_nodal, np.float64).reshape(-1)
    key = _digest(np.asarray(A_lookup), np.asarray(K1_lookup), Js, np.asarray(k_easy), np.array([V_mag]), M_nodal,
                  None if boundary_mask is None else np.asarray(boundary_mask, np.float64),
                  None if k1me is None else np.asarray(k1me, np.float64),
                  None if k1me_p is None else np.asarray(k1me_p, np.float64))
    cache = getattr(geom, "_mm_problems", None)
    if cache is None:
        cache = {}
        try:
            geom._mm_problems = cache
        except AttributeError:
            pass
    if key not in cache:
        gp = getattr(geom, "grad_phi", None)
        if gp is None:
            JT = np.asarray(geom.JinvT, np.float64)
            ghat = np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
            gp = np.einsum("eij,aj->eai", JT, ghat)
        cache[key] = Problem(conn, volume, np.asarray(gp, np.float64), mat_id, A_lookup, K1_lookup, Js, k_easy,
                             V_mag, M_nodal, boundary_mask, n_nodes=N)
        if k1me is not None or k1me_p is not None:
            cache[key].set_magnetoelastic(np.zeros(1) if k1me is None else k1me, k1me_p)
    return cache[key]
