"""ctypes binding of libmumag_cuda.so (declared in include/mumag_cuda.h).

The library is built in-tree (``python -m mumag_matrixfree2_gb300.build``); loading fails loudly
when it is missing: there is no CPU fallback behind this module.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libmumag_cuda.so"

MM_OK, MM_MAXITER, MM_NONFINITE, MM_BREAKDOWN = 0, 1, 2, 3
PRECOND = {"none": 0, "jacobi": 1, "amg": 2, "amgcl": 3}
METHODS = {"pcohen_hs": 0, "lbfgs": 1, "wg_np": 2, "plbfgs": 3, "cohen": 4, "pcg": 5, "pcohen": 6, "pcohen_exact": 7,
           "pcohen_hs_exact": 8, "dplbfgs": 9, "tn_split": 10, "tr": 11, "ptr": 12, "aapg": 13, "aapg_exact": 14,
           "pnag": 15, "pcohen_lbfgs": 16}
KERNELS = {"spmv_A": 0, "smooth": 1, "energy": 2, "hessian": 3}
# in-solve profile slots: slot = (fp32 * PROF_LEVELS + level) * len(PROF_KINDS) + kind
PROF_KINDS = ("pcg_dir", "pcg_step", "vc_residual0", "residual", "restrict", "coarse", "prolong", "smooth0",
              "smooth", "init_residual", "coarse_a", "coarse_b", "coarse_cycle")
PROF_LEVELS = 16
PROF_SLOTS = 2 * PROF_LEVELS * len(PROF_KINDS)

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_int64)
_vp = C.c_void_p


class MinParams(C.Structure):
    _fields_ = [
        ("method", C.c_int), ("max_iter", C.c_int), ("pc_iters", C.c_int), ("pc_auto", C.c_int),
        ("ls_max_evals", C.c_int), ("L", C.c_int), ("memory", C.c_int), ("wg_gamma", C.c_int),
        ("tau_f", C.c_double), ("eps_a", C.c_double), ("tau0", C.c_double),
        ("ls_eta1", C.c_double), ("ls_eta2", C.c_double), ("ls_C", C.c_double), ("ls_c", C.c_double),
        ("pc_force_eta", C.c_double), ("pc_force_alpha", C.c_double), ("pc_stagnation_nu", C.c_double),
        ("pc_reg", C.c_double), ("cg_tol", C.c_double), ("phi_tol", C.c_double), ("cg_maxiter", C.c_int),
        ("tn_iters", C.c_int), ("lr", C.c_double), ("mu", C.c_double), ("phi_extrapolate", C.c_int),
        ("cpp_semantics", C.c_int),
    ]


class MinInfo(C.Structure):
    _fields_ = [
        ("iters", C.c_int), ("evals", C.c_int), ("preco_iters", C.c_int), ("demag_iters", C.c_int),
        ("E", C.c_double), ("gnorm", C.c_double), ("seconds", C.c_double), ("status", C.c_int),
        ("demag_seconds", C.c_double), ("demag_wall_seconds", C.c_double), ("device_loop", C.c_int),
    ]


# name -> (restype, argtypes); every function declared in include/mumag_cuda.h
SIGNATURES = {
    "mm_version": (C.c_char_p, []),
    "mm_status_str": (C.c_char_p, [C.c_int]),
    "mm_last_error": (C.c_char_p, [_vp]),
    "mm_geom_compute": (C.c_int, [C.c_int, C.c_int, _dp, _ip, _ip, _dp, _dp, _dp]),
    "mm_boundary_mask": (C.c_int, [C.c_int, C.c_int, _ip, _dp]),
    "mm_morton_order": (C.c_int, [C.c_int, C.c_int, _dp, _ip, _ip, _ip]),
    "mm_node_degrees": (C.c_int, [C.c_int, C.c_int, _ip, _ip]),
    "mm_rcm_order": (C.c_int, [C.c_int, C.c_int, _ip, _ip, _ip]),
    "mm_setup_create": (C.c_int, [C.c_int, C.c_int, _ip, _dp, _dp, _ip, C.c_int, _dp, _dp, _dp, _dp, _dp,
                                  C.c_double, C.c_int, C.c_int, C.POINTER(_vp)]),
    "mm_setup_destroy": (C.c_int, [_vp]),
    "mm_setup_energy_info": (C.c_int, [_vp, _ip, _lp, _ip]),
    "mm_setup_energy_export": (C.c_int, [_vp, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp]),
    "mm_setup_levels": (C.c_int, [_vp, _ip]),
    "mm_setup_level_info": (C.c_int, [_vp, C.c_int, _ip, _lp, _lp, _ip]),
    "mm_setup_level_export": (C.c_int, [_vp, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp, _ip]),
    "mm_create": (C.c_int, [C.c_int, C.c_int, _ip, _dp, _dp, _ip, C.c_int, _dp, _dp, _dp, _dp, C.c_double, _dp,
                            _dp, C.POINTER(_vp)]),
    "mm_destroy": (C.c_int, [_vp]),
    "mm_build_poisson": (C.c_int, [_vp, C.c_double, C.c_int, C.c_int, C.c_int, _ip]),
    "mm_amg_level_info": (C.c_int, [_vp, C.c_int, _ip, _lp, _lp]),
    "mm_amg_export_level": (C.c_int, [_vp, C.c_int, _ip, _ip, _dp, _ip]),
    "mm_energy_grad": (C.c_int, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "mm_energy_grad_dev": (C.c_int, [_vp, _vp, _vp, _dp, _vp, _dp, _vp]),
    "mm_energy_grad_noalloc": (C.c_int, [_vp, _vp, _vp, _dp, _vp, _dp, _vp]),
    "mm_local_grad": (C.c_int, [_vp, _dp, _dp]),
    "mm_solve_py_g": (C.c_int, [_vp, _dp, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_double, _dp, _ip]),
    "mm_exchange_diagonal": (C.c_int, [_vp, _dp]),
    "mm_rhs": (C.c_int, [_vp, _dp, _dp, _dp]),
    "mm_apply_A": (C.c_int, [_vp, _dp, _dp]),
    "mm_precond": (C.c_int, [_vp, _dp, _dp]),
    "mm_solve_u": (C.c_int, [_vp, _dp, _dp, C.c_double, C.c_int, _ip, _dp]),
    "mm_solve_u_dev": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int, _ip, _dp]),
    "mm_solve_u_x0": (C.c_int, [_vp, _dp, _dp, _dp, C.c_double, C.c_int, _ip, _dp]),
    "mm_set_node_weights": (C.c_int, [_vp, _dp, _dp]),
    "mm_set_bias_field": (C.c_int, [_vp, _dp]),
    "mm_scale_correction_async": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "mm_scale_correction_dev": (C.c_int, [_vp, _vp, _vp, _vp, _dp]),
    "mm_set_magnetoelastic": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "mm_minimize": (C.c_int, [_vp, _dp, _dp, _dp, C.POINTER(MinParams), C.POINTER(MinInfo)]),
    "mm_minimize_dev": (C.c_int, [_vp, _dp, _vp, _vp, C.POINTER(MinParams), C.POINTER(MinInfo)]),
    "mm_time_kernel": (C.c_int, [_vp, C.c_int, C.c_int, _dp, _dp]),
    "mm_set_option": (C.c_int, [_vp, C.c_int, C.c_int]),
    "mm_get_option": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int)]),
    "mm_autotune": (C.c_int, [_vp, C.c_int, C.c_char_p, C.c_int]),
    "mm_profile_read": (C.c_int, [_vp, _lp, _dp, _dp]),
    "mm_profile_reset": (C.c_int, [_vp]),
    "mm_last_refinements": (C.c_int, [_vp, _ip]),
    "mm_last_solve_ms": (C.c_int, [_vp, _dp]),
    "mm_launch_count": (C.c_int, [_vp, _lp]),
    "mm_sync": (C.c_int, [_vp]),
    # learned warm start
    "mm_unet_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(_vp)]),
    "mm_unet_destroy": (C.c_int, [_vp]),
    "mm_unet_last_error": (C.c_char_p, [_vp]),
    "mm_unet_param_count": (C.c_int, [_vp, _lp]),
    "mm_unet_set_params": (C.c_int, [_vp, _fp]),
    "mm_unet_get_params": (C.c_int, [_vp, _fp]),
    "mm_unet_get_grads": (C.c_int, [_vp, _fp]),
    "mm_unet_forward": (C.c_int, [_vp, _fp, C.c_int, _fp]),
    "mm_unet_forward_dev": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "mm_unet_backward": (C.c_int, [_vp, _fp, C.c_int, _dp]),
    "mm_unet_backward_dev": (C.c_int, [_vp, _vp, C.c_int, _dp]),
    "mm_unet_adam": (C.c_int, [_vp, C.c_float, C.c_float, C.c_float, C.c_float]),
    "mm_unet_set_bias_training": (C.c_int, [_vp, C.c_int]),
    "mm_unet_voxelise_dev": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, C.c_double, C.c_double]),
    "mm_unet_interp_add_dev": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp, _vp, C.c_double, _vp]),
    "mm_unet_tensor_info": (C.c_int, [C.c_int, _ip, _ip]),
    "mm_unet_read_tensor": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _fp]),
    "mm_unet_sync": (C.c_int, [_vp]),
    "mm_unet_predict_dev": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_double,
                                      C.c_int, _vp, _vp, _vp, C.c_double, C.c_int, _vp, C.POINTER(_vp)]),
}

_lib = None


class MMError(RuntimeError):
    """A negative status returned by libmumag_cuda."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn} failed with status {code}: {msg}")
        self.code = code


def lib() -> C.CDLL:
    """Load the in-tree library (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m mumag_matrixfree2_gb300.build` "
                "(the cuda backend has no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(fn: str, rc: int, handle=None) -> int:
    if rc < 0:
        L = lib()
        msg = (L.mm_last_error(handle) or b"").decode() or L.mm_status_str(rc).decode()
        raise MMError(fn, rc, msg)
    return rc


def dptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_dp)


def iptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_ip)


def f64(a, shape=None) -> np.ndarray:
    out = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if shape is not None:
        out = out.reshape(shape)
    return out


def i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


# ------------------------------------------------------------------------------------------------
# setup helpers (host only)
# ------------------------------------------------------------------------------------------------
def geom_compute(knt, conn):
    """(conn_oriented (E,4) i32, volume (E,), JinvT (E,3,3), grad_phi (E,4,3))."""
    knt, conn = f64(knt), i32(np.asarray(conn)[:, :4])
    N, E = knt.shape[0], conn.shape[0]
    co = np.empty((E, 4), np.int32)
    vol, JT, gp = np.empty(E), np.empty((E, 3, 3)), np.empty((E, 4, 3))
    check("mm_geom_compute", lib().mm_geom_compute(N, E, dptr(knt), iptr(conn), iptr(co), dptr(vol), dptr(JT), dptr(gp)))
    return co, vol, JT, gp


def boundary_mask(conn, n_nodes: int) -> np.ndarray:
    conn = i32(np.asarray(conn)[:, :4])
    mask = np.empty(n_nodes)
    check("mm_boundary_mask", lib().mm_boundary_mask(n_nodes, conn.shape[0], iptr(conn), dptr(mask)))
    return mask


def morton_order(knt, conn):
    knt, conn = f64(knt), i32(np.asarray(conn)[:, :4])
    npm, epm = np.empty(knt.shape[0], np.int32), np.empty(conn.shape[0], np.int32)
    check("mm_morton_order", lib().mm_morton_order(knt.shape[0], conn.shape[0], dptr(knt), iptr(conn), iptr(npm), iptr(epm)))
    return npm, epm


def rcm_order(conn, n_nodes):
    """Reverse Cuthill-McKee node and element permutations (the target="cpu" branch of reorder_mesh,
    src/reorder_mesh.py:53-83).  Components start from the nodes in numpy's argsort order of their
    degrees, the order scipy.sparse.csgraph.reverse_cuthill_mckee seeds from; elements are ordered by
    the mean of their nodes' new numbers (numpy argsort, as the reference)."""
    conn = i32(np.asarray(conn)[:, :4])
    deg = np.empty(n_nodes, np.int32)
    check("mm_node_degrees", lib().mm_node_degrees(n_nodes, conn.shape[0], iptr(conn), iptr(deg)))
    seeds = np.ascontiguousarray(np.argsort(deg), dtype=np.int32)
    npm = np.empty(n_nodes, np.int32)
    check("mm_rcm_order", lib().mm_rcm_order(n_nodes, conn.shape[0], iptr(conn), iptr(seeds), iptr(npm)))
    inv = np.empty(n_nodes, np.int32)
    inv[npm] = np.arange(n_nodes, dtype=np.int32)
    epm = np.argsort(np.mean(inv[conn], axis=1)).astype(np.int32)
    return npm, epm


class HostSetup:
    """The product's host-side assembly and SA hierarchy, exported as numpy arrays."""

    def __init__(self, conn, volume, grad_phi, mat_id, A, K1, Js, k_easy, mask=None, reg=1e-12,
                 max_levels=10, max_coarse=1000, n_nodes=None):
        conn, mat_id = i32(conn), i32(mat_id)
        volume, grad_phi = f64(volume), f64(grad_phi)
        A, K1, Js, k_easy = f64(A), f64(K1), f64(Js), f64(k_easy)
        N = int(n_nodes if n_nodes is not None else conn.max() + 1)
        self.N = N
        mask = None if mask is None else f64(mask)
        h = _vp()
        check("mm_setup_create", lib().mm_setup_create(
            N, conn.shape[0], iptr(conn), dptr(volume), dptr(grad_phi), iptr(mat_id), len(A), dptr(A), dptr(K1),
            dptr(Js), dptr(k_easy), dptr(mask), float(reg), int(max_levels), int(max_coarse), C.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.mm_setup_destroy(self.h)
            self.h = None

    def energy_op(self) -> dict:
        L = lib()
        nr, nnz, sa = C.c_int(), C.c_int64(), C.c_int()
        check("mm_setup_energy_info", L.mm_setup_energy_info(self.h, C.byref(nr), C.byref(nnz), C.byref(sa)))
        n, k = nr.value, nnz.value
        out = dict(rows=np.empty(n, np.int32), ptr=np.empty(n + 1, np.int32), col=np.empty(k, np.int32),
                   mat=np.empty(k, np.int32), w=np.empty(k), q=np.empty(k), G=np.empty((k, 3)), D=np.empty((k, 3)),
                   diag_exchange=np.empty(self.N), single_axis=bool(sa.value))
        check("mm_setup_energy_export", L.mm_setup_energy_export(
            self.h, iptr(out["rows"]), iptr(out["ptr"]), iptr(out["col"]), iptr(out["mat"]), dptr(out["w"]),
            dptr(out["q"]), dptr(out["G"]), dptr(out["D"]), dptr(out["diag_exchange"])))
        return out

    def levels(self) -> list[dict]:
        import scipy.sparse as sp

        L = lib()
        nl = C.c_int()
        check("mm_setup_levels", L.mm_setup_levels(self.h, C.byref(nl)))
        res = []
        for lvl in range(nl.value):
            n, nA, nP, nc = C.c_int(), C.c_int64(), C.c_int64(), C.c_int()
            check("mm_setup_level_info", L.mm_setup_level_info(self.h, lvl, C.byref(n), C.byref(nA), C.byref(nP), C.byref(nc)))
            Ap, Ac, Av = np.empty(n.value + 1, np.int32), np.empty(nA.value, np.int32), np.empty(nA.value)
            has_P = nP.value > 0 or lvl < nl.value - 1
            Pp = np.zeros(n.value + 1, np.int32) if has_P else None
            Pc, Pv = np.empty(nP.value, np.int32), np.empty(nP.value)
            agg = np.empty(n.value, np.int32)
            check("mm_setup_level_export", L.mm_setup_level_export(
                self.h, lvl, iptr(Ap), iptr(Ac), dptr(Av), iptr(Pp), iptr(Pc), dptr(Pv), iptr(agg)))
            d = dict(A=sp.csr_matrix((Av, Ac, Ap), shape=(n.value, n.value)), agg=agg)
            if lvl < nl.value - 1:
                d["P"] = sp.csr_matrix((Pv, Pc, Pp), shape=(n.value, nc.value))
            res.append(d)
        return res
