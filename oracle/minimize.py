"""FP64 restatement of the reference's Riemannian minimizers and field sweep.

Test infrastructure (see ``oracle/__init__.py``).  Follows ``src/minimizers.py`` (the JAX path,
which is the GPU reference) and ``src/hysteresis_loop.py``.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def vdot(a, b) -> float:
    return float(np.dot(np.ravel(a), np.ravel(b)))


def cayley_update(m, H, tau):
    """``src/minimizers.py:71-79``."""
    k = 0.5 * tau * H
    k2 = np.sum(k * k, axis=1, keepdims=True)
    km = np.cross(k, m)
    kdotm = np.sum(k * m, axis=1, keepdims=True)
    m_new = ((1.0 - k2) * m + 2.0 * km + 2.0 * kdotm * k) / (1.0 + k2)
    return m_new / np.linalg.norm(m_new, axis=1, keepdims=True)


def cayley_transport(v, H, tau):
    """``src/minimizers.py:82-91``."""
    k = 0.5 * tau * H
    k2 = np.sum(k * k, axis=1, keepdims=True)
    kv = np.cross(k, v)
    kdotv = np.sum(k * v, axis=1, keepdims=True)
    return ((1.0 - k2) * v + 2.0 * kv + 2.0 * kdotv * k) / (1.0 + k2)


def tangent_grad(m, g):
    """``src/minimizers.py:94-96``."""
    return g - np.sum(m * g, axis=1, keepdims=True) * m


def check_convergence(it, E, E_prev, m, m_new, gnorm_inf, tau_f, eps_a) -> bool:
    """Gill-Murray-Wright U1-U4, ``src/minimizers.py:160-172``."""
    if it <= 0:
        return False
    diff = float(np.max(np.abs(m_new - m)))
    u1 = (E_prev - E) < tau_f * (1.0 + abs(E))
    u2 = diff < math.sqrt(tau_f) * 2.0
    u3 = gnorm_inf <= (tau_f ** (1.0 / 3.0)) * (1.0 + abs(E))
    u4 = gnorm_inf < eps_a
    return bool((u1 and u2 and u3) or u4)


@dataclass
class Ops:
    """The callables a minimizer needs (all FP64 numpy)."""

    energy_and_grad: object  # (m, U, B) -> (E, g)
    local_grad_only: object  # v -> C v
    solve_U: object  # (m, x0, tol) -> (U, it, rel_res)
    inv_M_rel: np.ndarray  # (N,1)
    inv_M_prec: np.ndarray  # (N,1)


def armijo_ls(ops: Ops, m, pg, H, E0, U_base, g_raw_init, B, phi_tol, eta1, eta2, C, c, s0, max_evals):
    """Curvilinear Armijo search returning (tau, E, g_raw, U, m, evals, demag), ``src/minimizers.py:265-385``."""

    def D(s, U_guess):
        m_t = cayley_update(m, H, s)
        U_t, it_d, _ = ops.solve_U(m_t, U_guess, phi_tol)
        E_t, g_t = ops.energy_and_grad(m_t, U_t, B)
        if not np.isfinite(E_t):
            E_t = 1e20
        return (E_t - E0) / (s * pg + 1e-30), E_t, g_t, U_t, m_t, it_d

    if pg >= 0:
        return 0.0, E0, g_raw_init, U_base, m, 0, 0
    s, s_min, it_exp, done = s0, 0.0, 0, False
    E_v, g_v, U_v, m_v, d_v, demag = E0, g_raw_init, U_base, m, 0.0, 0
    while it_exp < max_evals and not done:
        d, E_v, g_v, U_v, m_v, itd = D(s, U_v)
        d_v = d
        demag += itd
        stop = (abs(1.0 - d) >= eta2) or (d < 0)
        if not stop:
            s_min = s
            s = C * s
        it_exp += 1
        done = stop
    it_con = 0
    done = (d_v >= eta1) and (d_v < 1e10)
    while it_con < max_evals and not done:
        s = s_min + c * (s - s_min)
        d, E_v, g_v, U_v, m_v, itd = D(s, U_v)
        d_v = d
        demag += itd
        done = (d >= eta1) and (d < 1e10)
        it_con += 1
    if d_v >= 0:
        return s, E_v, g_v, U_v, m_v, it_exp + it_con, demag
    return 0.0, E0, g_raw_init, U_base, m, it_exp + it_con, demag


def apply_P(ops: Ops, m, g_ext, v, reg=0.0):
    """Extensive local Hessian action, ``src/minimizers.py:396-411``."""
    Cv = ops.local_grad_only(v)
    return Cv - np.sum(m * Cv, axis=1, keepdims=True) * m - np.sum(m * g_ext, axis=1, keepdims=True) * v + reg * v


def solve_Py_g(ops: Ops, m, g_ext, g_tan_ext, max_iter=20, tol=0.0, reg=0.0, stagnation_nu=1e-3, cpp_count=False):
    """Inner PCG with Steihaug exit; returns (y, iterations), ``src/minimizers.py:413-490``.

    The JAX path counts the trip that exits on negative curvature or stagnation; the C++ path
    (``src/cpp/cpp_mkl_minimizer.cpp:277-309``) leaves the loop before counting it: ``cpp_count``
    returns that count.
    """
    y = np.zeros_like(g_tan_ext)
    r = g_tan_ext.copy()
    z = r * ops.inv_M_prec
    p = z.copy()
    rho = vdot(r, z)
    target = tol * tol * rho
    Q, it, done = 0.0, 0, False
    while it < max_iter and rho > target and rho > 1e-25 and rho < 1e20 and not done:
        Ap = apply_P(ops, m, g_ext, p, reg)
        pAp = vdot(p, Ap)
        neg = pAp <= 0.0
        alpha = rho / (pAp + 1e-30)
        dq = 0.5 * alpha * rho
        stag = (it > 0) and (dq <= stagnation_nu * Q)
        done = neg or stag
        if not done:
            y = y + alpha * p
            r = r - alpha * Ap
        z = r * ops.inv_M_prec
        rho_next = vdot(r, z)
        if not done:
            p = z + (rho_next / (rho + 1e-30)) * p
        rho = rho_next
        Q = Q + dq
        it += 1
    if cpp_count and done:
        it -= 1
    z_fb = g_tan_ext * ops.inv_M_prec
    yn, zn = float(np.linalg.norm(y)), float(np.linalg.norm(z_fb))
    if yn > 10.0 * zn:
        y = y * (10.0 * zn / (yn + 1e-30))
    if not vdot(y, g_tan_ext) > 1e-12:
        y = z_fb
    return y, it


@dataclass
class Params:
    """Minimizer parameters as ``src/loop.py:945-979`` passes them (CLI defaults)."""

    max_iter: int = 2000
    tau_f: float = 1e-8
    eps_a: float = 1e-12
    tau0: float = 1e-2
    ls_eta1: float = 0.1
    ls_eta2: float = 0.1
    ls_C: float = 2.0
    ls_c: float = 0.5
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
    tn_iters: int = 5
    lr: float = 0.1
    mu: float = 0.9
    phi_extrapolate: bool = True

    @property
    def phi_tol(self) -> float:
        """``src/minimizers.py:3447-3452``."""
        return float(min(self.cg_tol, self.tau_f * 0.1))


METHODS = ("pcohen_hs", "lbfgs", "wg_np", "plbfgs", "cohen", "pcg", "pcohen", "pcohen_exact", "pcohen_hs_exact",
           "dplbfgs", "tn_split", "tr", "ptr", "aapg", "aapg_exact", "pnag", "pcohen_lbfgs")


def minimize(ops: Ops, m0, B, U0, prm: Params, method="pcohen_hs", flavour="jax"):
    """``make_minimizer(...).minimize``: init (``src/minimizers.py:3408-3435``, with each method's
    ``init_state_fn``, ``:2993-3400``) then the step loop.

    ``flavour="cpp"`` (methods "pcohen_hs" and "pcohen") follows the reference's C++ minimizer,
    ``run_cpp_pcohen_hs_minimization`` (``src/cpp/cpp_mkl_minimizer.cpp:542-763``), where it differs
    from the JAX path:

    * an inner solve on the initial state is counted in ``preco_iters`` (``:606-611``);
    * inner iterations are counted as the C++ loop counts them (see ``solve_Py_g``);
    * the convergence test compares the new energy with the energy two iterations back: ``E_prev``
      is assigned the current energy only after the test (``:620,723-726``).

    Returns (m, U, info) with info keys iters, E, gnorm, preco_iters, evals, demag_iters.
    """
    if method not in METHODS:
        raise NotImplementedError(method)
    if flavour not in ("jax", "cpp") or (flavour == "cpp" and method not in ("pcohen_hs", "pcohen")):
        raise NotImplementedError(f"{method} with flavour {flavour}")
    m = m0 / np.linalg.norm(m0, axis=1, keepdims=True)
    U, init_demag, _ = ops.solve_U(m, U0, prm.cg_tol)
    E, g_raw = ops.energy_and_grad(m, U, B)
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm = float(np.max(np.abs(g_tan)))
    N = m.shape[0]
    L = prm.L or N
    st = dict(m=m, U=U, U_prev=U, g=g_tan_ext, g_raw=g_raw, y=g_tan_ext, d=-g_tan_ext, E=E, gnorm=gnorm, it=0,
              conv=False, evals=1, preco=0, demag=int(init_demag), cpp=flavour == "cpp", E_lag=E)
    if flavour == "cpp":
        y0, pc0 = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, _pc_tol(prm, gnorm), prm.pc_reg,
                             prm.pc_stagnation_nu, cpp_count=True)
        st.update(y=y0, d=-y0, preco=pc0)
    mem = prm.memory
    hist = dict(S=np.zeros((mem, N, 3)), Y=np.zeros((mem, N, 3)), rho=np.zeros(mem), hist_it=0)
    if method in ("lbfgs", "plbfgs", "dplbfgs"):
        st.update(g=g_tan, **hist)
    elif method == "wg_np":
        st.update(g=g_tan, m_prev=m, g_tan_prev=g_tan)
    elif method == "cohen":
        st.update(y=g_tan, d=-g_tan, E_last=E)
    elif method in ("pcohen_exact", "pcohen_hs_exact"):
        st.update(g=g_tan, z=g_tan, d=-g_tan, H_prev=np.zeros_like(m), tau_prev=1.0)
    elif method == "tn_split":
        # TNState is built without the counters, so they start at zero (src/minimizers.py:3198-3203)
        st.update(g=g_tan, d=-g_tan, evals=0, demag=0)
    elif method in ("tr", "ptr"):
        st.update(delta=10.0)
    elif method == "aapg":
        st.update(F_prev=np.zeros_like(m))
    elif method == "aapg_exact":
        st.update(F_prev=np.zeros_like(m), H_prev=np.zeros_like(m), tau_prev=0.0)
    elif method == "pnag":
        st.update(v=np.zeros_like(m))
    elif method == "pcohen_lbfgs":
        st.update(z=g_tan_ext, p=-g_tan_ext, **hist)
    phi_tol = prm.phi_tol
    while not st["conv"] and st["it"] < prm.max_iter:
        if method in ("pcohen_hs", "pcohen", "pcg"):
            _pcohen_hs_step(ops, st, B, prm, phi_tol, L, variant=method)
        elif method == "lbfgs":
            _lbfgs_step(ops, st, B, prm, phi_tol)
        elif method == "wg_np":
            _wg_np_step(ops, st, B, prm, phi_tol)
        elif method == "plbfgs":
            _plbfgs_step(ops, st, B, prm, phi_tol)
        elif method == "dplbfgs":
            _dplbfgs_step(ops, st, B, prm, phi_tol)
        elif method == "cohen":
            _cohen_step(ops, st, B, prm, phi_tol, L)
        elif method in ("pcohen_exact", "pcohen_hs_exact"):
            _pcohen_exact_step(ops, st, B, prm, phi_tol, L, hs=method == "pcohen_hs_exact")
        elif method == "tn_split":
            _tn_split_step(ops, st, B, prm, phi_tol)
        elif method == "tr":
            _tr_step(ops, st, B, prm, phi_tol)
        elif method == "ptr":
            _ptr_step(ops, st, B, prm, phi_tol)
        elif method == "aapg":
            _aapg_step(ops, st, B, prm, phi_tol)
        elif method == "aapg_exact":
            _aapg_exact_step(ops, st, B, prm, phi_tol)
        elif method == "pnag":
            _pnag_step(ops, st, B, prm, phi_tol)
        else:
            _pcohen_lbfgs_step(ops, st, B, prm, phi_tol, L)
    info = dict(iters=st["it"], E=float(st["E"]), gnorm=float(st["gnorm"]), preco_iters=st["preco"],
                evals=st["evals"], demag_iters=st["demag"])
    return st["m"], st["U"], info


def _pc_tol(prm: Params, gnorm_inf: float) -> float:
    """Eisenstat-Walker forcing of the inner solve's accuracy (``src/minimizers.py:982-985``)."""
    return min(prm.pc_force_eta, gnorm_inf ** prm.pc_force_alpha) if prm.pc_auto else 0.0


def _ls(ops, st, B, prm, phi_tol, d, s0, m=None, E0=None, U=None, g_raw=None):
    """H = m x d, pg = g_raw . d and the Armijo search from (m, U, g_raw) (``src/minimizers.py:1022-1045``)."""
    m = st["m"] if m is None else m
    g_raw = st["g_raw"] if g_raw is None else g_raw
    H = np.cross(m, d)  # -cross(m, -d)
    pg = vdot(g_raw, d)
    out = armijo_ls(ops, m, pg, H, st["E"] if E0 is None else E0, st["U"] if U is None else U, g_raw, B, phi_tol,
                    prm.ls_eta1, prm.ls_eta2, prm.ls_C, prm.ls_c, s0, 15)
    return (H,) + out


def _pcohen_hs_step(ops, st, B, prm, phi_tol, L, variant="pcohen_hs"):
    """Preconditioned CG steps: "pcohen_hs" (Hestenes-Stiefel beta, ``src/minimizers.py:962-1071``),
    "pcohen" (Polak-Ribiere beta over the previous smoothed gradient, same lines) and "pcg" (HS beta,
    previous direction not re-projected, ``:839-947``)."""
    m, U, g_prev, g_raw, d_prev, E_prev = st["m"], st["U"], st["g"], st["g_raw"], st["d"], st["E"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    pc_tol = _pc_tol(prm, gnorm_inf)
    cpp = st.get("cpp", False)
    y, preco_it = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, pc_tol, prm.pc_reg, prm.pc_stagnation_nu,
                             cpp_count=cpp)
    gnorm_smooth = float(np.max(np.abs(y)))
    diff_g = g_tan_ext - g_prev
    if variant == "pcohen":
        num = vdot(y, diff_g)
        den = vdot(st["y"], g_prev) + 1e-30
    else:
        num = vdot(y, diff_g)
        den = vdot(d_prev, diff_g) + 1e-30
    beta = 0.0 if st["it"] % L == 0 else max(0.0, num / den)
    d = -y + beta * (d_prev if variant == "pcg" else tangent_grad(m, d_prev))
    if vdot(d, g_tan_ext) > 0:
        d = -y
    H = np.cross(m, d)  # -cross(m, -d)
    pg = vdot(g_raw, d)
    tau, E_new, g_new, U_new, m_new, ev, dem = armijo_ls(
        ops, m, pg, H, E_prev, U, g_raw, B, phi_tol, prm.ls_eta1, prm.ls_eta2, prm.ls_C, prm.ls_c, 1.0, 15)
    conv = check_convergence(st["it"], E_new, st["E_lag"] if cpp else E_prev, m, m_new, gnorm_smooth, prm.tau_f,
                             prm.eps_a)
    st.update(m=m_new, U=U_new, g=g_tan_ext, g_raw=g_new, y=y, d=d, E=E_new, gnorm=gnorm_smooth,
              it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, preco=st["preco"] + preco_it,
              demag=st["demag"] + dem, tau=tau, E_lag=E_prev)


def _lbfgs_step(ops, st, B, prm, phi_tol):
    """L-BFGS two-loop with tangent-space history transport, ``src/minimizers.py:1276-1379``."""
    mem = prm.memory
    m, U, E_prev, g_raw = st["m"], st["U"], st["E"], st["g_raw"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    S, Y, rho, hit = st["S"], st["Y"], st["rho"], st["hist_it"]
    n_hist = min(hit, mem)
    alphas = np.zeros(mem)
    q = g_tan_ext.copy()
    for i in range(n_hist):
        idx = (hit - 1 - i) % mem
        a = rho[idx] * vdot(S[idx], q)
        q = q - a * Y[idx]
        alphas[idx] = a
    last = (hit - 1) % mem
    if hit > 0:
        gamma = vdot(S[last], Y[last]) / (vdot(Y[last], Y[last] * ops.inv_M_rel) + 1e-30)
    else:
        gamma = 1.0
    gamma = min(max(gamma, 1e-3), 1e3)
    r = gamma * q * ops.inv_M_rel
    for i in range(n_hist):
        idx = (hit - n_hist + i) % mem
        b = rho[idx] * vdot(Y[idx], r)
        r = r + S[idx] * (alphas[idx] - b)
    d = -r
    if st["it"] == 0 or vdot(d, g_tan_ext) > 0:
        d = -g_tan
    H = np.cross(m, d)
    pg = vdot(g_raw, d)
    tau_init = prm.tau0 if st["it"] == 0 else 1.0
    tau, E_new, g_new, U_new, m_new, ev, dem = armijo_ls(
        ops, m, pg, H, E_prev, U, g_raw, B, phi_tol, prm.ls_eta1, prm.ls_eta2, prm.ls_C, prm.ls_c, tau_init, 15)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_inf, prm.tau_f, prm.eps_a)
    g_tan_new = tangent_grad(m_new, g_new * ops.inv_M_rel)
    s_new = tangent_grad(m_new, d * tau)
    y_new = tangent_grad(m_new, g_new) - tangent_grad(m_new, g_tan_ext)
    curv = vdot(y_new, s_new)
    ok = curv > 1e-12 * vdot(s_new, s_new)
    idx = hit % mem
    S = np.stack([tangent_grad(m_new, h) for h in S])
    Y = np.stack([tangent_grad(m_new, h) for h in Y])
    rho = rho.copy()
    if ok:
        S[idx], Y[idx], rho[idx] = s_new, y_new, 1.0 / (curv + 1e-30)
    st.update(m=m_new, U=U_new, g=g_tan_new, g_raw=g_new, S=S, Y=Y, rho=rho, E=E_new, gnorm=gnorm_inf,
              it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, demag=st["demag"] + dem,
              hist_it=hit + 1 if ok else hit, tau=tau)


def _plbfgs_step(ops, st, B, prm, phi_tol):
    """Preconditioned L-BFGS, ``src/minimizers.py:1526-1653``: the two-loop recursion's initial Hessian
    is the inner-PCG solve P^-1 (``solve_Py_g``), convergence uses the smoothed gradient y = P^-1 g_tan_ext,
    the fallback direction is -y, and the preconditioner count grows by one per iteration."""
    mem = prm.memory
    m, U, E_prev, g_raw = st["m"], st["U"], st["E"], st["g_raw"]
    g_tan_ext = tangent_grad(m, g_raw)
    y, _ = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, 0.0, 0.0, prm.pc_stagnation_nu)
    gnorm_smooth = float(np.max(np.abs(y)))
    S, Y, rho, hit = st["S"], st["Y"], st["rho"], st["hist_it"]
    n_hist = min(hit, mem)
    alphas = np.zeros(mem)
    q = g_tan_ext.copy()
    for i in range(n_hist):
        idx = (hit - 1 - i) % mem
        a = rho[idx] * vdot(S[idx], q)
        q = q - a * Y[idx]
        alphas[idx] = a
    r, _ = solve_Py_g(ops, m, g_raw, q, prm.pc_iters, 0.0, prm.pc_reg, prm.pc_stagnation_nu)
    for i in range(n_hist):
        idx = (hit - n_hist + i) % mem
        b = rho[idx] * vdot(Y[idx], r)
        r = r + S[idx] * (alphas[idx] - b)
    d = -r
    if st["it"] == 0 or vdot(d, g_tan_ext) > 0:
        d = -y
    H = np.cross(m, d)
    pg = vdot(g_raw, d)
    tau_init = prm.tau0 if st["it"] == 0 else 1.0
    tau, E_new, g_new, U_new, m_new, ev, dem = armijo_ls(
        ops, m, pg, H, E_prev, U, g_raw, B, phi_tol, prm.ls_eta1, prm.ls_eta2, prm.ls_C, prm.ls_c, tau_init, 15)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    s_new = tangent_grad(m_new, d * tau)
    y_new = tangent_grad(m_new, g_new) - tangent_grad(m_new, g_tan_ext)
    curv = vdot(y_new, s_new)
    ok = curv > 1e-12 * vdot(s_new, s_new)
    idx = hit % mem
    S = np.stack([tangent_grad(m_new, h) for h in S])
    Y = np.stack([tangent_grad(m_new, h) for h in Y])
    rho = rho.copy()
    if ok:
        S[idx], Y[idx], rho[idx] = s_new, y_new, 1.0 / (curv + 1e-30)
    st.update(m=m_new, U=U_new, g_raw=g_new, S=S, Y=Y, rho=rho, E=E_new, gnorm=gnorm_smooth,
              it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, preco=st["preco"] + 1, demag=st["demag"] + dem,
              hist_it=hit + 1 if ok else hit, tau=tau)


def _wg_np_step(ops, st, B, prm, phi_tol):
    """Barzilai-Borwein curvilinear step (Wen-Goldfarb), ``src/minimizers.py:1715-1798``."""
    m, U, E_prev, g_raw = st["m"], st["U"], st["E"], st["g_raw"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    z = g_tan
    s_d = (m - st["m_prev"]).reshape(-1)
    y_d = (g_tan - st["g_tan_prev"]).reshape(-1)
    sty, sts, yty = vdot(s_d, y_d), vdot(s_d, s_d), vdot(y_d, y_d)
    tau1 = sts / (sty + 1e-30)
    tau2 = sty / (yty + 1e-30)
    tau_bb = tau1 if st["it"] % 2 != 0 else tau2
    tau_bb = min(max(abs(tau_bb), 1e-6), 1e3)
    H = -np.cross(m, z)
    pg = -vdot(g_raw, z)
    if st["it"] < prm.wg_gamma:
        tau, E_new, g_new, U_new, m_new, ev, dem = armijo_ls(
            ops, m, pg, H, E_prev, U, g_raw, B, phi_tol, prm.ls_eta1, prm.ls_eta2, prm.ls_C, prm.ls_c, 1.0, 15)
    else:
        m_new = cayley_update(m, H, tau_bb)
        U_new, dem, _ = ops.solve_U(m_new, U, phi_tol)
        E_new, g_new = ops.energy_and_grad(m_new, U_new, B)
        tau, ev = tau_bb, 1
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_inf, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g=g_tan, g_raw=g_new, m_prev=m, g_tan_prev=g_tan, E=E_new, gnorm=gnorm_inf,
              it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, demag=st["demag"] + int(dem), tau=tau)


def _m_rel(ops: Ops):
    """M_rel = 1 / inv_M_rel where inv_M_rel > 1e-20, else 0 (``src/hysteresis_loop.py:353``)."""
    imr = ops.inv_M_rel
    return np.where(imr > 1e-20, 1.0 / np.where(imr > 1e-20, imr, 1.0), 0.0)


def _history_update(st, m_new, s_new, y_new, mem):
    """Re-project the (s, y) history onto T_m_new and store the new pair when its curvature is
    positive enough (``src/minimizers.py:1342-1360``)."""
    curv = vdot(y_new, s_new)
    ok = curv > 1e-12 * vdot(s_new, s_new)
    hit = st["hist_it"]
    S = np.stack([tangent_grad(m_new, h) for h in st["S"]])
    Y = np.stack([tangent_grad(m_new, h) for h in st["Y"]])
    rho = st["rho"].copy()
    if ok:
        idx = hit % mem
        S[idx], Y[idx], rho[idx] = s_new, y_new, 1.0 / (curv + 1e-30)
    st.update(S=S, Y=Y, rho=rho, hist_it=hit + 1 if ok else hit)


def _two_loop(st, q, mem, initial):
    """L-BFGS two-loop recursion over the stored pairs; ``initial`` maps the first loop's result to
    the initial-Hessian product (``src/minimizers.py:1284-1312``)."""
    S, Y, rho, hit = st["S"], st["Y"], st["rho"], st["hist_it"]
    n_hist = min(hit, mem)
    alphas = np.zeros(mem)
    q = q.copy()
    for i in range(n_hist):
        idx = (hit - 1 - i) % mem
        a = rho[idx] * vdot(S[idx], q)
        q = q - a * Y[idx]
        alphas[idx] = a
    r = initial(q)
    for i in range(n_hist):
        idx = (hit - n_hist + i) % mem
        b = rho[idx] * vdot(Y[idx], r)
        r = r + S[idx] * (alphas[idx] - b)
    return r


def _cohen_step(ops, st, B, prm, phi_tol, L):
    """Cohen CG (Polak-Ribiere beta on the mass-scaled tangent gradient, energy-based initial step),
    ``src/minimizers.py:646-720``."""
    m, g_prev, g_raw, y_prev, d_prev, E_prev = st["m"], st["g"], st["g_raw"], st["y"], st["d"], st["E"]
    g_tan_ext = tangent_grad(m, g_raw)
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    y = g_tan
    num = vdot(y, g_tan_ext - g_prev)
    den = vdot(y_prev, g_prev) + 1e-30
    beta = 0.0 if st["it"] % L == 0 else max(0.0, num / den)
    d = -y + beta * tangent_grad(m, d_prev)
    if vdot(d, g_tan_ext) > 0:
        d = -y
    pg = vdot(g_raw, d)
    tau_a = 2.0 * (st["E"] - st["E_last"]) / (-pg + 1e-30)
    tau_a = min(1.0, 1.01 * abs(tau_a))
    tau_a = min(max(tau_a, 1e-4), 10.0)
    s0 = tau_a if st["it"] > 0 else prm.tau0
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, d, s0)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_inf, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g=g_tan_ext, g_raw=g_new, y=y, d=d, E=E_new, E_last=E_prev, gnorm=gnorm_inf,
              it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, demag=st["demag"] + dem, tau=tau)


def _pcohen_exact_step(ops, st, B, prm, phi_tol, L, hs):
    """Preconditioned Cohen CG with Cayley transport of the previous direction and gradient
    (``src/minimizers.py:1093-1200``; PR beta, or HS with ``hs``).  The PR denominator uses the
    previous smoothed gradient untransported, as the reference does."""
    m, g_prev, g_raw, z_prev, d_prev, E_prev = st["m"], st["g"], st["g_raw"], st["z"], st["d"], st["E"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    z, preco_it = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, _pc_tol(prm, gnorm_inf), prm.pc_reg,
                             prm.pc_stagnation_nu)
    gnorm_smooth = float(np.max(np.abs(z)))
    if st["it"] > 0:
        d_t = cayley_transport(d_prev, st["H_prev"], st["tau_prev"])
        g_t = cayley_transport(g_prev, st["H_prev"], st["tau_prev"])
    else:
        d_t, g_t = np.zeros_like(d_prev), np.zeros_like(g_prev)
    diff_g = g_tan_ext - g_t
    num = vdot(z, diff_g)
    den = (vdot(d_t, diff_g) if hs else vdot(z_prev, g_t)) + 1e-30
    beta = 0.0 if st["it"] % L == 0 else max(0.0, num / den)
    d = -z + beta * d_t
    if vdot(d, g_tan_ext) > 0:
        d = -z
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, d, 1.0)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g=g_tan_ext, g_raw=g_new, z=z, d=d, E=E_new, gnorm=gnorm_smooth, H_prev=H,
              tau_prev=tau, it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, preco=st["preco"] + preco_it,
              demag=st["demag"] + dem, tau=tau)


def _tn_split_step(ops, st, B, prm, phi_tol):
    """Split truncated Newton: the inner Steihaug PCG solves P d = -g_tan_ext for the step
    (``src/minimizers.py:1448-1517``)."""
    m, g_raw, E_prev = st["m"], st["g_raw"], st["E"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    d, pc_it = solve_Py_g(ops, m, g_raw, -g_tan_ext, prm.pc_iters, _pc_tol(prm, gnorm_inf), prm.pc_reg,
                          prm.pc_stagnation_nu)
    s0 = prm.tau0 if st["it"] == 0 else 1.0
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, d, s0)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_inf, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g=g_tan, g_raw=g_new, d=d, E=E_new, gnorm=gnorm_inf, it=st["it"] + 1, conv=conv,
              evals=st["evals"] + ev, preco=st["preco"] + pc_it, demag=st["demag"] + dem, tau=tau)


def _dplbfgs_step(ops, st, B, prm, phi_tol):
    """Damped preconditioned L-BFGS (``src/minimizers.py:1820-1968``): P^-1 as the initial Hessian,
    Powell damping of y against B0 s = P s, and m_new recomputed by the Cayley map at the accepted step."""
    mem = prm.memory
    m, g_raw, E_prev = st["m"], st["g_raw"], st["E"]
    g_tan_ext = tangent_grad(m, g_raw)
    y, _ = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, 0.0, 0.0, prm.pc_stagnation_nu)
    gnorm_smooth = float(np.max(np.abs(y)))
    r = _two_loop(st, g_tan_ext, mem,
                  lambda q: solve_Py_g(ops, m, g_raw, q, prm.pc_iters, 0.0, prm.pc_reg, prm.pc_stagnation_nu)[0])
    d = -r
    if st["it"] == 0 or vdot(d, g_tan_ext) > 0:
        d = -y
    s0 = prm.tau0 if st["it"] == 0 else 1.0
    H, tau, E_new, g_new, U_new, _, ev, dem = _ls(ops, st, B, prm, phi_tol, d, s0)
    m_new = cayley_update(m, H, tau)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    s_k = tangent_grad(m_new, d * tau)
    y_k = tangent_grad(m_new, g_new) - tangent_grad(m_new, g_tan_ext)
    B0s = apply_P(ops, m_new, g_new, s_k)
    sy, sBs = vdot(s_k, y_k), vdot(s_k, B0s)
    theta = 1.0 if sy >= 0.2 * sBs else 0.8 * sBs / (sBs - sy + 1e-30)
    _history_update(st, m_new, s_k, theta * y_k + (1.0 - theta) * B0s, mem)
    st.update(m=m_new, U=U_new, g_raw=g_new, E=E_new, gnorm=gnorm_smooth, it=st["it"] + 1, conv=conv,
              evals=st["evals"] + ev, preco=st["preco"] + 2, demag=st["demag"] + dem, tau=tau)


def _aapg_step(ops, st, B, prm, phi_tol):
    """Anderson-accelerated preconditioned gradient, depth one over the previous smoothed gradient
    (``src/minimizers.py:2519-2636``; the accelerated m is not used by the step)."""
    m, g_raw, E_prev = st["m"], st["g_raw"], st["E"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    z, pc_it = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, _pc_tol(prm, gnorm_inf), prm.pc_reg,
                          prm.pc_stagnation_nu)
    gnorm_smooth = float(np.max(np.abs(z)))
    z_aa = z
    if st["it"] > 1:
        dF = z - st["F_prev"]
        gamma = vdot(z, dF) / (vdot(dF, dF) + 1e-30)
        z_aa = z - gamma * dF
    d = -z_aa
    if vdot(d, g_tan_ext) > 0:
        d = -z
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, d, 1.0)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g_raw=g_new, E=E_new, gnorm=gnorm_smooth, F_prev=z, it=st["it"] + 1, conv=conv,
              evals=st["evals"] + ev, preco=st["preco"] + pc_it, demag=st["demag"] + dem, tau=tau)


def _aapg_exact_step(ops, st, B, prm, phi_tol):
    """Anderson acceleration with the previous smoothed gradient moved by Cayley transport
    (``src/minimizers.py:2407-2504``)."""
    m, g_raw, E_prev = st["m"], st["g_raw"], st["E"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    z, pc_it = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, _pc_tol(prm, gnorm_inf), prm.pc_reg,
                          prm.pc_stagnation_nu)
    F_t = cayley_transport(st["F_prev"], st["H_prev"], st["tau_prev"]) if st["it"] > 0 else st["F_prev"]
    dF = z - F_t
    gamma = vdot(z, dF) / (vdot(dF, dF) + 1e-30)
    z_next = z - gamma * dF if st["it"] > 1 else z
    d = -z_next
    if vdot(d, g_tan_ext) > 0:
        d = -z
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, d, 1.0)
    gn = float(np.max(np.abs(z_next)))
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gn, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g_raw=g_new, E=E_new, gnorm=gn, F_prev=z, H_prev=H, tau_prev=tau, it=st["it"] + 1,
              conv=conv, evals=st["evals"] + ev, preco=st["preco"] + pc_it, demag=st["demag"] + dem, tau=tau)


def _pnag_step(ops, st, B, prm, phi_tol):
    """Preconditioned Nesterov accelerated gradient on the sphere (``src/minimizers.py:2726-2803``):
    gradient at the Cayley look-ahead m_look = R(m, -(m x v), mu), line search along
    mu P_m(v) - P_m(z) from m."""
    m, U, v_prev, g_raw, E_prev = st["m"], st["U"], st["v"], st["g_raw"], st["E"]
    mu = prm.mu
    m_look = cayley_update(m, -np.cross(m, v_prev), mu)
    U_guess = 2.0 * U - st["U_prev"] if (prm.phi_extrapolate and st["it"] > 0) else U
    U_look, it_look, _ = ops.solve_U(m_look, U_guess, phi_tol)
    _, g_look = ops.energy_and_grad(m_look, U_look, B)
    g_tan_look_ext = tangent_grad(m_look, g_look)
    z, pc_it = solve_Py_g(ops, m_look, g_look, g_tan_look_ext, prm.pc_iters, 0.0, prm.pc_reg, prm.pc_stagnation_nu)
    gnorm_smooth = float(np.max(np.abs(z)))
    v_dir = mu * tangent_grad(m, v_prev) - tangent_grad(m, z)
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, v_dir, prm.lr)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, U_prev=U, v=tau * v_dir, g_raw=g_new, E=E_new, gnorm=gnorm_smooth, it=st["it"] + 1,
              conv=conv, evals=st["evals"] + ev + 1, preco=st["preco"] + pc_it,
              demag=st["demag"] + dem + int(it_look), tau=tau)


def _pcohen_lbfgs_step(ops, st, B, prm, phi_tol, L):
    """Cohen CG (PR beta) on the L-BFGS-smoothed gradient (``src/minimizers.py:2816-2924``)."""
    mem = prm.memory
    m, g_raw, E_prev = st["m"], st["g_raw"], st["E"]
    g_tan_ext = tangent_grad(m, g_raw)
    hit = st["hist_it"]

    def initial(q):
        gamma = 1.0
        if hit > 0:
            last = (hit - 1) % mem
            gamma = vdot(st["S"][last], st["Y"][last]) / (vdot(st["Y"][last], st["Y"][last] * ops.inv_M_rel) + 1e-30)
        return gamma * q * ops.inv_M_rel

    z = _two_loop(st, g_tan_ext, mem, initial)
    gnorm_smooth = float(np.max(np.abs(z)))
    num = vdot(z, g_tan_ext - st["g"])
    den = vdot(st["g"], st["z"]) + 1e-30
    beta = 0.0 if st["it"] % L == 0 else max(0.0, num / den)
    p = -z + beta * tangent_grad(m, st["p"])
    if vdot(p, g_tan_ext) > 0:
        p = -z
    H, tau, E_new, g_new, U_new, m_new, ev, dem = _ls(ops, st, B, prm, phi_tol, p, 1.0)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    s_new = tangent_grad(m_new, p * tau)
    y_new = tangent_grad(m_new, g_new) - tangent_grad(m_new, g_tan_ext)
    _history_update(st, m_new, s_new, y_new, mem)
    st.update(m=m_new, U=U_new, g=g_tan_ext, g_raw=g_new, z=z, p=p, E=E_new, gnorm=gnorm_smooth, it=st["it"] + 1,
              conv=conv, evals=st["evals"] + ev, demag=st["demag"] + dem, tau=tau)


def solve_Py_g_tr(ops: Ops, m, g_ext, g_tan_ext, delta, max_iter=20, tol=0.0, reg=0.0):
    """Steihaug-Toint truncated PCG inside the M_rel-norm ball of radius delta; returns (y, iterations)
    (``src/minimizers.py:506-592``)."""
    Mr = _m_rel(ops)

    def vdot_M(a, b):
        return vdot(a * Mr, b)

    y = np.zeros_like(g_tan_ext)
    r = g_tan_ext.copy()
    z = r * ops.inv_M_prec
    p = z.copy()
    rho = vdot(r, z)
    target = tol * tol * rho
    it, done = 0, False
    while it < max_iter and rho > target and rho > 1e-25 and rho < 1e20 and not done:
        Ap = apply_P(ops, m, g_ext, p, reg)
        pAp = vdot(p, Ap)
        alpha = rho / (pAp + 1e-30)
        a_q = vdot_M(p, p) + 1e-30
        b_q = 2.0 * vdot_M(y, p)
        c_q = vdot_M(y, y) - delta**2
        alpha_tr = (-b_q + math.sqrt(max(0.0, b_q**2 - 4.0 * a_q * c_q))) / (2.0 * a_q)
        y_a = y + alpha * p
        done = (pAp <= 0.0) or (vdot_M(y_a, y_a) >= delta**2)
        y = y + (alpha_tr if done else alpha) * p
        r = r - alpha * Ap
        z = r * ops.inv_M_prec
        rho_next = vdot(r, z)
        if not done:
            p = z + (rho_next / (rho + 1e-30)) * p
        rho = rho_next
        it += 1
    z_fb = g_tan_ext * ops.inv_M_prec
    yn, zn = float(np.linalg.norm(y)), float(np.linalg.norm(z_fb))
    if yn > 10.0 * zn:
        y = y * (10.0 * zn / (yn + 1e-30))
    ym = math.sqrt(vdot_M(y, y) + 1e-30)
    if ym > delta:
        y = y * (delta / ym)
    return y, it


def _tr_radius(delta, rho_tr, d):
    """Nocedal-Wright radius update (``src/minimizers.py:2050-2060``)."""
    if rho_tr < 0.25:
        return 0.25 * delta
    if rho_tr > 0.75 and float(np.linalg.norm(d)) >= 0.9 * delta:
        return min(2.0 * delta, 100.0)
    return delta


def _tr_finish(ops, st, B, prm, phi_tol, d, pred, gnorm_inf, pc_it, demag_inner):
    """Trial step R(m, m x d, 1), ratio test, radius update and acceptance (``src/minimizers.py:2036-2090``)."""
    m, U, g_raw, E = st["m"], st["U"], st["g_raw"], st["E"]
    m_t = cayley_update(m, np.cross(m, d), 1.0)
    U_t, itd, _ = ops.solve_U(m_t, U, phi_tol)
    E_t, g_t = ops.energy_and_grad(m_t, U_t, B)
    if not np.isfinite(E_t):
        E_t = 1e20
    rho_tr = (E - E_t) / (pred + 1e-30)
    delta = _tr_radius(st["delta"], rho_tr, d)
    if rho_tr > 0.01:
        m_n, U_n, E_n, g_n, U_p = m_t, U_t, E_t, g_t, U
    else:
        m_n, U_n, E_n, g_n, U_p = m, U, E, g_raw, st["U_prev"]
    conv = check_convergence(st["it"], E_n, E, m, m_n, gnorm_inf, prm.tau_f, prm.eps_a)
    st.update(m=m_n, U=U_n, U_prev=U_p, E=E_n, g_raw=g_n, delta=delta, gnorm=gnorm_inf, it=st["it"] + 1, conv=conv,
              evals=st["evals"] + 1, preco=st["preco"] + pc_it, demag=st["demag"] + demag_inner + int(itd))


def _tr_step(ops, st, B, prm, phi_tol):
    """Trust-region Newton-CG on the local Hessian (``src/minimizers.py:2005-2103``)."""
    m, g_raw = st["m"], st["g_raw"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    d, pc_it = solve_Py_g_tr(ops, m, g_raw, -g_tan_ext, st["delta"], prm.tn_iters, _pc_tol(prm, gnorm_inf), prm.pc_reg)
    Pd = apply_P(ops, m, g_raw, d, prm.pc_reg)
    pred = -(vdot(g_raw, d) + 0.5 * vdot(d, Pd))
    _tr_finish(ops, st, B, prm, phi_tol, d, pred, gnorm_inf, pc_it, 0)


def _ptr_step(ops, st, B, prm, phi_tol):
    """Preconditioned trust region on the full Hessian (demag included through a Poisson solve per
    product), the local-Hessian solve as preconditioner (``src/minimizers.py:2140-2320``).  The inner
    solves use the function's default stagnation threshold 1e-3, as the reference's calls do."""
    m, g_raw = st["m"], st["g_raw"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    pc_tol = _pc_tol(prm, gnorm_inf)
    Mr = _m_rel(ops)
    delta = st["delta"]
    zero_B = np.zeros(3)
    mg = np.sum(m * g_raw, axis=1, keepdims=True)

    def hess(v, U_guess):
        U_v, itd, _ = ops.solve_U(v, U_guess, phi_tol)
        Cv = ops.energy_and_grad(v, U_v, zero_B)[1]
        vg = np.sum(v * g_raw, axis=1, keepdims=True)
        mC = np.sum(m * Cv, axis=1, keepdims=True)
        return Cv - (vg * m + mg * v + mC * m), int(itd), U_v

    def vdot_M(a, b):
        return vdot(a * Mr, b)

    d = np.zeros_like(g_tan)
    r = g_tan_ext.copy()
    z, pc_acc = solve_Py_g(ops, m, g_raw, r, prm.pc_iters, pc_tol, prm.pc_reg)
    p = -z
    rho = vdot(r, z)
    q, U_guess, i, dem, done = 0.0, np.zeros(m.shape[0]), 0, 0, False
    while i < prm.tn_iters and not done and rho > 0.0:
        Hp, itd, U_p = hess(p, U_guess)
        kappa = vdot(p, Hp)
        alpha = rho / (kappa + 1e-30)
        a_q = vdot_M(p, p) + 1e-30
        b_q = 2.0 * vdot_M(d, p)
        c_q = vdot_M(d, d) - delta**2
        alpha_tr = (-b_q + math.sqrt(max(0.0, b_q**2 - 4.0 * a_q * c_q))) / (2.0 * a_q)
        d_a = d + alpha * p
        done_now = (kappa <= 0.0) or (vdot_M(d_a, d_a) >= delta**2)
        af = alpha_tr if done_now else alpha
        q = q + af * vdot(r, p) + 0.5 * af**2 * kappa
        d = d + af * p
        r = r + alpha * Hp
        z, pc_it = solve_Py_g(ops, m, g_raw, r, prm.pc_iters, pc_tol, prm.pc_reg)
        rho_next = vdot(r, z)
        beta = rho_next / (rho + 1e-30)
        p = -z + beta * p
        U_guess = beta * U_p
        done = done or done_now or rho_next < 1e-8 or rho <= 0.0
        rho = rho_next
        pc_acc += pc_it
        dem += itd
        i += 1
    _tr_finish(ops, st, B, prm, phi_tol, d, -q, gnorm_inf, pc_acc, dem)


def volume_averaged_J_parallel(m, conn, volume, mat_id, Js_lookup, h_dir) -> float:
    """``src/hysteresis_loop.py:153-190``."""
    h = h_dir / (np.linalg.norm(h_dir) + 1e-30)
    m_avg = m[conn].mean(axis=1)
    Js_e = Js_lookup[mat_id - 1]
    Vmag = np.sum(np.where(Js_e > 0, volume, 0.0)) + 1e-30
    J_avg = np.sum(volume[:, None] * Js_e[:, None] * m_avg, axis=0) / Vmag
    return float(J_avg @ h)


def run_sweep(ops: Ops, p, m0, h_dir, B_vals, prm: Params, method="pcohen_hs", Js_ref=1.0, mfinal=None):
    """Field sweep of ``src/hysteresis_loop.py:377-642`` without file output.

    Returns a list of rows (B_tesla, J_tesla, E, iters, evals, demag_iters) and the final (m, U).
    """
    m = m0 / np.linalg.norm(m0, axis=1, keepdims=True)
    U = np.zeros(m.shape[0])
    hist = []
    for Bmag in B_vals:
        B = Bmag * h_dir
        m, U, info = minimize(ops, m, B, U, prm, method)
        J = volume_averaged_J_parallel(m, p.conn, p.volume, p.mat_id, p.Js_lookup, h_dir)
        hist.append((Bmag * Js_ref, J * Js_ref, info["E"], info["iters"], info["evals"], info["demag_iters"]))
        if mfinal is not None and J <= mfinal:
            break
    return hist, m, U


def compute_coercivity(H, M):
    """Coercive field of an M-H branch, ``examples/evaluate_materials/analyze_evaluations.py:19-44``.

    The zero crossing is found by linear interpolation after sorting by M; the returned H_c is the
    larger of |crossing| and |smallest H with M >= 0|.
    """
    H = np.asarray(H, np.float64)
    M = np.asarray(M, np.float64)
    idx = np.argsort(M)
    cross = float(np.interp(0.0, M[idx], H[idx]))
    mask = M >= 0
    H_left = float(np.min(H[mask])) if np.any(mask) else cross
    return max(abs(cross), abs(H_left))
