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


def solve_Py_g(ops: Ops, m, g_ext, g_tan_ext, max_iter=20, tol=0.0, reg=0.0, stagnation_nu=1e-3):
    """Inner PCG with Steihaug exit; returns (y, iterations), ``src/minimizers.py:413-490``."""
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

    @property
    def phi_tol(self) -> float:
        """``src/minimizers.py:3447-3452``."""
        return float(min(self.cg_tol, self.tau_f * 0.1))


def minimize(ops: Ops, m0, B, U0, prm: Params, method="pcohen_hs"):
    """``make_minimizer(...).minimize``: init (``src/minimizers.py:3408-3435``) then the step loop.

    Returns (m, U, info) with info keys iters, E, gnorm, preco_iters, evals, demag_iters.
    """
    m = m0 / np.linalg.norm(m0, axis=1, keepdims=True)
    U, init_demag, _ = ops.solve_U(m, U0, prm.cg_tol)
    E, g_raw = ops.energy_and_grad(m, U, B)
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm = float(np.max(np.abs(g_tan)))
    N = m.shape[0]
    L = prm.L or N
    st = dict(m=m, U=U, g=g_tan_ext, g_raw=g_raw, y=g_tan_ext, d=-g_tan_ext, E=E, gnorm=gnorm, it=0,
              conv=False, evals=1, preco=0, demag=int(init_demag))
    if method in ("lbfgs", "plbfgs"):
        mem = prm.memory
        st.update(g=g_tan, S=np.zeros((mem, N, 3)), Y=np.zeros((mem, N, 3)), rho=np.zeros(mem), hist_it=0)
    if method == "wg_np":
        st.update(g=g_tan, m_prev=m, g_tan_prev=g_tan)
    phi_tol = prm.phi_tol
    while not st["conv"] and st["it"] < prm.max_iter:
        if method == "pcohen_hs":
            _pcohen_hs_step(ops, st, B, prm, phi_tol, L)
        elif method == "lbfgs":
            _lbfgs_step(ops, st, B, prm, phi_tol)
        elif method == "wg_np":
            _wg_np_step(ops, st, B, prm, phi_tol)
        elif method == "plbfgs":
            _plbfgs_step(ops, st, B, prm, phi_tol)
        else:
            raise NotImplementedError(method)
    info = dict(iters=st["it"], E=float(st["E"]), gnorm=float(st["gnorm"]), preco_iters=st["preco"],
                evals=st["evals"], demag_iters=st["demag"])
    return st["m"], st["U"], info


def _pcohen_hs_step(ops, st, B, prm, phi_tol, L):
    """Preconditioned Cohen CG with Hestenes-Stiefel beta, ``src/minimizers.py:962-1071``."""
    m, U, g_prev, g_raw, d_prev, E_prev = st["m"], st["U"], st["g"], st["g_raw"], st["d"], st["E"]
    g_tan = tangent_grad(m, g_raw * ops.inv_M_rel)
    g_tan_ext = tangent_grad(m, g_raw)
    gnorm_inf = float(np.max(np.abs(g_tan)))
    pc_tol = min(prm.pc_force_eta, gnorm_inf ** prm.pc_force_alpha) if prm.pc_auto else 0.0
    y, preco_it = solve_Py_g(ops, m, g_raw, g_tan_ext, prm.pc_iters, pc_tol, prm.pc_reg, prm.pc_stagnation_nu)
    gnorm_smooth = float(np.max(np.abs(y)))
    diff_g = g_tan_ext - g_prev
    num = vdot(y, diff_g)
    den = vdot(d_prev, diff_g) + 1e-30
    beta = 0.0 if st["it"] % L == 0 else max(0.0, num / den)
    d = -y + beta * tangent_grad(m, d_prev)
    if vdot(d, g_tan_ext) > 0:
        d = -y
    H = np.cross(m, d)  # -cross(m, -d)
    pg = vdot(g_raw, d)
    tau, E_new, g_new, U_new, m_new, ev, dem = armijo_ls(
        ops, m, pg, H, E_prev, U, g_raw, B, phi_tol, prm.ls_eta1, prm.ls_eta2, prm.ls_C, prm.ls_c, 1.0, 15)
    conv = check_convergence(st["it"], E_new, E_prev, m, m_new, gnorm_smooth, prm.tau_f, prm.eps_a)
    st.update(m=m_new, U=U_new, g=g_tan_ext, g_raw=g_new, y=y, d=d, E=E_new, gnorm=gnorm_smooth,
              it=st["it"] + 1, conv=conv, evals=st["evals"] + ev, preco=st["preco"] + preco_it,
              demag=st["demag"] + dem, tau=tau)


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
