"""``make_minimizer`` with the reference's signature (``src/minimizers.py:2927-2963``), on the GPU.

Every method of the reference's command line runs on the GPU (``mm_minimize``): the preconditioned CG
family "pcohen_hs" (the hysteresis loop's default, ``:950-1073``), "pcohen", "pcg" (``:828-947``),
"cohen" (``:642-720``), "pcohen_exact" / "pcohen_hs_exact" (Cayley transport, ``:1081-1200``); the
quasi-Newton family "lbfgs" (``:1266-1381``), "plbfgs" (``:1526-1653``), "dplbfgs" (``:1808-1968``),
"pcohen_lbfgs" (``:2806-2924``); "wg_np" (Barzilai-Borwein, ``:1706-1800``); the Newton family
"tn_split" (``:1437-1517``), "tr" and "ptr" (trust regions, ``:1994-2320``); "aapg" / "aapg_exact"
(Anderson acceleration, ``:2395-2636``) and "pnag" (Nesterov, ``:2715-2803``).
"""

from __future__ import annotations

import numpy as np

from .cuda_backend import MinimizerParams, problem_for_geom

SUPPORTED = ("pcohen_hs", "lbfgs", "wg_np", "plbfgs", "cohen", "pcg", "pcohen", "pcohen_exact", "pcohen_hs_exact",
             "dplbfgs", "tn_split", "tr", "ptr", "aapg", "aapg_exact", "pnag", "pcohen_lbfgs")


def tangent_grad(m, g):
    """Project a raw gradient onto the tangent space (``src/minimizers.py:94-96``)."""
    return g - np.sum(m * g, axis=1, keepdims=True) * m


def cayley_update(m, H, tau):
    """Cayley rotation with renormalisation (``src/minimizers.py:71-79``), host helper."""
    k = 0.5 * tau * H
    k2 = np.sum(k * k, axis=1, keepdims=True)
    m_new = ((1.0 - k2) * m + 2.0 * np.cross(k, m) + 2.0 * np.sum(k * m, axis=1, keepdims=True) * k) / (1.0 + k2)
    return m_new / np.linalg.norm(m_new, axis=1, keepdims=True)


def make_minimizer(geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, V_mag, node_volumes, M_nodal, solve_U,
                   cg_tol, method: str = "pcg", **kwargs):
    """Return minimize(m0, B_ext, **params) -> (m, U, info) running each field step on the GPU."""
    if method not in SUPPORTED:
        raise NotImplementedError(f"method {method!r} is not part of the cuda backend (available: {SUPPORTED})")
    sp = getattr(solve_U, "problem", None)
    boundary_mask = kwargs.get("boundary_mask")
    if boundary_mask is None and sp is not None and sp.has_mask:
        boundary_mask = sp.mask_host
    # the magnetoelastic constants reach the energy operator as make_energy_kernels' keywords do
    prob = problem_for_geom(geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, V_mag, M_nodal, boundary_mask,
                            k1me=kwargs.get("k1me"), k1me_p=kwargs.get("k1me_p"))
    if not prob.poisson_built:
        if sp is not None:
            if sp.precision != "fp64":
                prob.set_precision(sp.precision)
            prob.build_poisson(sp.reg, sp.precond_type, sp.max_levels, sp.max_coarse)
        else:
            prob.build_poisson(1e-12, "amgcl")
    memory = int(kwargs.get("memory", 5))
    B_bias = kwargs.get("B_bias")

    def minimize(m0, B_ext, **params):
        sparse_ops = params.get("sparse_ops") or {}
        if sparse_ops.get("inv_M_rel") is not None or sparse_ops.get("inv_M_prec") is not None:
            prob.set_node_weights(sparse_ops.get("inv_M_rel"), sparse_ops.get("inv_M_prec"))
        bias = sparse_ops.get("B_bias", B_bias)
        prob.set_bias_field(None if bias is None else np.broadcast_to(np.asarray(bias, np.float64), (prob.N, 3)))
        tau_f = float(params.get("tau_f", 1e-6))
        prm = MinimizerParams(
            method=method, max_iter=int(params.get("max_iter", 2000)), tau_f=tau_f,
            eps_a=float(params.get("eps_a", 1e-12)), tau0=float(params.get("tau0", 1e-2)),
            ls_eta1=float(params.get("ls_eta1", 0.1)), ls_eta2=float(params.get("ls_eta2", 0.1)),
            ls_C=float(params.get("ls_C", 2.0)), ls_c=float(params.get("ls_c", 0.5)), ls_max_evals=15,
            pc_iters=int(params.get("pc_iters", 10)), pc_auto=bool(params.get("pc_auto", False)),
            pc_force_eta=float(params.get("pc_force_eta", 0.5)),
            pc_force_alpha=float(params.get("pc_force_alpha", 0.5)),
            pc_stagnation_nu=float(params.get("pc_stagnation_nu", 1e-3)), pc_reg=float(params.get("pc_reg", 0.0)),
            memory=int(params.get("memory", memory)), wg_gamma=int(params.get("wg_gamma", 2)),
            L=params.get("L"), cg_tol=float(cg_tol),
            phi_tol=float(params["phi_tol"]) if "phi_tol" in params else float(min(cg_tol, 0.1 * tau_f)),
            cg_maxiter=int(params.get("cg_maxiter", 2000)), tn_iters=int(params.get("tn_iters", 5)),
            lr=float(params.get("lr", 0.1)), mu=float(params.get("mu", 0.9)),
            phi_extrapolate=bool(params.get("phi_extrapolate", False)),
            cpp_semantics=bool(params.get("cpp_mkl", False)))
        U0 = params.get("U0")
        if U0 is None:  # a device-resident m (torch CUDA tensor) gets a device U
            U0 = m0.new_zeros(prob.N) if hasattr(m0, "new_zeros") else np.zeros(prob.N)
        if not params.get("inplace", False):
            # the reference's minimize returns new arrays and leaves m0 and U0 untouched; a field
            # sweep that carries its state on the GPU passes inplace=True to skip the two copies
            m0 = m0.clone() if hasattr(m0, "clone") else m0
            U0 = U0.clone() if hasattr(U0, "clone") else U0
        m, U, info = prob.minimize(B_ext, m0, U0, prm)
        if params.get("verbose", True):
            print(f"          number of iterations   : {info['iters']}")
            print(f"number of iterations for preco   : {info['preco_iters']}")
            print(f"number of function evaluations   : {info['evals']}")
            print(f"number of iterations for demag   : {info['demag_iters']}")
            print("done")
        return m, U, info

    minimize.problem = prob
    return minimize


def time_field_steps(workload: str = "cube80_h1.6_air200", method: str = "pcohen_hs", first: int = 120,
                     steps: int = 15, precision: str = "fp64") -> dict:
    """Minimize the field steps first .. first+steps-1 of the +8 T -> -8 T sweep (0.1 T, tilted 1 deg)
    of a synthetic cube workload, after three warm-up steps from the first fields; the timed steps
    run inside the NVTX range "steps" so that a profiler can select exactly their launches.  Returns
    the host time and the minimizer's counters, with the demag solves' share."""
    import time

    import torch

    from . import fem_utils
    from . import synthetic as syn

    knt, ijk = syn.box_mesh(syn.WORKLOADS[workload])
    A, K1, Js, k, Js_ref = syn.reduced_materials([syn.Material(), syn.AIR])
    s = fem_utils.prepare(knt, ijk, A, K1, Js, k)
    prob = fem_utils.make_problem(s)
    prob.set_precision(precision)
    prob.build_poisson(1e-12, "amgcl")
    prob.autotune(20)
    h = syn.tilted_field_direction(1.0)
    m, U = syn.initial_state(s.N, seed=0), np.zeros(s.N)
    prm = MinimizerParams(method=method, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10, pc_iters=10)
    Bs = syn.field_values(8.0 / Js_ref, -8.0 / Js_ref, 0.1 / Js_ref)
    for B in Bs[:3]:
        m, U, _ = prob.minimize(B * h, m, U, prm)
    tot = dict(seconds=0.0, demag_device_s=0.0, demag_host_s=0.0, iters=0, evals=0, preco_iters=0, demag_iters=0)
    torch.cuda.nvtx.range_push("steps")
    for B in Bs[first:first + steps]:
        t = time.perf_counter()
        m, U, info = prob.minimize(B * h, m, U, prm)
        tot["seconds"] += time.perf_counter() - t
        tot["demag_device_s"] += info["demag_time"]
        tot["demag_host_s"] += info["demag_wall_time"]
        for key in ("iters", "evals", "preco_iters", "demag_iters"):
            tot[key] += info[key]
    torch.cuda.nvtx.range_pop()
    return tot


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="time field steps of the GPU minimizer on a synthetic cube")
    ap.add_argument("--workload", default="cube80_h1.6_air200")
    ap.add_argument("--method", default="pcohen_hs", choices=SUPPORTED)
    ap.add_argument("--first", type=int, default=120)
    ap.add_argument("--steps", type=int, default=15)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "fp32_precond"])
    a = ap.parse_args()
    print(json.dumps(time_field_steps(a.workload, a.method, a.first, a.steps, a.precision)))
