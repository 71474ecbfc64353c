"""Field sweep with the reference's interface (``src/hysteresis_loop.py:34-657``) on the GPU backend.

Every field step is one ``minimize`` call that runs entirely in libmumag_cuda; the host computes the
volume-averaged polarisation and writes the reference's CSV, .mh and VTU snapshot files
(``io_utils``) with the reference's snapshot rule (``:585-640``).
"""

from __future__ import annotations

import time
from dataclasses import dataclass
from pathlib import Path
from typing import Any

import numpy as np

from . import io_utils
from .cuda_backend import problem_for_geom
from .minimizers import make_minimizer
from .poisson_solve import make_solve_U
from .synthetic import field_values


@dataclass
class LoopParams:
    """Same fields and defaults as the reference (``src/hysteresis_loop.py:34-125``)."""

    h_dir: np.ndarray
    B_start: float
    B_end: float
    dB: float
    loop: bool = True
    gamma: int = 5
    max_iter: int = 2000
    tau_f: float = 1e-8
    eps_a: float = 1e-12
    tau0: float = 1e-2
    tau_min: float = 1e-6
    tau_max: float = 1.0
    ls_eta1: float = 0.1
    ls_eta2: float = 0.1
    ls_C: float = 2.0
    ls_c: float = 0.5
    ls_s0: float = 1.0
    ls_max_evals: int = 15
    out_dir: str = "hyst_out"
    csv_name: str = "hysteresis.csv"
    snapshot_every: int = 1
    verbose: bool = False
    Js_ref: float = 1.0
    cg_maxiter: int = 2000
    cg_tol: float = 1e-8
    poisson_reg: float = 1e-12
    poisson_solver: str = "jax"
    mfinal: float | None = None
    mstep: float | None = None
    bias_type: str | None = None
    bias_strength: float = 0.0
    method: str = "pcohen_hs"
    pc_iters: int = 15
    pc_auto: bool = True
    pc_force_eta: float = 0.5
    pc_force_alpha: float = 0.5
    pc_stagnation_nu: float = 0.01
    memory: int = 5
    tn_iters: int = 5
    lr: float = 0.1
    mu: float = 0.9
    pc_reg: float = 0.0
    phi_extrapolate: bool = True
    wg_gamma: int = 5
    wg_threshold: float = 1e-6
    benchmark: bool = False
    L: int | None = None
    cpp_mkl: bool = False


def volume_averaged_J_parallel(m, conn, volume, mat_id, Js_lookup, h_dir) -> float:
    """``src/hysteresis_loop.py:153-190`` on the host (element form, used by the tests)."""
    h = np.asarray(h_dir, np.float64)
    h = h / (np.linalg.norm(h) + 1e-30)
    m_avg = m[conn].mean(axis=1)
    Js_e = np.asarray(Js_lookup)[mat_id - 1]
    Vmag = np.sum(np.where(Js_e > 0, volume, 0.0)) + 1e-30
    return float((np.sum(volume[:, None] * Js_e[:, None] * m_avg, axis=0) / Vmag) @ h)


def volume_averaged_m(m, conn, volume, mat_id, Js_lookup) -> np.ndarray:
    """``src/hysteresis_loop.py:193-223`` on the host (element form, used by the tests)."""
    m_avg = m[conn].mean(axis=1)
    Js_e = np.asarray(Js_lookup)[mat_id - 1]
    Vmag = np.sum(np.where(Js_e > 0, volume, 0.0)) + 1e-30
    return np.sum(np.where(Js_e[:, None] > 0, volume[:, None] * m_avg, 0.0), axis=0) / Vmag


def coercive_field(B, J) -> float:
    """H_c of one descending branch as ``examples/evaluate_materials/analyze_evaluations.py:19-44``
    evaluates it: the field where J crosses zero (linear interpolation in J-sorted order), or, if
    larger in magnitude, the lowest field at which J is still non-negative."""
    B = np.asarray(B, np.float64)
    J = np.asarray(J, np.float64)
    order = np.argsort(J)
    zero_cross = float(np.interp(0.0, J[order], B[order]))
    nonneg = J >= 0
    lowest = float(B[nonneg].min()) if nonneg.any() else zero_cross
    return max(abs(zero_cross), abs(lowest))


class NodalAverages:
    """The two volume averages of ``src/hysteresis_loop.py:153-223`` as nodal dot products.

    Both averages are linear in m: sum_e V_e c_e mean_{a in e}(m_a) = sum_a m_a sum_{e ni a} V_e c_e / 4,
    so the per-node weights are formed once per mesh and every field step costs one (N,3) product
    instead of a gather over all elements.  Equal to the element form up to summation order.
    """

    def __init__(self, conn, volume, mat_id, Js_lookup, n_nodes: int):
        conn = np.asarray(conn)
        volume = np.asarray(volume, np.float64)
        Js_e = np.asarray(Js_lookup, np.float64)[np.asarray(mat_id) - 1]
        Vmag = np.sum(np.where(Js_e > 0, volume, 0.0)) + 1e-30
        quarter = lambda c: np.repeat(0.25 * c, 4)  # noqa: E731
        self.wJ = np.bincount(conn.reshape(-1), weights=quarter(volume * Js_e), minlength=n_nodes) / Vmag
        self.wm = np.bincount(conn.reshape(-1), weights=quarter(np.where(Js_e > 0, volume, 0.0)),
                              minlength=n_nodes) / Vmag

    def J_parallel(self, m, h) -> float:
        return float((self.wJ @ m) @ h)

    def m_avg(self, m) -> np.ndarray:
        return self.wm @ m


def _torch_cuda():
    """torch when a CUDA device is present (the loop then keeps its state on the GPU), else None."""
    try:
        import torch
    except ImportError:
        return None
    return torch if torch.cuda.is_available() else None


def _host(a) -> np.ndarray:
    return a.cpu().numpy() if hasattr(a, "cpu") else np.asarray(a)


def run_hysteresis_loop(points, geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, m0, params: LoopParams, V_mag,
                        node_volumes, M_nodal, B_bias=None, precond_type: str = "amgcl", order: int = 3,
                        energy_assembly: str = "segment_sum", grad_backend: str = "stored_grad_phi",
                        chunk_elems: int = 200_000, boundary_mask=None, *, mode: str = "assembled",
                        precision: str = "fp64", write_files: bool = True, device_loop: bool = True,
                        **_unused) -> dict[str, Any]:
    """Sweep the applied field and minimise at every value (``src/hysteresis_loop.py:226-657``).

    Returns {"out_dir", "csv_path", "last_m", "last_U", "history", "steps"} where history rows are
    (B_ext [T], J_par [T], mx, my, mz, E [J/m^3]) as in the reference and steps holds per-step
    (iters, evals, preco_iters, demag_iters, seconds).  ``device_loop`` (an addition) runs the CG
    minimizers' iterations as one device graph per field step (MM_OPT_MIN_GRAPH); False keeps the
    host-driven loop.
    """
    out_dir = Path(params.out_dir)
    csv_path = out_dir / params.csv_name
    if write_files:
        out_dir.mkdir(parents=True, exist_ok=True)
        io_utils.write_hysteresis_header(csv_path)
    h = np.array([float(x) for x in params.h_dir.split(",")]) if isinstance(params.h_dir, str) else \
        np.asarray(params.h_dir, np.float64)
    h = h / (np.linalg.norm(h) + 1e-30)
    # one device problem for the solver and the minimizer: the energy operator and the hierarchy are
    # built once (make_minimizer finds this problem in the geometry's cache)
    prob = problem_for_geom(geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, V_mag, M_nodal, boundary_mask)
    prob.set_option("min_graph", int(bool(device_loop)))
    solve_U = make_solve_U(geom, Js_lookup, precond_type=precond_type, cg_maxiter=params.cg_maxiter,
                           cg_tol=params.cg_tol, poisson_reg=params.poisson_reg, boundary_mask=boundary_mask,
                           mode=mode, precision=precision, problem=prob)
    minimize = make_minimizer(geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, V_mag, node_volumes, M_nodal,
                              solve_U, params.cg_tol, method=params.method, memory=params.memory,
                              boundary_mask=boundary_mask, B_bias=B_bias)
    m = np.asarray(m0, np.float64)
    avg = NodalAverages(geom.conn, geom.volume, geom.mat_id, Js_lookup, m.shape[0])
    m = m / np.linalg.norm(m, axis=1, keepdims=True)
    U = np.zeros(m.shape[0])
    # m and U stay on the GPU between field steps (no host round trip of the state per step); the
    # two averages are taken there and only their values come back
    torch = _torch_cuda()
    if torch is not None:
        m = torch.from_numpy(np.ascontiguousarray(m)).cuda()
        U = torch.zeros(m.shape[0], dtype=torch.float64, device="cuda")
        wJ_d = torch.from_numpy(avg.wJ).cuda()
        wm_d = torch.from_numpy(avg.wm).cuda()
        h_d = torch.from_numpy(h).cuda()
    B_vals = field_values(params.B_start, params.B_end, params.dB, params.loop)
    history, steps = [], []
    config_idx, J_last = 0, None
    total = dict(time=0.0, iters=0, preco=0, evals=0, demag=0, demag_time=0.0, demag_wall_time=0.0,
                 device_loop_steps=0)
    for step_idx, Bmag in enumerate(B_vals):
        t0 = time.perf_counter()
        m, U, info = minimize(m, Bmag * h, U0=U, max_iter=params.max_iter, tau_f=params.tau_f, eps_a=params.eps_a,
                              tau0=params.tau0, ls_eta1=params.ls_eta1, ls_eta2=params.ls_eta2, ls_C=params.ls_C,
                              ls_c=params.ls_c, pc_iters=params.pc_iters, pc_auto=params.pc_auto,
                              pc_force_eta=params.pc_force_eta, pc_force_alpha=params.pc_force_alpha,
                              pc_stagnation_nu=params.pc_stagnation_nu, memory=params.memory, pc_reg=params.pc_reg,
                              wg_gamma=params.wg_gamma, L=params.L, tn_iters=params.tn_iters, lr=params.lr,
                              mu=params.mu, phi_extrapolate=params.phi_extrapolate, cpp_mkl=params.cpp_mkl,
                              verbose=params.verbose, inplace=True)
        dt = time.perf_counter() - t0
        if torch is not None:
            J = float((wJ_d @ m) @ h_d)
            mx, my, mz = (wm_d @ m).cpu().numpy()
        else:
            J = avg.J_parallel(m, h)
            mx, my, mz = avg.m_avg(m)
        B_t, J_t = float(Bmag) * params.Js_ref, J * params.Js_ref
        E_si = info["E"] * params.Js_ref**2 / (2.0 * 4e-7 * np.pi)
        history.append([B_t, J_t, mx, my, mz, E_si])
        steps.append((info["iters"], info["evals"], info["preco_iters"], info["demag_iters"], dt))
        total["time"] += dt
        total["iters"] += info["iters"]
        total["preco"] += info["preco_iters"]
        total["evals"] += info["evals"]
        total["demag"] += info["demag_iters"]
        total["demag_time"] += info.get("demag_time", 0.0)
        total["demag_wall_time"] += info.get("demag_wall_time", 0.0)
        total["device_loop_steps"] += int(bool(info.get("device_loop", False)))
        # a state is saved on the first step, then when J moved by mstep or, without mstep, every
        # snapshot_every steps; each save after the first starts a new configuration index
        if J_last is None:
            save = True
        elif params.mstep is not None:
            save = abs(J - J_last) >= params.mstep
        else:
            save = params.snapshot_every > 0 and step_idx % params.snapshot_every == 0
        if save:
            if J_last is not None:
                config_idx += 1
            J_last = J
            if write_files and params.snapshot_every > 0:
                io_utils.write_vtu_tetra(out_dir / io_utils.snapshot_name(config_idx, B_t), points,
                                         np.asarray(geom.conn), point_data={"m": _host(m).astype(np.float32),
                                                                            "U": _host(U).astype(np.float32)},
                                         cell_data={"mat_id": np.asarray(geom.mat_id).astype(np.int32)})
        if write_files:
            io_utils.append_hysteresis_row(csv_path, config_idx, B_t, J_t, float(info["E"]), float(info["gnorm"]))
        print(f"step {step_idx:05d}  B={B_t:+.6e} T  J_par={J_t:+.6e} T  E={info['E']:.6e}  t={dt:.3f}s  "
              f"it={info['iters']}  t/it={dt / max(1, info['iters']):.3e}s  nf={info['evals']}  "
              f"icg_amg={info['demag_iters']}")
        if params.mfinal is not None and J <= params.mfinal:
            print(f"\n[loop] mfinal reached ({J_t:.4f} T <= {params.mfinal * params.Js_ref:.4f} T). Stopping sweep.")
            break
    print(f"\nHysteresis loop finished in {total['time']:.3f} s.\nTotal minimizer iterations: {total['iters']}\n"
          f"Total preconditioner iterations: {total['preco']}\nTotal function evaluations: {total['evals']}\n"
          f"Total Poisson (demag) iterations: {total['demag']}")
    hist = np.array(history)
    if write_files:
        io_utils.write_mh(out_dir / "hysteresis", hist)
    return {"out_dir": str(out_dir), "csv_path": str(csv_path), "last_m": _host(m), "last_U": _host(U), "history": hist,
            "steps": steps, "totals": total}
