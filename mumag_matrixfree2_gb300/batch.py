"""Many independent particles (uneven meshes, own materials) swept through the hysteresis loop at once.

Each particle is its own problem in libmumag_cuda (its own device buffers, hierarchy and CUDA
stream).  A pool of host threads drives the problems' field steps concurrently: the C-ABI calls
release the GIL, every call stays on its problem's stream, so the GPU overlaps the kernels of many
small instances whose single-instance kernels are launch- and latency-bound.  Per-instance results
(polarisation curve, coercive field, step latencies) are gathered on the host.
"""

from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from . import fem_utils
from . import synthetic as syn
from .cuda_backend import MinimizerParams
from .hysteresis_loop import NodalAverages, coercive_field


@dataclass
class ParticleResult:
    index: int
    nodes: int
    tets: int
    setup_s: float
    step_s: list = field(default_factory=list)
    J: list = field(default_factory=list)
    pcg_iters: int = 0
    min_iters: int = 0
    launches: int = 0  # kernels the sweep launched (graph nodes included)
    Hc_T: float = 0.0


def run_particle(index: int, p: syn.Particle, B_T, h_dir, precision: str = "fp64", params: MinimizerParams | None = None,
                 seed: int = 0, theta_e3: int = 0, max_coarse: int = 1000) -> ParticleResult:
    """Mesh, set up and sweep one particle (called from a worker thread); theta_e3 > 0 sets the
    hierarchy's strength threshold (MM_OPT_SA_THETA_E3)."""
    t0 = time.perf_counter()
    knt, ijk = syn.ellipsoid_mesh(p)
    A, K1, Js, k, Js_ref = syn.reduced_materials([p.material, syn.AIR])
    s = fem_utils.prepare(knt, ijk, A, K1, Js, k)
    prob = fem_utils.make_problem(s)
    if precision != "fp64":
        prob.set_precision(precision)
    if theta_e3 > 0:
        prob.set_option("sa_theta_e3", theta_e3)
    prob.build_poisson(1e-12, "amgcl", max_coarse=max_coarse)
    avg = NodalAverages(s.geom.conn, s.geom.volume, s.geom.mat_id, s.Js_lookup, s.N)
    prm = params or MinimizerParams(method="pcohen_hs", tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10, pc_iters=10)
    res = ParticleResult(index, s.N, int(ijk.shape[0]), time.perf_counter() - t0)
    h = np.asarray(h_dir, np.float64)
    m = syn.initial_state(s.N, seed=seed, direction=tuple(h))
    U = np.zeros(s.N)
    launches0 = prob.launch_count()
    for B in B_T:
        t1 = time.perf_counter()
        m, U, info = prob.minimize((float(B) / Js_ref) * h, m, U, prm)
        res.step_s.append(time.perf_counter() - t1)
        res.J.append(avg.J_parallel(m, h) * Js_ref)
        res.pcg_iters += info["demag_iters"]
        res.min_iters += info["iters"]
    res.launches = prob.launch_count() - launches0
    res.Hc_T = coercive_field(np.asarray(B_T), np.asarray(res.J))
    prob.close()
    return res


def run_batch(particles, B_T, h_dir=(0.0, 0.0, 1.0), workers: int = 16, precision: str = "fp64",
              params: MinimizerParams | None = None, theta_e3: int = 0, max_coarse: int = 1000) -> dict:
    """Sweep every particle through B_T [T] with `workers` concurrent host threads (one problem and
    CUDA stream each).  Returns per-particle results and the aggregate throughput."""
    import torch

    dev = torch.cuda.current_device()
    lock = threading.Lock()
    done: list[ParticleResult] = []

    def job(i):
        torch.cuda.set_device(dev)
        r = run_particle(i, particles[i], B_T, h_dir, precision, params, theta_e3=theta_e3, max_coarse=max_coarse)
        with lock:
            done.append(r)
        return r

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(job, range(len(particles))))
    wall = time.perf_counter() - t0
    done.sort(key=lambda r: r.index)
    steps = np.concatenate([np.asarray(r.step_s) for r in done])
    return {"particles": len(done), "workers": workers, "precision": precision, "field_steps": len(B_T),
            "wall_s": wall, "loops_per_s": len(done) / wall,
            "setup_s_total": float(sum(r.setup_s for r in done)),
            "sweep_s_total": float(sum(sum(r.step_s) for r in done)),
            "step_latency_ms": {"p50": float(1e3 * np.percentile(steps, 50)),
                                "p99": float(1e3 * np.percentile(steps, 99))},
            "nodes": {"min": int(min(r.nodes for r in done)), "median": int(np.median([r.nodes for r in done])),
                      "max": int(max(r.nodes for r in done)), "total": int(sum(r.nodes for r in done))},
            "pcg_iters_total": int(sum(r.pcg_iters for r in done)),
            "gpu_launches_total": int(sum(r.launches for r in done)),
            "results": done}
