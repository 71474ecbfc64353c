#!/usr/bin/env python
"""Benchmark of the demag Poisson solve (the reference's headline unit of work).

One step = one demag PCG solve (SA-AMG V-cycle with SPAI0 smoothing, FP64) from U = 0 to relative
residual 1e-10 for the seeded initial magnetisation, on the 80 nm cube at 1.6 nm spacing inside a
graded 200 nm air box (357,911 nodes, 2,058,000 tetrahedra).

  python bench.py [--gpus N --steps K --warmup W]          this project's CUDA path
  python bench.py --impl reference [...]                   the reference algorithm on the host CPU
                                                           (the oracle port: the reference's own
                                                           code needs JAX/PyAMG or Intel MKL)

With torchrun (N > 1) every rank solves its own replica (one solve does not shard) and rank 0
prints one JSON line with the aggregate throughput.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "demag PCG solves/s & loop wall time: mixed+learned vs plain FP64, same tol"
PUBLISHED_SOLVES_PER_S = 1000.0 / 200.3  # reference, RTX 4060 Laptop, 2.3M-tet mesh, 1e-10 from x0 = 0
L2_FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="cube80_h1.6_air200")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as td

        td.init_process_group("nccl")
    return rank, local, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as td

        td.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as td

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def workload_inputs(name):
    from mumag_matrixfree2_gb300 import synthetic as syn

    w = syn.WORKLOADS[name]
    knt, ijk = syn.box_mesh(w)
    A, K1, Js, k, Js_ref = syn.reduced_materials([syn.Material(), syn.AIR])
    m0 = syn.initial_state(knt.shape[0], seed=0)
    return knt, ijk, (A, K1, Js, k), m0


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the timed kernel from the committed ncu summary, if there is one."""
    f = ROOT / "profiles" / "smooth_level0_cube80.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait(timeout=10)
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) > 8 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) > 8 for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_solves(knt, ijk, mats, m0, tol, n_solves):
    """The oracle (numpy/scipy FP64 port of the reference's PCG + V-cycle) timed on the host."""
    from oracle import fem as ofem
    from oracle import poisson as opo

    A, K1, Js, k = mats
    p = ofem.make_problem(knt, ijk, A, K1, Js, k)
    su = opo.SolveU(p, ofem.assembled_operators(p, parts=("A", "D")), cg_tol=tol)
    zero = np.zeros(p.N)
    su(m0, zero, tol)  # warm the caches once
    t0 = time.perf_counter()
    its = []
    for _ in range(n_solves):
        _, it, _ = su(m0, zero, tol, return_info=True)
        its.append(it)
    dt = time.perf_counter() - t0
    return n_solves / dt, its


def run_reference(a):
    rank, local, ws = dist()
    if rank != 0:
        return
    knt, ijk, mats, m0 = workload_inputs(a.workload)
    from oracle import fem as ofem
    from oracle import poisson as opo

    A, K1, Js, k = mats
    p = ofem.make_problem(knt, ijk, A, K1, Js, k)
    su = opo.SolveU(p, ofem.assembled_operators(p, parts=("A", "D")), cg_tol=a.tol)
    zero = np.zeros(p.N)
    for _ in range(a.warmup):
        su(m0, zero, a.tol)
    t0 = time.perf_counter()
    its = []
    for _ in range(a.steps):
        _, it, _ = su(m0, zero, a.tol, return_info=True)
        its.append(it)
    dt = time.perf_counter() - t0
    v = a.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1000.0 * dt / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "nodes": int(p.N), "tets": int(len(ijk)), "tol": a.tol,
                   "precond": "SA-AMG V(1,1) SPAI0", "pcg_iters_per_solve": its[0]},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": 1, "kind": "port",
                         "sample": f"{a.steps} cold-start solves (scipy CSR SpMV, one thread)"},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def run_ours(a):
    import torch

    rank, local, ws = dist()
    torch.cuda.set_device(local)
    from mumag_matrixfree2_gb300 import build as _b

    _b.build()
    from mumag_matrixfree2_gb300 import fem_utils

    knt, ijk, mats, m0 = workload_inputs(a.workload)
    t0 = time.perf_counter()
    s = fem_utils.prepare(knt, ijk, *mats)
    prob = fem_utils.make_problem(s)
    n_levels = prob.build_poisson(1e-12, "amgcl")
    setup_s = time.perf_counter() - t0
    N = s.N
    m_dev = torch.from_numpy(m0).cuda()
    U_dev = torch.zeros(N, dtype=torch.float64, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def one():
        U_dev.zero_()
        torch.cuda.synchronize()
        _, it, rr, rc = prob.solve_u(m_dev, U_dev, a.tol)
        if rc != 0 or not rr <= a.tol:
            raise RuntimeError(f"solve did not converge: status {rc}, rel_res {rr}")
        return it, rr

    for _ in range(a.warmup):
        one()
    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = prob.launch_count()
    dev_ms, its, rrs = 0.0, [], []
    for k in range(a.steps):
        flush.fill_(k & 0xFF)  # L2 flush between timed solves (outside the solve's events)
        it, rr = one()
        dev_ms += prob.last_solve_ms()
        its.append(it)
        rrs.append(rr)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    launches = prob.launch_count() - launches0
    t_dev = max_over_ranks(dev_ms / 1000.0, ws)
    value = ws * a.steps / t_dev

    # end to end through the public API with host buffers: H2D of m and U0, D2H of U every step
    m_host = np.ascontiguousarray(m0)
    zero = np.zeros(N)
    barrier(ws)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(a.steps):
        U, it, rr, rc = prob.solve_u(m_host, zero, a.tol)
    e2e_s = max_over_ranks(time.perf_counter() - t1, ws)
    e2e = ws * a.steps / e2e_s

    # roofline of the dominant kernel (level-0 SPAI0 smoothing sweep), timed alone with events
    ms_k, bytes_k = prob.time_kernel("smooth", 20)
    peak, peak_kind = peaks()
    achieved = bytes_k / (ms_k * 1e-3) / 1e9
    lv = prob.amg_levels()

    cpu = None
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        v_cpu, its_cpu = cpu_solves(knt, ijk, mats, m0, a.tol, 2)
        cpu = {"value": v_cpu, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"2 cold-start solves of the same workload by the numpy/scipy FP64 oracle "
                         f"({its_cpu[0]} PCG iterations each)"}
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1000.0 * t_dev / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": value / PUBLISHED_SOLVES_PER_S, "dtype": "f64", "data": "synthetic",
            "config": {"workload": a.workload, "nodes": N, "tets": int(len(ijk)), "tol": a.tol,
                       "precond": "SA-AMG V(1,1) SPAI0", "amg_levels": n_levels,
                       "level_sizes": [int(x["A"].shape[0]) for x in lv],
                       "pcg_iters_per_solve": its[0], "rel_res": max(rrs), "setup_s": setup_s,
                       "l2": "256 MiB buffer written between timed solves (outside the solve events)",
                       "parallelism": f"replicas x{ws}",
                       "vs_baseline_note": "published 200.3 ms/solve: RTX 4060 Laptop, 361,812 nodes / 2,304,342 tets"},
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(N * 3 * 8 + N * 8),
                    "d2h_bytes_per_step": int(N * 8)},
            "roofline": {"bound": "hbm", "kernel": "k_smooth_dot (level-0 SPAI0 sweep)", "achieved": achieved,
                         "peak": peak, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": profiled_traffic(), "bytes_per_launch": bytes_k, "ms_per_launch": ms_k},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
