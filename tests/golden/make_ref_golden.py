"""Generate the fixtures of tests/golden/ref_cpp_*.npz from the reference's own C++ minimizer.

The reference's CPU path, ``src/cpp/cpp_mkl_minimizer.cpp``, is compiled unchanged against the
MKL-API shim into ``oracle/_ref/libcpp_mkl_minimizer.so`` (``python -m oracle.build_ref``, which
needs the reference source).  This script runs that library on the synthetic workloads and stores
what the GPU tests compare with, since the library cannot run on the GPU host:

* ``ref_cpp_<workload>.npz`` for the 8 nm and 40 nm cubes: ``evaluate_energy_and_grad`` (E and g),
  ``solve_poisson`` (U), ``solve_Py_g`` after 1 and after 10 inner iterations, and three field steps
  of ``run_cpp_pcohen_hs_minimization`` from the seeded initial state (iterations, evaluations, inner
  iterations, energy and m); vectors at every ``stride``-th node plus whole-vector sums;
* ``ref_cpp_loop_<workload>.npz``: the field sweep +8 -> -8 T in 0.1 T steps (161 fields) of the
  reference's ``--cpp-mkl`` loop on the 40 nm cube and (with ``--cube80``) the 80 nm cube: J(B),
  energies, iteration counts, the coercive field and the switching step.

Usage: ``python tests/golden/make_ref_golden.py [--no-loop] [--cube80]`` (a few minutes on 8 cores;
the 80 nm loop takes about half an hour).
"""

import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from mumag_matrixfree2_gb300 import synthetic as syn  # noqa: E402
from oracle import build_ref, ref_cpp  # noqa: E402
from oracle import minimize as omin  # noqa: E402
from tests import helpers as H  # noqa: E402


def sums(v: np.ndarray) -> np.ndarray:
    v = np.asarray(v, np.float64).reshape(-1)
    return np.array([v.sum(), (v * v).sum(), np.abs(v).max()])


def case_fixture(lib, name: str, stride: int) -> None:
    s, p, Js_ref = H.case(name)
    cp = ref_cpp.CppProblem(lib, p)
    idx = H.ref_sample(p.N, stride)
    m, U_in, B = H.ref_state(name)
    E, g = cp.energy_and_grad(m, U_in, B)
    U = cp.solve_poisson(m)
    it_s, rr_s = lib.last_solve()
    gt = omin.tangent_grad(m, g)
    y1, it1 = cp.solve_Py_g(m, g, gt, 1, 0.0, 0.0, 1e-3)
    y10, it10 = cp.solve_Py_g(m, g, gt, 10, 0.0, 0.0, 1e-3)
    prm = H.ref_min_params()
    h = syn.tilted_field_direction(1.0)
    mm = syn.initial_state(p.N)
    UU = np.zeros(p.N)
    steps = []
    for BT in H.REF_FIELDS_T:
        mm, UU, info = cp.minimize(mm, (BT / Js_ref) * h, UU, prm)
        steps.append((info["iters"], info["evals"], info["preco_iters"], info["E"], mm[idx].copy()))
    out = HERE / f"ref_cpp_{name}.npz"
    np.savez_compressed(
        out, N=p.N, stride=stride, idx=idx, B=B, E=E, g=g[idx], g_sums=sums(g), U=U[idx], U_sums=sums(U),
        pardiso_relres=rr_s, pardiso_iters=it_s, y1=y1[idx], y1_sums=sums(y1), it1=it1, y10=y10[idx],
        y10_sums=sums(y10), it10=it10, fields_T=np.array(H.REF_FIELDS_T),
        min_iters=np.array([st[0] for st in steps]), min_evals=np.array([st[1] for st in steps]),
        min_preco=np.array([st[2] for st in steps]), min_E=np.array([st[3] for st in steps]),
        min_m=np.stack([st[4] for st in steps]), library=str(lib.kind))
    print("wrote", out.name, "E", E, "steps", [st[:4] for st in steps])


def loop_fixture(lib, name: str = "cube40_h2_air200") -> None:
    s, p, Js_ref = H.case(name)
    cp = ref_cpp.CppProblem(lib, p)
    prm = H.ref_min_params()
    h = syn.tilted_field_direction(1.0)
    B_vals = syn.field_values(8.0 / Js_ref, -8.0 / Js_ref, 0.1 / Js_ref)
    t = time.time()
    rows, _, _ = ref_cpp.run_sweep(cp, syn.initial_state(p.N), h, B_vals, prm, Js_ref=Js_ref)
    r = np.array(rows)
    B_T, J_T = r[:, 0], r[:, 1]
    Hc = omin.compute_coercivity(B_T, J_T)
    switch = int(np.argmax(J_T < 0)) if np.any(J_T < 0) else -1
    out = HERE / f"ref_cpp_loop_{name}.npz"
    np.savez_compressed(out, B_T=B_T, J_T=J_T, E=r[:, 2], iters=r[:, 3].astype(int), evals=r[:, 4].astype(int),
                        demag=r[:, 5].astype(int), preco=r[:, 6].astype(int), Hc_T=Hc, switch_index=switch,
                        library=str(lib.kind))
    print(f"wrote {out.name}: Hc {Hc:.6f} T, switch at step {switch} ({B_T[switch]:.2f} T), "
          f"{int(r[:, 3].sum())} iterations, {time.time() - t:.0f} s")


def main(argv) -> None:
    build_ref.build()
    lib = ref_cpp.load("reference")
    if lib is None:
        sys.exit("oracle/_ref/libcpp_mkl_minimizer.so is missing: the reference source is needed to build it")
    for name, stride in H.REF_CASES.items():
        case_fixture(lib, name, stride)
    if "--no-loop" not in argv:
        loop_fixture(lib)
    if "--cube80" in argv:
        loop_fixture(lib, "cube80_h1.6_air200")


if __name__ == "__main__":
    main(sys.argv[1:])
