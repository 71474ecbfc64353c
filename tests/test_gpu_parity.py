"""GPU kernels (through the C-ABI) against the FP64 oracle.  Tolerances are stated per check:
FP64 operators to 1e-10 relative (the reference's parity bar for energies and gradients), the
potential to the PCG tolerance, integer work bit-exact."""

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import fem_utils
from mumag_matrixfree2_gb300.cuda_backend import MinimizerParams
from oracle import fem as ofem
from oracle import minimize as omin
from oracle import poisson as opo

from .helpers import case, random_state

pytestmark = pytest.mark.gpu

RTOL = 1e-10  # FP64 parity bar for energies, gradients and operator products


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def small(cuda_ok):
    s, p, Js_ref = case("cube16_h2_air48")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    ops = ofem.assembled_operators(p)
    return s, p, ops, prob


def test_energy_and_gradient(small):
    s, p, ops, prob = small
    m = random_state(p.N, seed=1)
    U = np.random.default_rng(2).standard_normal(p.N)
    B = np.array([0.1, -0.05, -0.3])
    E, g = prob.energy_and_grad(m, U, B)
    E0, g0 = ofem.energy_and_grad_asm(p, ops, m, U, B)
    assert abs(E - E0) <= RTOL * abs(E0)
    assert rel(g, g0) <= RTOL
    bias = 0.01 * np.random.default_rng(3).standard_normal((p.N, 3))
    E, g = prob.energy_and_grad(m, U, B, bias)
    E0, g0 = ofem.energy_and_grad_asm(p, ops, m, U, B, bias)
    assert abs(E - E0) <= RTOL * abs(E0) and rel(g, g0) <= RTOL


def test_energy_multi_axis(cuda_ok):
    s, p, _ = case("cube8_h2_air24", tilt_axis=True)
    prob = fem_utils.make_problem(s)
    ops = ofem.assembled_operators(p)
    m = random_state(p.N, seed=4)
    U = np.random.default_rng(5).standard_normal(p.N)
    E, g = prob.energy_and_grad(m, U, [0.0, 0.0, 0.2])
    E0, g0 = ofem.energy_and_grad_mf(p, m, U, [0.0, 0.0, 0.2])
    assert abs(E - E0) <= RTOL * abs(E0) and rel(g, g0) <= RTOL


def test_float_float_energy_matches_fp64(cuda_ok):
    """The float-float energy operator of the mixed-precision problems (MM_OPT_ENERGY_FF) against the
    FP64 one and the oracle: energy to 1e-12 relative, gradient to 1e-11 of its largest entry; a
    problem with several easy axes keeps the FP64 evaluation (bit-identical)."""
    s, p, _ = case("cube16_h2_air48")
    m = random_state(p.N, seed=31)
    U = np.random.default_rng(32).standard_normal(p.N)
    B = np.array([0.1, -0.05, -0.3])
    probs = {}
    for ff in (0, 1):
        prob = fem_utils.make_problem(s)
        prob.set_option("energy_ff", ff)
        probs[ff] = prob
    E64, g64 = probs[0].energy_and_grad(m, U, B)
    E0, g0 = ofem.energy_and_grad_mf(p, m, U, B)
    for lanes in (1, 2, 8, 4):  # every lane count of the kernel (the shuffle merge of the row sums)
        probs[1].set_option("energy_ff_lanes", lanes)
        Eff, gff = probs[1].energy_and_grad(m, U, B)
        assert abs(Eff - E64) <= 1e-12 * abs(E64), lanes
        assert rel(gff, g64) <= 1e-11, lanes
        assert abs(Eff - E0) <= RTOL * abs(E0) and rel(gff, g0) <= RTOL
    ms, nbytes = probs[1].time_kernel("energy", 5)
    assert ms > 0 and nbytes > 0
    from mumag_matrixfree2_gb300 import synthetic as syn

    knt, ijk = syn.box_mesh(syn.WORKLOADS["cube8_h2_air24"])
    ijk = ijk.copy()
    right = knt[ijk[:, :4]].mean(axis=1)[:, 0] > 0
    ijk[(ijk[:, 4] == 1) & right, 4] = 3  # half of the magnet gets a tilted easy axis
    A, K1, Js, k, _ = syn.reduced_materials([syn.Material(), syn.AIR,
                                             syn.Material(axis=(np.sin(0.3), 0.0, np.cos(0.3)))])
    s2 = fem_utils.prepare(knt, ijk, A, K1, Js, k)
    a, b = fem_utils.make_problem(s2), fem_utils.make_problem(s2)
    b.set_option("energy_ff", 1)
    m2 = random_state(s2.N, seed=33)
    U2 = np.random.default_rng(34).standard_normal(s2.N)
    Ea, ga = a.energy_and_grad(m2, U2, B)
    Eb, gb = b.energy_and_grad(m2, U2, B)
    assert Ea == Eb and np.array_equal(ga, gb)


def test_local_hessian_rhs_and_diagonal(small):
    s, p, ops, prob = small
    v = np.random.default_rng(6).standard_normal((p.N, 3))
    assert rel(prob.local_grad(v), ofem.local_grad_only_asm(p, ops, v)) <= RTOL
    m = random_state(p.N, seed=7)
    b, bb = prob.rhs(m)
    b0 = ofem.rhs_from_m_asm(ops, m)
    assert rel(b, b0) <= RTOL and abs(bb - b0 @ b0) <= RTOL * (b0 @ b0)
    assert rel(prob.exchange_diagonal(), ofem.exchange_diagonal(p)) <= RTOL


def test_poisson_operator_and_vcycle(small):
    s, p, ops, prob = small
    U = np.random.default_rng(8).standard_normal(p.N)
    assert rel(prob.apply_A(U), ops["A"] @ U) <= RTOL
    H = opo.build_hierarchy(ops["A"])
    r = np.random.default_rng(9).standard_normal(p.N)
    z0 = opo.vcycle_spai0(H, lambda v: ops["A"] @ v, r)
    assert rel(prob.precond(r), z0) <= 1e-9


@pytest.mark.parametrize("precond", ["amgcl", "amg", "jacobi", "none"])
def test_solve_matches_oracle(cuda_ok, precond):
    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, precond)
    su = opo.SolveU(p, precond_type=precond, cg_tol=1e-10)
    m = random_state(p.N, seed=10)
    U0, it0, rr0 = su(m, np.zeros(p.N), 1e-10, return_info=True)
    U, it, rr, rc = prob.solve_u(m, np.zeros(p.N), 1e-10)
    assert rc == 0 and rr <= 1e-10
    assert abs(it - it0) <= 1, (it, it0)
    assert rel(U, U0) <= 1e-8
    # warm start from the converged potential of a nearby state
    m2 = random_state(p.N, seed=11, amplitude=0.31)
    U0b, it0b, _ = su(m2, U0, 1e-10, return_info=True)
    Ub, itb, rrb, _ = prob.solve_u(m2, U, 1e-10)
    assert abs(itb - it0b) <= 1 and rrb <= 1e-10 and rel(Ub, U0b) <= 1e-8


def test_solve_cfg_mesh_and_determinism(cuda_ok):
    s, p, _ = case("cube40_h2_air200")
    prob = fem_utils.make_problem(s)
    nl = prob.build_poisson(1e-12, "amgcl")
    assert nl == 4
    su = opo.SolveU(p, ofem.assembled_operators(p, parts=("A", "D")), cg_tol=1e-10)
    m = random_state(p.N, seed=12, amplitude=0.05)
    U0, it0, rr0 = su(m, np.zeros(p.N), 1e-10, return_info=True)
    U1, it1, rr1, _ = prob.solve_u(m, np.zeros(p.N), 1e-10)
    U2, it2, rr2, _ = prob.solve_u(m, np.zeros(p.N), 1e-10)
    assert abs(it1 - it0) <= 1 and rr1 <= 1e-10
    assert rel(U1, U0) <= 1e-8
    assert it1 == it2 and np.array_equal(U1, U2)  # fixed grids and fixed reduction trees


def test_solve_into_out_leaves_x0_untouched(cuda_ok):
    """solve_u(m, x0, tol, out=U): x0 is read on the device as it is (not modified), U lands in `out`,
    identical to the in-place host solve and to the device solve."""
    import torch

    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    m = random_state(p.N, seed=23, amplitude=0.2)
    x0 = 0.01 * np.random.default_rng(24).standard_normal(p.N)
    x0_copy = x0.copy()
    out = torch.empty(p.N, dtype=torch.float64, pin_memory=True).numpy()
    U1, it1, rr1, rc1 = prob.solve_u(m, x0, 1e-10, out=out)
    assert U1 is out and np.array_equal(x0, x0_copy)
    U2, it2, rr2, rc2 = prob.solve_u(m, x0, 1e-10)
    assert rc1 == rc2 == 0 and it1 == it2 and np.array_equal(U1, U2)
    Ud = torch.from_numpy(x0.copy()).cuda()
    _, it3, _, _ = prob.solve_u(torch.from_numpy(m).cuda(), Ud, 1e-10)
    assert it3 == it1 and np.array_equal(Ud.cpu().numpy(), U1)


def test_solve_without_mask_projects_the_mean(cuda_ok):
    s, p, _ = case("cube8_h2_air24", with_boundary=False)
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    su = opo.SolveU(p, cg_tol=1e-9)
    m = random_state(p.N, seed=13)
    U0, it0, _ = su(m, np.zeros(p.N), 1e-9, return_info=True)
    U, it, rr, _ = prob.solve_u(m, np.zeros(p.N), 1e-9)
    assert abs(it - it0) <= 1 and abs(U.mean()) < 1e-12 * np.abs(U).max()
    assert rel(U, U0) <= 1e-6


def test_maxiter_is_reported(cuda_ok):
    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    U, it, rr, rc = prob.solve_u(random_state(p.N, seed=14), np.zeros(p.N), 1e-14, maxiter=2)
    assert it == 2 and rc == 1 and rr > 1e-14


def _oracle_ops(p, ops, su, bias=None):
    d = ofem.exchange_diagonal(p)
    return omin.Ops(
        energy_and_grad=lambda m, U, B: ofem.energy_and_grad_asm(p, ops, m, U, B, bias),
        local_grad_only=lambda v: ofem.local_grad_only_asm(p, ops, v),
        solve_U=lambda m, x0, tol: su(m, x0, tol, return_info=True),
        inv_M_rel=np.where(p.M_nodal > 1e-20, p.V_mag / np.where(p.M_nodal > 0, p.M_nodal, 1), 0.0)[:, None],
        inv_M_prec=np.where(d > 1e-20, 1.0 / np.where(d > 0, d, 1), 1.0)[:, None],
    )


@pytest.mark.parametrize("method", omin.METHODS)
def test_minimizer_matches_oracle(cuda_ok, method):
    """Every minimizer of the reference's command line: same iterations, energy evaluations and
    inner (preconditioner) iterations as the oracle, same energy and state."""
    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    ops = ofem.assembled_operators(p)
    su = opo.SolveU(p, ops, cg_tol=1e-10)
    O = _oracle_ops(p, ops, su)
    m0 = random_state(p.N, seed=15, amplitude=0.2)
    B = np.array([0.0, 0.0, -0.3])
    prm = omin.Params(max_iter=12, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
    m_ref, U_ref, info_ref = omin.minimize(O, m0, B, np.zeros(p.N), prm, method)
    mp = MinimizerParams(method=method, max_iter=12, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
    m, U, info = prob.minimize(B, m0, np.zeros(p.N), mp)
    assert info["iters"] == info_ref["iters"]
    assert info["evals"] == info_ref["evals"]
    assert info["preco_iters"] == info_ref["preco_iters"]
    if method == "plbfgs":
        assert info["preco_iters"] == info["iters"]
    assert abs(info["E"] - info_ref["E"]) <= 1e-9 * abs(info_ref["E"])
    assert np.max(np.abs(m - m_ref)) <= 1e-7


def test_device_resident_minimize_equals_host_minimize(cuda_ok):
    """minimize with m and U as CUDA tensors (mm_minimize_dev, updated in place) runs the same
    iteration as with host arrays: bit-identical state and counts."""
    import torch

    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    m0 = random_state(p.N, seed=25, amplitude=0.2)
    B = np.array([0.0, 0.0, -0.3])
    mp = MinimizerParams(method="pcohen_hs", max_iter=15, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
    m1, U1, i1 = prob.minimize(B, m0, np.zeros(p.N), mp)
    md = torch.from_numpy(m0.copy()).cuda()
    Ud = torch.zeros(p.N, dtype=torch.float64, device="cuda")
    m2, U2, i2 = prob.minimize(B, md, Ud, mp)
    assert m2 is md and U2 is Ud
    assert (i1["iters"], i1["evals"], i1["preco_iters"], i1["demag_iters"]) == \
        (i2["iters"], i2["evals"], i2["preco_iters"], i2["demag_iters"])
    assert np.array_equal(m2.cpu().numpy(), m1) and np.array_equal(U2.cpu().numpy(), U1)


@pytest.mark.parametrize("pc_iters", [0, 1, 3])
def test_inner_iteration_cap_matches_oracle(cuda_ok, pc_iters):
    """The device-driven inner solve at small iteration caps (0: the loop body never updates, the
    fallback direction is taken): same counts, energy and state as the oracle."""
    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    ops = ofem.assembled_operators(p)
    su = opo.SolveU(p, ops, cg_tol=1e-10)
    O = _oracle_ops(p, ops, su)
    m0 = random_state(p.N, seed=19, amplitude=0.2)
    B = np.array([0.0, 0.0, -0.3])
    prm = omin.Params(max_iter=10, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10, pc_iters=pc_iters)
    m_ref, _, info_ref = omin.minimize(O, m0, B, np.zeros(p.N), prm, "pcohen_hs")
    mp = MinimizerParams(method="pcohen_hs", max_iter=10, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10, pc_iters=pc_iters)
    m, _, info = prob.minimize(B, m0, np.zeros(p.N), mp)
    assert (info["iters"], info["evals"], info["preco_iters"]) == (info_ref["iters"], info_ref["evals"],
                                                                  info_ref["preco_iters"])
    assert info["preco_iters"] <= pc_iters * info["iters"]
    assert abs(info["E"] - info_ref["E"]) <= 1e-9 * abs(info_ref["E"])
    assert np.max(np.abs(m - m_ref)) <= 1e-7


@pytest.mark.parametrize("method", ["pcohen_hs", "ptr"])
def test_minimizer_with_bias_field_matches_oracle(cuda_ok, method):
    """A per-node bias field (sparse_ops["B_bias"]) enters every energy evaluation of the step,
    including the full-Hessian products of the preconditioned trust region."""
    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    ops = ofem.assembled_operators(p)
    su = opo.SolveU(p, ops, cg_tol=1e-10)
    bias = 0.05 * np.random.default_rng(4).standard_normal((p.N, 3))
    O = _oracle_ops(p, ops, su, bias)
    m0 = random_state(p.N, seed=16, amplitude=0.2)
    B = np.array([0.0, 0.0, -0.3])
    prm = omin.Params(max_iter=8, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
    m_ref, _, info_ref = omin.minimize(O, m0, B, np.zeros(p.N), prm, method)
    prob.set_bias_field(bias)
    m, _, info = prob.minimize(B, m0, np.zeros(p.N), MinimizerParams(method=method, max_iter=8, tau_f=1e-8, eps_a=1e-6,
                                                                     cg_tol=1e-10))
    prob.set_bias_field(None)
    assert (info["iters"], info["evals"], info["preco_iters"]) == (info_ref["iters"], info_ref["evals"],
                                                                  info_ref["preco_iters"])
    assert abs(info["E"] - info_ref["E"]) <= 1e-9 * abs(info_ref["E"])
    assert np.max(np.abs(m - m_ref)) <= 1e-7


@pytest.mark.parametrize("method", ["pcohen_hs", "plbfgs", "pcohen_lbfgs", "tn_split", "pcohen_exact"])
def test_fp32_inner_solve_reaches_the_fp64_minimum(cuda_ok, method):
    """The minimizer's inner preconditioner solve in FP32 (entries, vectors, float-float inner
    products) against the FP64 one on the same problem: both stop converged on the same minimum,
    energy to 1e-9 relative, state to 1e-4, with a comparable number of outer iterations."""
    s, p, _ = case("cube16_h2_air48")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    m0 = random_state(p.N, seed=17, amplitude=0.3)
    B = np.array([0.0, 0.01, -0.4])
    out = {}
    for inner in ("fp64", "fp32"):
        prob.set_inner_precision(inner)
        mp = MinimizerParams(method=method, max_iter=400, tau_f=1e-12, eps_a=1e-8, cg_tol=1e-10)
        out[inner] = prob.minimize(B, m0, np.zeros(p.N), mp)
    prob.set_inner_precision("auto")
    (m64, _, i64), (m32, _, i32) = out["fp64"], out["fp32"]
    assert i64["status"] == 0 and i32["status"] == 0, (i64, i32)
    assert i32["preco_iters"] == 0 or i32["preco_iters"] >= 0.5 * i64["preco_iters"]
    assert abs(i32["E"] - i64["E"]) <= 1e-9 * abs(i64["E"])
    assert np.max(np.abs(m32 - m64)) <= 1e-4
    assert i32["iters"] <= 1.25 * i64["iters"] + 3, (i32["iters"], i64["iters"])


@pytest.mark.parametrize("inner", ["fp64", "fp32"])
def test_inner_solve_graph_equals_host_polled_loop(cuda_ok, inner):
    """The inner solve's WHILE graph and the host-polled loop run the same kernels with the same
    device-side decisions: bit-identical minimizer results."""
    s, p, _ = case("cube8_h2_air24")
    m0 = random_state(p.N, seed=18, amplitude=0.2)
    B = np.array([0.0, 0.0, -0.3])
    out = []
    for graph in (1, 0):
        prob = fem_utils.make_problem(s)
        prob.set_option("graph", graph)
        prob.build_poisson(1e-12, "amgcl")
        prob.set_inner_precision(inner)
        mp = MinimizerParams(method="pcohen_hs", max_iter=15, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
        out.append(prob.minimize(B, m0, np.zeros(p.N), mp))
    (m1, U1, i1), (m0_, U0, i0) = out
    assert i1["preco_iters"] == i0["preco_iters"] > 0 and i1["iters"] == i0["iters"]
    assert np.array_equal(m1, m0_) and np.array_equal(U1, U0)


@pytest.mark.parametrize("method,precision,cpp", [("pcohen_hs", "fp64", False), ("pcohen", "fp64", False),
                                                  ("pcg", "fp64", False), ("pcohen_hs", "fp32_precond", False),
                                                  ("pcohen_hs", "fp64", True), ("pcohen", "fp32_precond", True)])
def test_device_minimizer_graph_equals_host_loop(cuda_ok, method, precision, cpp):
    """MM_OPT_MIN_GRAPH: the CG minimizers' iterations as one graph (the minimizer loop with the inner
    solve, the Armijo trials and their demag PCG as nested WHILE nodes) take the host-driven loop's
    iterations, evaluations, inner and demag iterations and reach its state bit for bit, on a first
    call and on a second field that replays the cached graph; the info says which loop ran."""
    s, p, _ = case("cube16_h2_air48")
    m0 = random_state(p.N, seed=19, amplitude=0.2)
    runs = {}
    for g in (1, 0):
        prob = fem_utils.make_problem(s)
        if precision != "fp64":
            prob.set_precision(precision)
        prob.build_poisson(1e-12, "amgcl")
        prob.set_option("min_graph", g)
        mp = MinimizerParams(method=method, max_iter=40, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10, cpp_semantics=cpp)
        m1, U1, i1 = prob.minimize(np.array([0.0, 0.0, -0.3]), m0, np.zeros(p.N), mp)
        m2, U2, i2 = prob.minimize(np.array([0.02, 0.0, -0.6]), m1, U1, mp)
        runs[g] = ((m1, U1, i1), (m2, U2, i2))
    for (mg, Ug, ig), (mh, Uh, ih) in zip(runs[1], runs[0]):
        assert ig["device_loop"] and not ih["device_loop"]
        for k in ("iters", "evals", "preco_iters", "demag_iters", "status"):
            assert ig[k] == ih[k], (k, ig[k], ih[k])
        assert ig["evals"] > ig["iters"] > 2
        assert ig["E"] == ih["E"] and ig["gnorm"] == ih["gnorm"]
        assert np.array_equal(mg, mh) and np.array_equal(Ug, Uh)


@pytest.mark.parametrize("precond", ["jacobi", "none"])
def test_device_minimizer_graph_with_single_level_preconditioners(cuda_ok, precond):
    """The minimizer graph with the Jacobi or no preconditioner in its demag solves (one-level
    preconditioners; a copy node that a conditional body cannot hold makes the capture fall back to
    the host loop): the same counts and state as the host-driven loop either way."""
    s, p, _ = case("cube8_h2_air24")
    m0 = random_state(p.N, seed=21, amplitude=0.2)
    out = {}
    for g in (1, 0):
        prob = fem_utils.make_problem(s)
        prob.build_poisson(1e-12, precond)
        prob.set_option("min_graph", g)
        mp = MinimizerParams(method="pcohen_hs", max_iter=25, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
        out[g] = prob.minimize(np.array([0.0, 0.0, -0.3]), m0, np.zeros(p.N), mp)
    (mg, Ug, ig), (mh, Uh, ih) = out[1], out[0]
    assert not ih["device_loop"]
    for k in ("iters", "evals", "preco_iters", "demag_iters"):
        assert ig[k] == ih[k], (k, ig[k], ih[k])
    assert np.array_equal(mg, mh) and np.array_equal(Ug, Uh)


@pytest.mark.parametrize("name", ["cube8_h2_air24", "cube40_h2_air200"])
def test_mixed_precision_meets_the_fp64_tolerance(cuda_ok, name):
    """FP32 correction solves inside FP64 iterative refinement: the true FP64 residual meets the
    same tolerance and the potential matches the plain FP64 solve to that tolerance."""
    s, p, _ = case(name)
    plain = fem_utils.make_problem(s)
    plain.build_poisson(1e-12, "amgcl")
    mixed = fem_utils.make_problem(s)
    mixed.set_precision("mixed")
    mixed.build_poisson(1e-12, "amgcl")
    ops = opo.SolveU(p, ofem.assembled_operators(p, parts=("A", "D")), cg_tol=1e-10)
    m = random_state(p.N, seed=31, amplitude=0.05)
    U64, it64, rr64, _ = plain.solve_u(m, np.zeros(p.N), 1e-10)
    U32, it32, rr32, rc = mixed.solve_u(m, np.zeros(p.N), 1e-10)
    assert rc == 0 and rr32 <= 1e-10 and mixed.last_refinements() >= 1
    b = ops.rhs(m)
    true_rr = np.linalg.norm(b - ops.apply_A(U32)) / np.linalg.norm(b)
    assert true_rr <= 1.5e-10  # checked in FP64 on the host
    assert rel(U32, U64) <= 1e-8


@pytest.mark.parametrize("name", ["cube8_h2_air24", "cube40_h2_air200"])
def test_fp32_preconditioner_keeps_the_fp64_pcg(cuda_ok, name):
    """The FP64 PCG with the V-cycle applied in FP32: the stopping test is the plain method's (recursive
    FP64 residual), the true FP64 residual meets the tolerance, the iterations stay within one of the
    FP64 preconditioner's and the potential matches the plain solve to the tolerance; the split
    finest-level product agrees with the FP64 one."""
    s, p, _ = case(name)
    plain = fem_utils.make_problem(s)
    plain.build_poisson(1e-12, "amgcl")
    pc = fem_utils.make_problem(s)
    pc.set_precision("fp32_precond")
    pc.build_poisson(1e-12, "amgcl")
    ops = opo.SolveU(p, ofem.assembled_operators(p, parts=("A", "D")), cg_tol=1e-10)
    for seed, x0 in ((31, None), (32, "warm")):
        m = random_state(p.N, seed=seed, amplitude=0.05)
        U0 = np.zeros(p.N) if x0 is None else plain.solve_u(random_state(p.N, seed=seed + 10, amplitude=0.05),
                                                            np.zeros(p.N), 1e-10)[0]
        U64, it64, rr64, _ = plain.solve_u(m, U0.copy(), 1e-10)
        Upc, itpc, rrpc, rc = pc.solve_u(m, U0.copy(), 1e-10)
        assert rc == 0 and rrpc <= 1e-10 and abs(itpc - it64) <= 1, (itpc, it64)
        b = ops.rhs(m)
        true_rr = np.linalg.norm(b - ops.apply_A(Upc)) / np.linalg.norm(b)
        assert true_rr <= 1.5e-10
        assert rel(Upc, U64) <= 1e-8
    pc.set_option("graph", 0)  # the host-polled loop: same iterations
    m = random_state(p.N, seed=31, amplitude=0.05)
    _, it_h, rr_h, rc_h = pc.solve_u(m, np.zeros(p.N), 1e-10)
    _, it_g, _, _ = plain.solve_u(m, np.zeros(p.N), 1e-10)
    assert rc_h == 0 and rr_h <= 1e-10 and abs(it_h - it_g) <= 1
    # the finest-level product in FP64 instead of the FP32-split operator: same iterations, the
    # potentials agree to the split's rounding (~2^-47 relative per product)
    U_split, it_split, _, _ = pc.solve_u(m, np.zeros(p.N), 1e-10)
    pc.set_option("split_a0", 0)
    U_f64, it_f64, rr_f64, rc_f64 = pc.solve_u(m, np.zeros(p.N), 1e-10)
    pc.set_option("split_a0", 1)
    assert rc_f64 == 0 and rr_f64 <= 1e-10 and it_f64 == it_split
    assert rel(U_split, U_f64) <= 1e-11


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fused_coarse_correction_matches_the_level_by_level_vcycle(cuda_ok, precision):
    """The two coarsest levels applied as x2 = T b + W (Z b) against the five level-by-level kernels:
    the same V-cycle (to rounding) and the same solve."""
    from mumag_matrixfree2_gb300 import synthetic as syn

    part = syn.random_particles(8, seed=0)[3]  # 110,032 nodes, a 4-level hierarchy (58 coarsest rows)
    knt, ijk = syn.ellipsoid_mesh(part)
    A, K1, Js, k, _ = syn.reduced_materials([part.material, syn.AIR])
    s = fem_utils.prepare(knt, ijk, A, K1, Js, k)
    probs = []
    for fuse in (0, 3):
        prob = fem_utils.make_problem(s)
        prob.set_precision(precision)
        prob.build_poisson(1e-12, "amgcl")
        prob.set_option("coarse_fuse", fuse)
        probs.append(prob)
    assert probs[1].n_levels == 4
    r = np.random.default_rng(41).standard_normal(s.N)
    z0, z1 = probs[0].precond(r), probs[1].precond(r)
    assert rel(z1, z0) <= (1e-11 if precision == "fp64" else 1e-5)
    m = random_state(s.N, seed=42, amplitude=0.05)
    U0, it0, rr0, rc0 = probs[0].solve_u(m, np.zeros(s.N), 1e-10)
    U1, it1, rr1, rc1 = probs[1].solve_u(m, np.zeros(s.N), 1e-10)
    assert rc1 == 0 and rr1 <= 1e-10 and abs(it1 - it0) <= 1
    assert rel(U1, U0) <= 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp32_precond"])
def test_fused_restriction_matches_the_residual_pass(cuda_ok, precision):
    """Restriction with R_l (I - A_l S_l) formed on the host against the residual kernel followed by
    R_l: the same V-cycle (to rounding) and the same solve, with the oracle's iteration count."""
    s, p, _ = case("cube40_h2_air200")
    probs = []
    for fr in (0, 3):
        prob = fem_utils.make_problem(s)
        prob.set_precision(precision)
        prob.build_poisson(1e-12, "amgcl")
        prob.set_option("fuse_restrict", fr)
        probs.append(prob)
    assert probs[0].n_levels >= 3
    r = np.random.default_rng(43).standard_normal(s.N) * s.boundary_mask
    z0, z1 = probs[0].precond(r), probs[1].precond(r)
    assert rel(z1, z0) <= (1e-11 if precision == "fp64" else 1e-5)
    m = random_state(s.N, seed=44, amplitude=0.05)
    U0, it0, rr0, rc0 = probs[0].solve_u(m, np.zeros(s.N), 1e-10)
    U1, it1, rr1, rc1 = probs[1].solve_u(m, np.zeros(s.N), 1e-10)
    assert rc1 == 0 and rr1 <= 1e-10 and abs(it1 - it0) <= 1
    assert rel(U1, U0) <= 1e-8
    if precision == "fp64":
        _, it_o, _ = opo.SolveU(p, cg_tol=1e-10)(m, np.zeros(p.N), 1e-10, return_info=True)
        assert abs(it1 - it_o) <= 1


@pytest.mark.parametrize("precision", ["fp64", "fp32_precond", "mixed"])
def test_coarse_cycle_in_one_launch_equals_five_launches(cuda_ok, precision):
    """MM_OPT_COARSE_CYCLE: the V-cycle's levels 1 .. 3 of the 80 nm cube's four-level hierarchy in one
    cooperative launch with grid barriers give the five-launch V-cycle's results bit for bit (same
    rows, same lanes per row, same order): the same preconditioned vector, the same solve inside the
    PCG loop graph, and the profiled (host-polled) solve runs the one-launch kernel once per V-cycle."""
    s, p, _ = case("cube80_h1.6_air200")
    probs = []
    for cc in (0, 3):
        prob = fem_utils.make_problem(s)
        if precision != "fp64":
            prob.set_precision(precision)
        assert prob.build_poisson(1e-12, "amgcl") == 4
        prob.set_option("coarse_fuse", 3)  # the one-launch cycle covers the fused coarse correction
        prob.set_option("coarse_cycle", cc)
        probs.append(prob)
    if precision == "fp64":
        r = np.random.default_rng(45).standard_normal(s.N) * s.boundary_mask
        assert np.array_equal(probs[0].precond(r), probs[1].precond(r))
    m = random_state(s.N, seed=46, amplitude=0.05)
    U0, it0, rr0, rc0 = probs[0].solve_u(m, np.zeros(s.N), 1e-10)
    U1, it1, rr1, rc1 = probs[1].solve_u(m, np.zeros(s.N), 1e-10)
    assert probs[1].get_option("coarse_cycle") == 3  # the loop graph held the cooperative launch
    assert rc0 == rc1 == 0 and it0 == it1 and rr0 == rr1 and np.array_equal(U0, U1)
    probs[1].set_option("profile", 1)
    probs[1].profile(reset=True)
    U2, it2, _, _ = probs[1].solve_u(m, np.zeros(s.N), 1e-10)
    rows = {(r["kernel"], r["precision"]): r["launches"] for r in probs[1].profile(reset=True)}
    cycles = [n for (k, _), n in rows.items() if k == "coarse_cycle"]
    assert cycles and min(cycles) > 0 and not any(k == "coarse_a" for k, _ in rows)
    assert np.array_equal(U2, U1)


@pytest.mark.parametrize("precision", ["fp64", "fp32_precond"])
def test_every_compressed_row_shape_gives_the_same_solve(cuda_ok, precision):
    """MM_OPT_CSR_LANES: every compressed-row operator read with 2 .. 32 lanes per row (the shapes the
    autotuner chooses among): the same preconditioned vector to rounding and the same solve
    (iterations +-1, potential to 1e-10 of its scale) on the 80 nm cube's four levels."""
    s, p, _ = case("cube80_h1.6_air200")
    m = random_state(s.N, seed=47, amplitude=0.05)
    r = np.random.default_rng(48).standard_normal(s.N) * s.boundary_mask
    ref = None
    for lanes in (8, 2, 4, 16, 32):
        prob = fem_utils.make_problem(s)
        if precision != "fp64":
            prob.set_precision(precision)
        prob.build_poisson(1e-12, "amgcl")
        prob.set_option("csr_lanes", lanes)
        z = prob.precond(r)
        U, it, rr, rc = prob.solve_u(m, np.zeros(s.N), 1e-10)
        assert rc == 0 and rr <= 1e-10
        if ref is None:
            ref = (z, U, it)
            continue
        assert rel(z, ref[0]) <= 1e-12, lanes
        assert abs(it - ref[2]) <= 1 and rel(U, ref[1]) <= 1e-10, lanes


def test_autotuner_keeps_results_within_tolerance(cuda_ok):
    """The autotuner changes launch shapes and the coarse path only: the solve converges to the same
    potential with the same iterations (+-1), and the report covers every compressed-row operator."""
    s, p, _ = case("cube40_h2_air200")
    prob = fem_utils.make_problem(s)
    prob.set_precision("mixed")
    prob.build_poisson(1e-12, "amgcl")
    m = random_state(p.N, seed=51, amplitude=0.05)
    U0, it0, rr0, _ = prob.solve_u(m, np.zeros(p.N), 1e-10)
    rep = prob.autotune(reps=5)
    assert rep["operators"] and all(o["tpr"] in (2, 4, 8, 16, 32) for o in rep["operators"])
    assert {o["precision"] for o in rep["operators"]} == {"fp64", "fp32"}
    U1, it1, rr1, rc1 = prob.solve_u(m, np.zeros(p.N), 1e-10)
    assert rc1 == 0 and rr1 <= 1e-10 and abs(it1 - it0) <= 1 and rel(U1, U0) <= 1e-8


def test_magnetoelastic_term_matches_oracle(cuda_ok):
    """Per-element k1me / k1me_p (shorter than E: zero-padded, as the reference pads them) in the
    energy, gradient and local Hessian, against the matrix-free oracle at the FP64 bar."""
    from mumag_matrixfree2_gb300.energy_kernels import make_energy_kernels

    s, p, _ = case("cube8_h2_air24")
    rng = np.random.default_rng(61)
    mag = np.flatnonzero(s.Js_lookup[s.geom.mat_id - 1] > 0)
    n = int(mag.max()) + 1
    k1me = np.zeros(n)
    k1me[mag] = 0.3 * rng.standard_normal(mag.size)
    k1me_p = np.zeros(n - 5)
    k1me_p[mag[mag < n - 5]] = 0.2 * rng.standard_normal(int((mag < n - 5).sum()))
    eg, _, _, lg = make_energy_kernels(s.geom, s.A_lookup, s.K1_lookup, s.Js_lookup, s.k_easy, s.V_mag, s.M_nodal,
                                       k1me=k1me, k1me_p=k1me_p, boundary_mask=s.boundary_mask)
    m = random_state(p.N, seed=62)
    U = rng.standard_normal(p.N)
    B = np.array([0.05, 0.0, -0.2])
    E, g = eg(m, U, B)
    E0, g0 = ofem.energy_and_grad_mf(p, m, U, B, k1me=k1me, k1me_p=k1me_p)
    assert abs(E - E0) <= RTOL * abs(E0) and rel(g, g0) <= RTOL
    v = rng.standard_normal((p.N, 3))
    assert rel(lg(v), ofem.local_grad_only_mf(p, v, k1me=k1me, k1me_p=k1me_p)) <= RTOL
    # the term changes the result (the test is not vacuous)
    E1, _ = ofem.energy_and_grad_mf(p, m, U, B)
    assert abs(E1 - E0) > 1e-6 * abs(E0)


def test_solves_on_reused_device_memory(cuda_ok):
    """Problems created after others were destroyed get device memory that held old data (an FP32 view
    of FP64 values can be NaN).  Every precision and loop form still converges to the plain solve:
    buffers are zeroed when allocated and the first PCG direction ignores the previous one."""
    s, p, _ = case("cube40_h2_air200")
    m = random_state(p.N, seed=31, amplitude=0.05)
    ref = None
    for prec in ("fp64", "fp32_precond", "mixed"):
        for graph in (1, 0):
            pr = fem_utils.make_problem(s)
            if prec != "fp64":
                pr.set_precision(prec)
            pr.set_option("graph", graph)
            pr.build_poisson(1e-12, "amgcl")
            U, it, rr, rc = pr.solve_u(m, np.zeros(p.N), 1e-10)
            assert rc == 0 and rr <= 1e-10 and it < 40, (prec, graph, it, rr, rc)
            if ref is None:
                ref = U
            assert rel(U, ref) <= 1e-8
            del pr


def test_level1_filter_keeps_the_solve(cuda_ok):
    """The level-1 operator without its weak couplings (the default) against the plain Galerkin one
    (MM_OPT_SA_FILTER_E6 < 0): fewer entries with the row sums kept, each hierarchy equal to the
    oracle's built the same way, and both solves at the tolerance with the oracle's iterations."""
    s, p, _ = case("cube40_h2_air200")
    ops = ofem.assembled_operators(p, parts=("A", "D"))
    m = random_state(s.N, seed=44, amplitude=0.05)
    res = {}
    for opt in (0, -1):
        prob = fem_utils.make_problem(s)
        prob.set_option("sa_filter_e6", opt)
        prob.build_poisson(1e-12, "amgcl")
        res[opt] = (prob, prob.amg_levels())
    A1f, A1 = res[0][1][1]["A"], res[-1][1][1]["A"]
    assert A1f.nnz < 0.7 * A1.nnz  # 40 nm cube: 305,284 of 476,414 entries
    scale = abs(A1).max()
    assert np.abs(np.asarray(A1f.sum(axis=1)) - np.asarray(A1.sum(axis=1))).max() <= 1e-12 * scale
    saved = opo.FILTER_EPS
    try:
        for opt, eps in ((0, 0.002), (-1, 0.0)):
            opo.FILTER_EPS = eps
            H = opo.build_hierarchy(ops["A"])
            prob, lv = res[opt]
            assert [x["A"].shape[0] for x in lv] == [lvl.A.shape[0] for lvl in H.levels]
            for a, b in zip(lv, H.levels):
                assert abs(a["A"] - b.A).max() <= 1e-13 * abs(b.A).max()
            su = opo.SolveU(p, ops, cg_tol=1e-10, hierarchy=H)
            U_o, it_o, _ = su(m, np.zeros(p.N), 1e-10, return_info=True)
            U, it, rr, rc = prob.solve_u(m, np.zeros(s.N), 1e-10)
            assert rc == 0 and rr <= 1e-10 and abs(it - it_o) <= 1
            assert rel(U, U_o) <= 1e-8
    finally:
        opo.FILTER_EPS = saved
