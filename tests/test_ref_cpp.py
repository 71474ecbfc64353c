"""The oracle pinned to the reference's own C++ minimizer (CPU tests).

``oracle/_ref/libcpp_mkl_minimizer.so`` is the reference's ``src/cpp/cpp_mkl_minimizer.cpp``
compiled unchanged against the project's MKL-API shim; where its source is not available only the
fixture tests run (``tests/golden/ref_cpp_*.npz``, written by ``make_ref_golden.py`` from that
library).  The tolerances are the reference's own cross-implementation bar of 1e-10
(``tests/test_compare_kernels.py:303,309,376``) or tighter.
"""

from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

from mumag_matrixfree2_gb300 import synthetic as syn
from oracle import build_ref, ref_cpp
from oracle import fem as ofem
from oracle import minimize as omin
from oracle import poisson as opo
from tests import helpers as H

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def libs():
    build_ref.build()
    return ref_cpp.load("reference"), ref_cpp.load("port")


def need_ref(libs):
    if libs[0] is None:
        pytest.skip("the reference source is not available here, so oracle/_ref was not built")
    return libs[0]


def oracle_ops(p, cp, cg_tol=1e-12):
    ops = ofem.assembled_operators(p)
    solver = opo.SolveU(p, ops, cg_tol=cg_tol)
    return ops, omin.Ops(energy_and_grad=lambda m, U, B: ofem.energy_and_grad_asm(p, ops, m, U, B),
                         local_grad_only=lambda v: ofem.local_grad_only_asm(p, ops, v),
                         solve_U=lambda m, x0, tol: solver(m, x0, tol, return_info=True),
                         inv_M_rel=cp.inv_M_rel[:, None], inv_M_prec=cp.inv_M_prec[:, None])


def test_shim_blas_and_pardiso(libs):
    """The shim itself: CSR products equal scipy's, pardiso() reaches its relative residual."""
    port = libs[1]
    s, p, _ = H.case("cube16_h2_air48")
    cp = ref_cpp.CppProblem(port, p)
    ops = ref_cpp.interleaved_operators(p)
    rng = np.random.default_rng(3)
    m = rng.standard_normal((p.N, 3))
    U_in = rng.standard_normal(p.N)
    E, g = cp.energy_and_grad(m, U_in, np.zeros(3))
    g_ref = (ops["K_eff"] @ m.reshape(-1) + ops["G"] @ U_in) / p.V_mag
    assert np.allclose(g.reshape(-1), g_ref, rtol=0, atol=1e-14 * np.abs(g_ref).max())
    U = cp.solve_poisson(m)
    it, rr = port.last_solve()
    b = (ops["D"] @ m.reshape(-1)) * p.boundary_mask
    res = np.linalg.norm(b - ops["A"] @ U) / np.linalg.norm(b)
    assert 0 < it < 100 and rr <= 1e-12 and res <= 2e-12


def test_reference_energy_and_gradient_match_oracle(libs):
    lib = need_ref(libs)
    for name in ("cube8_h2_air24", "cube16_h2_air48"):
        s, p, _ = H.case(name)
        cp = ref_cpp.CppProblem(lib, p)
        m, U, B = H.ref_state(name)
        E, g = cp.energy_and_grad(m, U, B)
        E0, g0 = ofem.energy_and_grad_mf(p, m, U, B)
        assert abs(E - E0) <= 1e-12 * abs(E0)
        assert np.abs(g - g0).max() <= 1e-12 * np.abs(g0).max()


def test_reference_inner_solve_matches_oracle(libs):
    """solve_Py_g after one inner iteration (the reference's own check) and after ten."""
    lib = need_ref(libs)
    s, p, _ = H.case("cube16_h2_air48")
    cp = ref_cpp.CppProblem(lib, p)
    ops, oo = oracle_ops(p, cp)
    m, U, B = H.ref_state("cube16_h2_air48")
    _, g = ofem.energy_and_grad_asm(p, ops, m, U, B)
    gt = omin.tangent_grad(m, g)
    for iters in (1, 10):
        y, it = cp.solve_Py_g(m, g, gt, iters, 0.0, 0.0, 1e-3)
        y0, it0 = omin.solve_Py_g(oo, m, g, gt, iters, 0.0, 0.0, 1e-3, cpp_count=True)
        assert it == it0
        assert np.abs(y - y0).max() <= 1e-12 * np.abs(y0).max()


def test_reference_demag_solve_matches_oracle(libs):
    lib = need_ref(libs)
    s, p, _ = H.case("cube16_h2_air48")
    cp = ref_cpp.CppProblem(lib, p)
    m, _, _ = H.ref_state("cube16_h2_air48")
    U = cp.solve_poisson(m)
    U0, _, rr = opo.SolveU(p, cg_tol=1e-12)(m, np.zeros(p.N), 1e-12, return_info=True)
    assert rr <= 1e-12
    assert np.abs(U - U0).max() <= 1e-10 * np.abs(U0).max()


@pytest.mark.parametrize("method", ["pcohen_hs", "pcohen"])
def test_reference_minimizer_matches_oracle_cpp_flavour(libs, method):
    """run_cpp_pcohen_hs_minimization vs the oracle's minimizer with the C++ conventions: same
    iterations, evaluations and inner iterations on each field step, same energy and state."""
    lib = need_ref(libs)
    s, p, Js_ref = H.case("cube8_h2_air24")
    cp = ref_cpp.CppProblem(lib, p)
    _, oo = oracle_ops(p, cp)
    prm = H.ref_min_params()
    h = syn.tilted_field_direction(1.0)
    m = mo = syn.initial_state(p.N)
    U = Uo = np.zeros(p.N)
    for BT in H.REF_FIELDS_T:
        B = (BT / Js_ref) * h
        m, U, info = cp.minimize(m, B, U, prm, method)
        mo, Uo, io = omin.minimize(oo, mo, B, Uo, prm, method, flavour="cpp")
        assert (info["iters"], info["evals"], info["preco_iters"]) == (io["iters"], io["evals"], io["preco_iters"])
        assert abs(info["E"] - io["E"]) <= 1e-11 * abs(io["E"])
        assert np.abs(m - mo).max() <= 1e-10


def test_port_equals_reference(libs):
    """The restated entry points (timed as the CPU baseline where the reference source is absent)
    give the reference library's results."""
    ref, port = need_ref(libs), libs[1]
    s, p, _ = H.case("cube16_h2_air48")
    a, b = ref_cpp.CppProblem(ref, p), ref_cpp.CppProblem(port, p)
    m, U, B = H.ref_state("cube16_h2_air48")
    Ea, ga = a.energy_and_grad(m, U, B)
    Eb, gb = b.energy_and_grad(m, U, B)
    assert abs(Ea - Eb) <= 1e-14 * abs(Ea) and np.abs(ga - gb).max() <= 1e-15 * np.abs(ga).max()
    assert np.array_equal(a.solve_poisson(m), b.solve_poisson(m))


@pytest.mark.parametrize("name", list(H.REF_CASES))
def test_fixtures_match_oracle(name):
    """The committed fixtures of the reference's C++ against the oracle (runs without the reference)."""
    f = np.load(GOLDEN / f"ref_cpp_{name}.npz")
    s, p, _ = H.case(name)
    idx = f["idx"]
    assert int(f["N"]) == p.N and np.array_equal(idx, H.ref_sample(p.N, int(f["stride"])))
    m, U, B = H.ref_state(name)
    E0, g0 = ofem.energy_and_grad_mf(p, m, U, B)
    assert abs(float(f["E"]) - E0) <= 1e-12 * abs(E0)
    assert np.abs(f["g"] - g0[idx]).max() <= 1e-12 * np.abs(g0).max()
    assert np.allclose(f["g_sums"][:2], [g0.sum(), (g0 * g0).sum()], rtol=1e-10, atol=1e-14)
    U0, _, _ = opo.SolveU(p, cg_tol=1e-12)(m, np.zeros(p.N), 1e-12, return_info=True)
    assert np.abs(f["U"] - U0[idx]).max() <= 1e-10 * np.abs(U0).max()


def test_loop_fixture_shape():
    """The reference loop fixture: 161 fields from +8 to -8 T, one switch, a coercive field."""
    f = np.load(GOLDEN / "ref_cpp_loop_cube40_h2_air200.npz")
    B, J = f["B_T"], f["J_T"]
    assert len(B) == 161 and abs(B[0] - 8.0) < 1e-9 and abs(B[-1] + 8.0) < 1e-9
    k = int(f["switch_index"])
    assert J[0] > 1.5 and J[-1] < -1.5 and np.all(J[:k] > 0) and J[k] < 0
    assert abs(float(f["Hc_T"]) - omin.compute_coercivity(B, J)) < 1e-12
    assert sp.issparse(sp.csr_matrix((1, 1)))  # scipy available for the fixture users
