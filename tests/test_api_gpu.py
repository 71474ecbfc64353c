"""The reference-API mirror (make_energy_kernels / make_solve_U / make_minimizer / run_hysteresis_loop)
against the FP64 oracle, and the mixed-precision loop against the plain FP64 loop."""

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import fem_utils
from mumag_matrixfree2_gb300.energy_kernels import compute_exchange_diagonal, make_energy_kernels
from mumag_matrixfree2_gb300.hysteresis_loop import LoopParams, run_hysteresis_loop
from mumag_matrixfree2_gb300.minimizers import make_minimizer
from mumag_matrixfree2_gb300.poisson_solve import make_solve_U
from mumag_matrixfree2_gb300 import synthetic as syn
from oracle import fem as ofem
from oracle import minimize as omin
from oracle import poisson as opo

from .helpers import case, random_state

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300))


def test_factories_match_oracle(cuda_ok):
    s, p, _ = case("cube8_h2_air24")
    g = s.geom
    eg, eo, go, lg = make_energy_kernels(g, s.A_lookup, s.K1_lookup, s.Js_lookup, s.k_easy, s.V_mag, s.M_nodal,
                                         mode="assembled")
    ops = ofem.assembled_operators(p)
    m = random_state(p.N, seed=41)
    U = np.random.default_rng(42).standard_normal(p.N)
    B = np.array([0.0, 0.1, -0.4])
    E, gr = eg(m, U, B)
    E0, g0 = ofem.energy_and_grad_asm(p, ops, m, U, B)
    assert abs(E - E0) <= 1e-10 * abs(E0) and rel(gr, g0) <= 1e-10
    assert abs(eo(m, U, B) - E0) <= 1e-10 * abs(E0)
    assert rel(lg(m), ofem.local_grad_only_asm(p, ops, m)) <= 1e-10
    assert rel(compute_exchange_diagonal(g, s.A_lookup, s.V_mag), ofem.exchange_diagonal(p)) <= 1e-10
    solve_U = make_solve_U(g, s.Js_lookup, precond_type="amgcl", cg_tol=1e-10, boundary_mask=s.boundary_mask)
    U1, it, rr = solve_U(m, np.zeros(p.N), return_info=True)
    U0, it0, rr0 = opo.SolveU(p, ops, cg_tol=1e-10)(m, np.zeros(p.N), return_info=True)
    assert abs(it - it0) <= 1 and rr <= 1e-10 and rel(U1, U0) <= 1e-8


def _oracle_ops(p, ops, su):
    d = ofem.exchange_diagonal(p)
    return omin.Ops(
        energy_and_grad=lambda m, U, B: ofem.energy_and_grad_asm(p, ops, m, U, B),
        local_grad_only=lambda v: ofem.local_grad_only_asm(p, ops, v),
        solve_U=lambda m, x0, tol: su(m, x0, tol, return_info=True),
        inv_M_rel=np.where(p.M_nodal > 1e-20, p.V_mag / np.where(p.M_nodal > 0, p.M_nodal, 1), 0.0)[:, None],
        inv_M_prec=np.where(d > 1e-20, 1.0 / np.where(d > 0, d, 1), 1.0)[:, None],
    )


def _sweep_params(Js_ref, out_dir):
    h = syn.tilted_field_direction(1.0)
    return LoopParams(h_dir=h, B_start=8.0 / Js_ref, B_end=-8.0 / Js_ref, dB=0.5 / Js_ref, loop=False, tau_f=1e-8,
                      eps_a=1e-12, cg_tol=1e-10, pc_iters=10, pc_stagnation_nu=0.01, Js_ref=Js_ref,
                      out_dir=str(out_dir), max_iter=2000)


def _switch(hist):
    J = hist[:, 1]
    return int(np.argmax(J < 0)) if np.any(J < 0) else -1


def test_hysteresis_sweep_matches_oracle(cuda_ok, tmp_path):
    """Field sweep +8 T -> -8 T (0.5 T steps, 1 deg tilt) of an 8 nm NdFeB cube in air: the GPU loop
    gives the oracle's switching step, coercive field (0.5 %) and per-step polarisation."""
    s, p, Js_ref = case("cube8_h2_air24")
    prm = _sweep_params(Js_ref, tmp_path / "gpu")
    m0 = syn.initial_state(p.N, seed=0)
    res = run_hysteresis_loop(s.knt, s.geom, s.A_lookup, s.K1_lookup, s.Js_lookup, s.k_easy, m0, prm, s.V_mag,
                              s.node_volumes, s.M_nodal, boundary_mask=s.boundary_mask, precond_type="amgcl")
    ops = ofem.assembled_operators(p)
    su = opo.SolveU(p, ops, cg_tol=1e-10)
    O = _oracle_ops(p, ops, su)
    B_vals = syn.field_values(prm.B_start, prm.B_end, prm.dB, False)
    oprm = omin.Params(max_iter=2000, tau_f=1e-8, eps_a=1e-12, cg_tol=1e-10)
    hist_o, _, _ = omin.run_sweep(O, p, m0, np.asarray(prm.h_dir), B_vals, oprm, Js_ref=Js_ref)
    hist_o = np.array(hist_o)
    hist = res["history"]
    assert len(hist) == len(hist_o)
    sw, sw_o = _switch(hist), _switch(hist_o)
    assert sw == sw_o and sw > 0
    Hc = omin.compute_coercivity(hist[:, 0], hist[:, 1])
    Hc_o = omin.compute_coercivity(hist_o[:, 0], hist_o[:, 1])
    assert abs(Hc - Hc_o) <= 5e-3 * abs(Hc_o)
    assert np.max(np.abs(hist[:sw, 1] - hist_o[:sw, 1])) <= 1e-6
    assert (tmp_path / "gpu" / "hysteresis.csv").read_text().startswith("config,B_ext_T,J_par_T,E,gnorm")


def test_mixed_precision_loop_matches_plain(cuda_ok, tmp_path):
    s, p, Js_ref = case("cube16_h2_air48")
    m0 = syn.initial_state(p.N, seed=0)
    out = {}
    for precision in ("fp64", "mixed"):
        g = fem_utils.TetGeom(conn=s.geom.conn, volume=s.geom.volume, mat_id=s.geom.mat_id, grad_phi=s.geom.grad_phi,
                              x_nodes=s.knt)  # a fresh geometry object: its own device problem
        prm = _sweep_params(Js_ref, tmp_path / precision)
        out[precision] = run_hysteresis_loop(s.knt, g, s.A_lookup, s.K1_lookup, s.Js_lookup, s.k_easy, m0, prm,
                                             s.V_mag, s.node_volumes, s.M_nodal, boundary_mask=s.boundary_mask,
                                             precond_type="amgcl", precision=precision, write_files=False)
    h64, h32 = out["fp64"]["history"], out["mixed"]["history"]
    assert _switch(h64) == _switch(h32) > 0
    Hc64 = omin.compute_coercivity(h64[:, 0], h64[:, 1])
    Hc32 = omin.compute_coercivity(h32[:, 0], h32[:, 1])
    assert abs(Hc32 - Hc64) <= 5e-3 * abs(Hc64)
    sw = _switch(h64)
    assert np.max(np.abs(h64[:sw, 1] - h32[:sw, 1])) <= 1e-5
