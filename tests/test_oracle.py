"""The oracle against the reference's golden data and known answers (CPU only)."""

from pathlib import Path

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import synthetic as syn
from oracle import fem as ofem
from oracle import minimize as omin
from oracle import poisson as opo

from .helpers import case

GOLD = Path(__file__).resolve().parent / "golden"
MU0 = 4e-7 * np.pi


def test_grid_box_matches_reference_mesher():
    # the reference's structured mesher output (and with it the reference's tests/single_solid.npz)
    d = np.load(GOLD / "grid_box_20x20x20_h2.npz")
    assert bool(d["equals_reference_single_solid"])
    knt, ijk = syn.box_mesh(syn.WORKLOADS["cube20_h2"])
    assert np.array_equal(knt, d["knt"]) and np.array_equal(ijk, d["ijk"])
    for name, ext, h in [("grid_box_8x6x4_h2.npz", (8.0, 6.0, 4.0), 2.0),
                         ("grid_box_10x7x5_h1.5.npz", (10.0, 7.0, 5.0), 1.5)]:
        d = np.load(GOLD / name)
        axes = [np.linspace(-L / 2, L / 2, int(np.ceil(L / h)) + 1) for L in ext]
        knt, tets = syn.kuhn_box_mesh(*axes)
        assert np.array_equal(knt, d["knt"])
        assert np.array_equal(tets, d["ijk"][:, :4])


@pytest.mark.parametrize("name", ["morton_cube8_h2_air24.npz", "morton_grid_box_10x7x5_h1.5.npz"])
def test_morton_order_matches_reference(name):
    d = np.load(GOLD / name)
    node_perm, elem_perm = ofem.morton_order(d["knt_in"], d["ijk_in"])
    assert np.array_equal(node_perm, d["node_perm"])
    inv = np.empty_like(node_perm)
    inv[node_perm] = np.arange(len(node_perm))
    ijk = d["ijk_in"][elem_perm].copy()
    ijk[:, :4] = inv[ijk[:, :4]]
    assert np.array_equal(ijk, d["ijk"])
    assert np.array_equal(d["knt_in"][node_perm], d["knt"])


def test_boundary_mask_is_box_surface():
    s, p, _ = case("cube8_h2_air24")
    lo, hi = p.knt.min(axis=0), p.knt.max(axis=0)
    on_face = np.any((p.knt == lo) | (p.knt == hi), axis=1)
    assert np.array_equal(p.boundary_mask == 0, on_face)


def test_orientation_fix_gives_positive_volumes():
    s, p, _ = case("cube8_h2_air24")
    x0 = p.knt[p.conn[:, 0]]
    J = np.stack([p.knt[p.conn[:, k]] - x0 for k in (1, 2, 3)], axis=2)
    assert np.all(np.linalg.det(J) > 0)
    assert np.allclose(p.volume.sum(), 24.0**3)


def test_assembled_equals_matrix_free():
    # src/energy_kernels.py assembled vs matrix-free (the reference compares its two
    # implementations in tests/test_compare_kernels.py at 1e-10)
    _, p, _ = case("cube8_h2_air24")
    ops = ofem.assembled_operators(p)
    rng = np.random.default_rng(3)
    m = rng.standard_normal((p.N, 3))
    U = rng.standard_normal(p.N)
    E1, g1 = ofem.energy_and_grad_mf(p, m, U, [0.1, -0.2, 0.3])
    E2, g2 = ofem.energy_and_grad_asm(p, ops, m, U, [0.1, -0.2, 0.3])
    assert abs(E1 - E2) <= 1e-12 * abs(E1)
    assert np.abs(g1 - g2).max() <= 1e-12 * np.abs(g1).max()
    assert np.allclose(ofem.local_grad_only_mf(p, m), ofem.local_grad_only_asm(p, ops, m), rtol=0, atol=1e-12 * np.abs(g1).max())
    assert np.allclose(ofem.rhs_from_m_mf(p, m), ofem.rhs_from_m_asm(ops, m), rtol=0, atol=1e-13)
    # the Dirichlet assembled operator acts like the masked matrix-free one on interior rows
    mask = p.boundary_mask
    y1 = ofem.apply_A_asm(ops, U * mask) * mask
    y2 = ofem.apply_A_mf(p, U * mask, mask=mask)
    assert np.abs(y1 - y2).max() <= 1e-12 * np.abs(y1).max()


def _analytic_case():
    # 20 nm cube at h = 2 nm inside a graded air box; Js = 1.6 T, K1 = 4.3 MJ/m^3, A = 7.7 pJ/m
    w = syn.BoxWorkload("cube20_air60", L=20.0, h=2.0, r=1.25, n_air=5, box=60.0)
    knt, ijk = syn.box_mesh(w)
    mats = [syn.Material(Js=1.6, A=7.7e-12, K1=4.3e6), syn.AIR]
    A, K1, Js, k, Js_ref = syn.reduced_materials(mats)
    return knt, ijk, A, K1, Js, k, Js_ref


def test_analytic_energies():
    """Known answers of the reference's tests/test_energy.py:21-145 on this project's mesh."""
    knt, ijk, A, K1, Js, k, Js_ref = _analytic_case()
    p = ofem.make_problem(knt, ijk, A, K1, Js, k)
    Kd = Js_ref**2 / (2 * MU0)
    V_si = p.V_mag * 1e-27
    si = Kd * V_si
    N = p.N
    zero = np.zeros(N)
    kw = np.pi / 20.0
    m_hel = np.stack([np.cos(kw * knt[:, 0]), np.sin(kw * knt[:, 0]), np.zeros(N)], 1)
    e_ex, _ = ofem.energy_and_grad_mf(p, m_hel, zero, np.zeros(3))
    assert abs(e_ex * si - 7.7e-12 * (kw * 1e9) ** 2 * V_si) / (7.7e-12 * (kw * 1e9) ** 2 * V_si) < 0.02
    m_x = np.tile([1.0, 0, 0], (N, 1))
    pz = ofem.make_problem(knt, ijk, A * 0, K1 * 0, Js, k)
    e_z, _ = ofem.energy_and_grad_mf(pz, m_x, zero, np.array([0.1 / Js_ref, 0, 0]))
    E_z = -(1.0 / MU0) * 1.6 * V_si * 0.1
    assert abs(e_z * si - E_z) / abs(E_z) < 1e-6
    m45 = np.tile(np.array([1.0, 0, 1.0]) / np.sqrt(2), (N, 1))
    pa = ofem.make_problem(knt, ijk, A * 0, K1, Js * 0, k)
    pa.M_nodal[:] = 0.0
    pa.V_mag = p.V_mag
    e_an, _ = ofem.energy_and_grad_mf(pa, m45, zero, np.zeros(3))
    assert abs(e_an * si - (-4.3e6 * V_si * 0.5)) / (4.3e6 * V_si * 0.5) < 1e-6
    su = opo.SolveU(pz, cg_tol=1e-12)
    u = su(m_x, zero)
    e_dem, _ = ofem.energy_and_grad_mf(pz, m_x, u, np.zeros(3))
    assert abs(e_dem - 1.0 / 3.0) < 0.05


def test_fd_gradients():
    """Central differences as tests/test_gradients.py:105-277 (first 5 magnetic nodes, abs 1e-5)."""
    knt, ijk, A, K1, Js, k, Js_ref = _analytic_case()
    p = ofem.make_problem(knt, ijk, A, K1, Js, k)
    N = p.N
    nodes = np.unique(p.conn[p.mat_id == 1])[:5]
    m = np.stack([np.cos(0.1 * knt[:, 0]), np.sin(0.1 * knt[:, 0]), 0.3 * np.ones(N)], 1)
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    su = opo.SolveU(p, cg_tol=1e-12)
    U = su(m, np.zeros(N))
    B = np.array([0.05, -0.02, 0.1])
    E0, g = ofem.energy_and_grad_mf(p, m, U, B)
    eps = 1e-6
    for i in nodes:
        for j in range(3):
            mp, mm = m.copy(), m.copy()
            mp[i, j] += eps
            mm[i, j] -= eps
            # exchange + anisotropy + Zeeman are exact quadratic/linear forms: FD of E(m; U fixed)
            # equals g minus half the demag part (the energy trick counts U as fixed)
            Ep, _ = ofem.energy_and_grad_mf(p, mp, U, B)
            Em, _ = ofem.energy_and_grad_mf(p, mm, U, B)
            g_nodem = g[i, j] - 0.5 * ofem.energy_and_grad_mf(p, np.zeros_like(m), U, np.zeros(3))[1][i, j]
            assert abs((Ep - Em) / (2 * eps) - g_nodem) < 1e-5
            # with U re-solved from m the FD of the reduced energy is the full gradient
            Ep2, _ = ofem.energy_and_grad_mf(p, mp, su(mp, U), B)
            Em2, _ = ofem.energy_and_grad_mf(p, mm, su(mm, U), B)
            assert abs((Ep2 - Em2) / (2 * eps) - g[i, j]) < 1e-5


def test_oracle_pcg_converges_to_tolerance():
    _, p, _ = case("cube16_h2_air48")
    su = opo.SolveU(p, cg_tol=1e-10)
    m = np.tile([0.3, 0.1, 1.0], (p.N, 1))
    U, it, rr = su(m, np.zeros(p.N), 1e-10, return_info=True)
    assert rr <= 1e-10 and 0 < it < 60
    b = su.rhs(m)
    true_rr = np.linalg.norm(b - su.apply_A(U)) / np.linalg.norm(b)
    assert true_rr < 1e-9


def test_oracle_minimizer_decreases_energy():
    _, p, _ = case("cube8_h2_air24")
    ops = ofem.assembled_operators(p)
    su = opo.SolveU(p, ops, cg_tol=1e-10)
    d = ofem.exchange_diagonal(p)
    O = omin.Ops(
        energy_and_grad=lambda m, U, B: ofem.energy_and_grad_asm(p, ops, m, U, B),
        local_grad_only=lambda v: ofem.local_grad_only_asm(p, ops, v),
        solve_U=lambda m, x0, tol: su(m, x0, tol, return_info=True),
        inv_M_rel=np.where(p.M_nodal > 1e-20, p.V_mag / np.where(p.M_nodal > 0, p.M_nodal, 1), 0.0)[:, None],
        inv_M_prec=np.where(d > 1e-20, 1.0 / np.where(d > 0, d, 1), 1.0)[:, None],
    )
    m0 = syn.initial_state(p.N, amplitude=0.2)
    B = np.array([0.0, 0.0, -0.5])
    for method in omin.METHODS:
        prm = omin.Params(max_iter=30, tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10)
        U0, _, _ = su(m0, np.zeros(p.N), 1e-10, return_info=True)
        E0, _ = O.energy_and_grad(m0, U0, B)
        m, U, info = omin.minimize(O, m0, B, np.zeros(p.N), prm, method)
        assert info["E"] < E0
        assert np.allclose(np.linalg.norm(m, axis=1), 1.0)


def test_filter_weak_keeps_row_sums_and_symmetry():
    """The level-1 filter of the oracle's hierarchy: a symmetric decision (|a_ij| + |a_ji| against
    2 eps sqrt(|a_ii a_jj|)), the dropped values added to their row's diagonal (row sums kept), the
    kept off-diagonal entries untouched."""
    import scipy.sparse as sp

    rng = np.random.default_rng(5)
    n = 80
    M = sp.random(n, n, density=0.15, random_state=rng, format="csr")
    M.data = M.data * rng.choice([-1.0, 1.0], size=M.nnz) * np.exp(-6.0 * rng.random(M.nnz))
    A = (M + M.T).tocsr()
    A = (A + sp.diags(np.asarray(abs(A).sum(axis=1)).ravel() + 1.0)).tocsr()
    A.sort_indices()
    eps = 0.01
    F = opo.filter_weak(A, eps)
    assert F.nnz < A.nnz
    assert abs(F - F.T).max() == 0.0
    assert np.allclose(np.asarray(F.sum(axis=1)).ravel(), np.asarray(A.sum(axis=1)).ravel(), rtol=1e-14, atol=1e-14)
    d = A.diagonal()
    C = F.tocoo()
    off = C.row != C.col
    kept = np.asarray(abs(A)[C.row[off], C.col[off]]).ravel() * 2.0
    assert np.all(kept >= 2.0 * eps * np.sqrt(np.abs(d[C.row[off]] * d[C.col[off]])))
    assert np.array_equal(np.asarray(A[C.row[off], C.col[off]]).ravel(), C.data[off])
