"""The product's C++ host setup (through the C-ABI) against the oracle; CPU only."""

from pathlib import Path

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import _abi
from mumag_matrixfree2_gb300 import synthetic as syn
from oracle import fem as ofem
from oracle import poisson as opo

from .helpers import case

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", ["cube8_h2_air24", "cube16_h2_air48"])
def test_geometry_and_mask(name):
    knt, ijk = syn.box_mesh(syn.WORKLOADS[name])
    conn, vol, JT = ofem.compute_volume_JinvT(knt, ijk[:, :4])
    c2, v2, JT2, gp2 = _abi.geom_compute(knt, ijk)
    assert np.array_equal(conn, c2)  # integer orientation fix: bit-exact
    assert np.allclose(v2, vol, rtol=1e-14, atol=0)
    assert np.allclose(JT2, JT, rtol=0, atol=1e-14 * np.abs(JT).max())
    assert np.allclose(gp2, ofem.grad_phi_from_JinvT(JT), rtol=0, atol=1e-14 * np.abs(JT).max())
    assert np.array_equal(_abi.boundary_mask(c2, knt.shape[0]), ofem.outer_boundary_mask(conn, knt.shape[0]))


@pytest.mark.parametrize("name", ["morton_cube8_h2_air24.npz", "morton_grid_box_10x7x5_h1.5.npz"])
def test_morton_matches_reference(name):
    d = np.load(GOLD / name)
    node_perm, elem_perm = _abi.morton_order(d["knt_in"], d["ijk_in"])
    assert np.array_equal(node_perm, d["node_perm"])
    inv = np.empty_like(node_perm)
    inv[node_perm] = np.arange(len(node_perm))
    ijk = d["ijk_in"][elem_perm].copy()
    ijk[:, :4] = inv[ijk[:, :4]]
    assert np.array_equal(ijk, d["ijk"])


@pytest.mark.parametrize("name", ["cube8_h2_air24", "cube16_h2_air48", "cube40_h2_air200"])
def test_amg_hierarchy_bit_exact_aggregates(name):
    s, p, _ = case(name)
    hs = _abi.HostSetup(s.geom.conn, s.geom.volume, s.geom.grad_phi, s.geom.mat_id, s.A_lookup, s.K1_lookup,
                        s.Js_lookup, s.k_easy, mask=s.boundary_mask, n_nodes=s.N)
    lv = hs.levels()
    ops = ofem.assembled_operators(p)
    H = opo.build_hierarchy(ops["A"])
    assert [x["A"].shape[0] for x in lv] == [x.A.shape[0] for x in H.levels]
    for a, b in zip(lv, H.levels):
        scale = abs(b.A).max()
        assert abs(a["A"] - b.A).max() <= 1e-13 * scale
        if b.agg is not None:
            assert np.array_equal(a["agg"], b.agg)
            assert abs(a["P"] - b.P).max() <= 1e-13


@pytest.mark.parametrize("tilt", [False, True])
def test_energy_operator_matches_assembled_matrices(tilt):
    s, p, _ = case("cube8_h2_air24", tilt_axis=tilt)
    hs = _abi.HostSetup(s.geom.conn, s.geom.volume, s.geom.grad_phi, s.geom.mat_id, s.A_lookup, s.K1_lookup,
                        s.Js_lookup, s.k_easy, mask=s.boundary_mask, n_nodes=s.N)
    eo = hs.energy_op()
    ops = ofem.assembled_operators(p)
    rng = np.random.default_rng(7)
    m = rng.standard_normal((p.N, 3))
    U = rng.standard_normal(p.N)
    rows = np.repeat(eo["rows"], np.diff(eo["ptr"]))
    kk = p.k_easy[eo["mat"]]
    t = -eo["q"] * np.einsum("ec,ec->e", kk, m[eo["col"]])
    contrib = eo["w"][:, None] * m[eo["col"]] + t[:, None] * kk + eo["G"] * U[eo["col"]][:, None]
    g = np.stack([np.bincount(rows, weights=contrib[:, c], minlength=p.N) for c in range(3)], 1)
    g_ref = (ops["K_eff"] @ m.reshape(-1)).reshape(-1, 3) + (ops["G"] @ U).reshape(3, -1).T
    assert np.abs(g - g_ref).max() <= 1e-13 * np.abs(g_ref).max()
    b = np.bincount(rows, weights=np.einsum("ec,ec->e", eo["D"], m[eo["col"]]), minlength=p.N)
    b_ref = ofem.rhs_from_m_asm(ops, m)
    assert np.abs(b - b_ref).max() <= 1e-13 * np.abs(b_ref).max()
    assert np.allclose(eo["diag_exchange"] / p.V_mag, ofem.exchange_diagonal(p), rtol=1e-13, atol=0)


@pytest.mark.parametrize("name", ["cube8_h2_air24", "cube16_h2_air48"])
def test_rcm_order_equals_scipy(name):
    """Reverse Cuthill-McKee of the edge graph: node permutation bit-exact against
    scipy.sparse.csgraph.reverse_cuthill_mckee on the same symmetric graph; elements ordered by the
    mean new node number as src/reorder_mesh.py:79-83 orders them."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import reverse_cuthill_mckee

    knt, ijk = syn.box_mesh(syn.WORKLOADS[name])
    conn = ijk[:, :4].astype(np.int64)
    N = knt.shape[0]
    pairs = [(a, b) for a in range(4) for b in range(4) if a != b]
    rows = np.concatenate([conn[:, a] for a, _ in pairs])
    cols = np.concatenate([conn[:, b] for _, b in pairs])
    adj = sp.coo_matrix((np.ones(len(rows), dtype=bool), (rows, cols)), shape=(N, N)).tocsr()
    ref = reverse_cuthill_mckee(adj, symmetric_mode=True)
    npm, epm = _abi.rcm_order(conn, N)
    assert np.array_equal(npm, ref)
    inv = np.empty(N, np.int64)
    inv[ref] = np.arange(N)
    assert np.array_equal(epm, np.argsort(np.mean(inv[conn], axis=1)))
    # the renumbered mesh has a smaller bandwidth than the grid order
    bw = lambda c: int(np.max(np.ptp(c, axis=1)))  # noqa: E731
    assert bw(inv[conn]) < bw(conn)


def test_concurrent_setups_equal_a_lone_setup():
    """Setups running at once share the host's threads (fewer threads per parallel pass); every pass
    gives the same result for any thread count, so each concurrent hierarchy equals a lone one bit for
    bit.  The C-ABI calls release the GIL, so the four setups overlap."""
    from concurrent.futures import ThreadPoolExecutor

    s, _, _ = case("cube40_h2_air200")

    def build(_=None):
        hs = _abi.HostSetup(s.geom.conn, s.geom.volume, s.geom.grad_phi, s.geom.mat_id, s.A_lookup, s.K1_lookup,
                            s.Js_lookup, s.k_easy, mask=s.boundary_mask, n_nodes=s.N)
        return hs.energy_op(), hs.levels()

    e0, lv0 = build()
    with ThreadPoolExecutor(max_workers=4) as ex:
        runs = list(ex.map(build, range(4)))
    for e, lv in runs:
        for k in ("rows", "ptr", "col", "mat", "w", "q", "G", "D", "diag_exchange"):
            assert np.array_equal(e[k], e0[k]), k
        assert len(lv) == len(lv0)
        for a, b in zip(lv, lv0):
            assert np.array_equal(a["agg"], b["agg"])
            for k in ("A", "P"):
                if k in b:
                    assert (a[k] != b[k]).nnz == 0 and np.array_equal(a[k].indices, b[k].indices), k
