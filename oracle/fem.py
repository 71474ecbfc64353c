"""FP64 restatement of the reference's P1-tetrahedron geometry, assembly and energy operators.

Test infrastructure (see ``oracle/__init__.py``).  Reference files are cited as path:line of
MaMMoS-project/mumag_matrixfree2.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp

GRAD_HAT = np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


# --------------------------------------------------------------------------------------------
# geometry (src/loop.py:56-102, src/fem_utils.py:174-212, src/add_shell.py:105-136)
# --------------------------------------------------------------------------------------------
def compute_volume_JinvT(knt: np.ndarray, conn: np.ndarray):
    """Orientation fix (swap local nodes 1 and 2 where det J < 0), volumes and inv(J)^T.

    Follows ``src/loop.py:56-90``.
    """
    knt = np.asarray(knt, dtype=np.float64)
    conn = np.asarray(conn, dtype=np.int64)
    x0 = knt[conn[:, 0]]
    J = np.stack([knt[conn[:, 1]] - x0, knt[conn[:, 2]] - x0, knt[conn[:, 3]] - x0], axis=2)
    detJ = np.linalg.det(J)
    neg = detJ < 0
    if np.any(neg):
        conn = conn.copy()
        tmp = conn[neg, 1].copy()
        conn[neg, 1] = conn[neg, 2]
        conn[neg, 2] = tmp
        x0 = knt[conn[:, 0]]
        J = np.stack([knt[conn[:, 1]] - x0, knt[conn[:, 2]] - x0, knt[conn[:, 3]] - x0], axis=2)
        detJ = np.linalg.det(J)
    volume = np.abs(detJ) / 6.0
    JinvT = np.swapaxes(np.linalg.inv(J), 1, 2)
    return conn.astype(np.int32), volume.astype(np.float64), JinvT.astype(np.float64)


def grad_phi_from_JinvT(JinvT: np.ndarray) -> np.ndarray:
    """Shape-function gradients (E,4,3), ``src/loop.py:93-102``."""
    return np.einsum("eij,aj->eai", JinvT, GRAD_HAT)


def outer_boundary_mask(conn: np.ndarray, n_nodes: int) -> np.ndarray:
    """1.0 interior, 0.0 on faces that belong to exactly one tetrahedron (``src/add_shell.py:105-136``)."""
    t4 = np.asarray(conn)[:, :4].astype(np.int64)
    fp = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]])
    keys = np.sort(t4[:, fp].reshape(-1, 3), axis=1)
    _, inv, cnt = np.unique(keys, axis=0, return_inverse=True, return_counts=True)
    faces = keys[cnt[inv.ravel()] == 1]
    mask = np.ones(n_nodes, dtype=np.float64)
    mask[np.unique(faces)] = 0.0
    return mask


def node_sum(conn: np.ndarray, contrib: np.ndarray, n_nodes: int) -> np.ndarray:
    """Scatter-add element-vertex contributions (E,4[,k]) to nodes, in element order."""
    idx = np.asarray(conn).reshape(-1)
    if contrib.ndim == 2:
        return np.bincount(idx, weights=contrib.reshape(-1), minlength=n_nodes)
    out = np.empty((n_nodes, contrib.shape[2]))
    for c in range(contrib.shape[2]):
        out[:, c] = np.bincount(idx, weights=contrib[:, :, c].reshape(-1), minlength=n_nodes)
    return out


def node_volumes(conn: np.ndarray, volume: np.ndarray, n_nodes: int) -> np.ndarray:
    """Lumped nodal volumes sum_e Ve/4 (``src/fem_utils.py:174-212``)."""
    return node_sum(conn, np.broadcast_to((0.25 * volume)[:, None], (len(volume), 4)), n_nodes)


@dataclass
class Problem:
    """Everything the operators need, in reduced units (``src/loop.py:845-939``)."""

    knt: np.ndarray
    conn: np.ndarray  # (E,4) int32, oriented
    volume: np.ndarray
    grad_phi: np.ndarray  # (E,4,3)
    mat_id: np.ndarray  # (E,) int32, 1-based
    A_lookup: np.ndarray
    K1_lookup: np.ndarray
    Js_lookup: np.ndarray
    k_easy: np.ndarray  # (G,3)
    V_mag: float
    M_nodal: np.ndarray
    boundary_mask: np.ndarray | None

    @property
    def N(self) -> int:
        return self.knt.shape[0]


def make_problem(knt, ijk, A_lookup, K1_lookup, Js_lookup, k_easy, with_boundary=True) -> Problem:
    """Geometry precompute, V_mag, M_nodal and the Dirichlet mask as ``src/loop.py:856-939`` does."""
    ijk = np.asarray(ijk)
    conn32, volume, JinvT = compute_volume_JinvT(knt, ijk[:, :4])
    mat_id = ijk[:, 4].astype(np.int32) if ijk.shape[1] > 4 else np.ones(len(ijk), np.int32)
    if mat_id.min() == 0:
        mat_id = mat_id + 1
    Js_lookup = np.asarray(Js_lookup, dtype=np.float64)
    is_mag = np.isin(mat_id, np.where(Js_lookup > 0)[0] + 1)
    V_mag = float(np.sum(volume[is_mag])) or 1.0
    M_nodal = node_volumes(conn32, volume * Js_lookup[mat_id - 1], knt.shape[0])
    mask = outer_boundary_mask(conn32, knt.shape[0]) if with_boundary else None
    return Problem(
        knt=np.asarray(knt, np.float64), conn=conn32, volume=volume, grad_phi=grad_phi_from_JinvT(JinvT),
        mat_id=mat_id, A_lookup=np.asarray(A_lookup, np.float64), K1_lookup=np.asarray(K1_lookup, np.float64),
        Js_lookup=Js_lookup, k_easy=np.asarray(k_easy, np.float64), V_mag=V_mag, M_nodal=M_nodal,
        boundary_mask=mask,
    )


# --------------------------------------------------------------------------------------------
# matrix-free element loops (src/energy_kernels.py:199-566, src/poisson_solve.py:210-299)
# --------------------------------------------------------------------------------------------
def _coeffs(p: Problem):
    g = p.mat_id - 1
    A_Ve = 2.0 * p.A_lookup[g] * p.volume  # src/energy_kernels.py:208
    K1_Ve = 2.0 * p.K1_lookup[g] * p.volume / 20.0  # :209
    Js_Ve = 2.0 * p.Js_lookup[g] * p.volume / 4.0  # :210
    return A_Ve, K1_Ve, Js_Ve, p.k_easy[g]


def _exchange_aniso_contrib(p: Problem, v: np.ndarray) -> np.ndarray:
    """Per element-vertex exchange + anisotropy contribution (E,4,3), ``src/energy_kernels.py:374-400``."""
    A_Ve, K1_Ve, _, k = _coeffs(p)
    B = p.grad_phi  # (E,4,3): B[e,a,i] = d phi_a / d x_i
    v_e = v[p.conn]  # (E,4,3)
    grad_v = np.einsum("ebi,ebc->eci", B, v_e)  # (E, comp c, dir i)
    Km = np.einsum("eai,eci->eac", B, grad_v)  # (E, a, c)
    contrib = A_Ve[:, None, None] * Km
    proj = np.einsum("ebc,ec->eb", v_e, k)  # (E,4)
    factor = -K1_Ve[:, None] * (proj.sum(axis=1, keepdims=True) + proj)
    return contrib + factor[:, :, None] * k[:, None, :]


def _magnetoelastic_contrib(p: Problem, v: np.ndarray, k1me, k1me_p=None) -> np.ndarray:
    """Per element-vertex magnetoelastic contribution (E,4,3), ``src/energy_kernels.py:212-224,319-329,
    411-426``: Kx_Ve = 2 (k1me + k1me_p) Ve / 20 and Ky_Ve = 2 (k1me - k1me_p) Ve / 20 per element (the
    per-element arrays zero-padded to E), g_a,x += Kx_Ve (sum_b v_b,x + v_a,x), likewise y."""
    E = p.conn.shape[0]
    kx = np.zeros(E)
    kx[: len(k1me)] = k1me
    kp = np.zeros(E)
    if k1me_p is not None:
        kp[: len(k1me_p)] = k1me_p
    Kx_Ve = 2.0 * (kx + kp) * p.volume / 20.0
    Ky_Ve = 2.0 * (kx - kp) * p.volume / 20.0
    v_e = v[p.conn]
    out = np.zeros_like(v_e)
    out[:, :, 0] = Kx_Ve[:, None] * (v_e[:, :, 0].sum(axis=1, keepdims=True) + v_e[:, :, 0])
    out[:, :, 1] = Ky_Ve[:, None] * (v_e[:, :, 1].sum(axis=1, keepdims=True) + v_e[:, :, 1])
    return out


def energy_and_grad_mf(p: Problem, m, U, B_ext, B_bias=None, k1me=None, k1me_p=None):
    """Matrix-free energy and gradient, ``src/energy_kernels.py:340-459``."""
    _, _, Js_Ve, _ = _coeffs(p)
    contrib = _exchange_aniso_contrib(p, m)
    if k1me is not None:
        contrib = contrib + _magnetoelastic_contrib(p, m, k1me, k1me_p)
    grad_u = np.einsum("ebi,eb->ei", p.grad_phi, U[p.conn])  # :403-407
    contrib = contrib + Js_Ve[:, None, None] * grad_u[:, None, :]
    g_quad = node_sum(p.conn, contrib, p.N)
    B_eff = np.asarray(B_ext, np.float64)[None, :] + (0.0 if B_bias is None else B_bias)
    g_z = -2.0 * p.M_nodal[:, None] * B_eff  # :438-445
    g_total = g_quad + g_z
    E = 0.5 * np.sum(m * (g_total + g_z))  # :457
    return E / p.V_mag, g_total / p.V_mag


def local_grad_only_mf(p: Problem, v, k1me=None, k1me_p=None):
    """Exchange + anisotropy (+ magnetoelastic) Hessian action, ``src/energy_kernels.py:272-338``."""
    c = _exchange_aniso_contrib(p, v)
    if k1me is not None:
        c = c + _magnetoelastic_contrib(p, v, k1me, k1me_p)
    return node_sum(p.conn, c, p.N) / p.V_mag


def exchange_diagonal(p: Problem) -> np.ndarray:
    """sum_e 2 A Ve |grad phi_a|^2 / V_mag, ``src/energy_kernels.py:492-566``."""
    A_Ve, _, _, _ = _coeffs(p)
    return node_sum(p.conn, A_Ve[:, None] * np.sum(p.grad_phi**2, axis=2), p.N) / p.V_mag


def apply_A_mf(p: Problem, U, reg=1e-12, mask=None):
    """Matrix-free Poisson operator, ``src/poisson_solve.py:210-252``."""
    grad_U = np.einsum("ebi,eb->ei", p.grad_phi, U[p.conn])
    contrib = p.volume[:, None] * np.einsum("eai,ei->ea", p.grad_phi, grad_U)
    y = node_sum(p.conn, contrib, p.N) + reg * U
    return y if mask is None else y * mask


def rhs_from_m_mf(p: Problem, m):
    """Matrix-free demag right-hand side, ``src/poisson_solve.py:254-280``."""
    Js = p.Js_lookup[p.mat_id - 1]
    msum = m[p.conn].sum(axis=1)  # (E,3)
    dot = 0.25 * np.einsum("eai,ei->ea", p.grad_phi, msum)
    return node_sum(p.conn, (p.volume * Js)[:, None] * dot, p.N)


# --------------------------------------------------------------------------------------------
# CPU assembly (src/amg_utils.py:21-111, :660-789; layouts src/loop.py:1133-1166)
# --------------------------------------------------------------------------------------------
def _pairs(conn):
    rows = np.repeat(conn, 4, axis=1).reshape(-1)
    cols = np.tile(conn, (1, 4)).reshape(-1)
    return rows, cols


def assemble_poisson(p: Problem, reg=1e-12, with_boundary=True) -> sp.csr_matrix:
    """Stiffness matrix with Dirichlet rows/cols replaced by identity, ``src/amg_utils.py:21-84``."""
    N = p.N
    Ke = p.volume[:, None, None] * np.einsum("eai,ebi->eab", p.grad_phi, p.grad_phi)
    rows, cols = _pairs(p.conn)
    A = sp.coo_matrix((Ke.reshape(-1), (rows, cols)), shape=(N, N)).tocsr()
    A.sum_duplicates()
    mask = p.boundary_mask if with_boundary else None
    if mask is not None:
        is_b = mask == 0
        row_idx = np.repeat(np.arange(N), np.diff(A.indptr))
        A.data[is_b[row_idx]] = 0.0
        A.data[is_b[A.indices]] = 0.0
        A.eliminate_zeros()
    A = (A + reg * sp.eye(N, format="csr")).tocsr()
    if mask is not None:
        d = A.diagonal()
        d[mask == 0] = 1.0
        A.setdiag(d)
    A.sort_indices()
    return A


def assemble_divergence(p: Problem):
    """Dx, Dy, Dz with (D_i)_ab = Js Ve/4 (grad phi_a)_i, ``src/amg_utils.py:660-702``."""
    N = p.N
    f = p.Js_lookup[p.mat_id - 1] * p.volume / 4.0
    rows, cols = _pairs(p.conn)
    out = []
    for i in range(3):
        De = f[:, None, None] * np.repeat(p.grad_phi[:, :, i][:, :, None], 4, axis=2)
        D = sp.coo_matrix((De.reshape(-1), (rows, cols)), shape=(N, N)).tocsr()
        D.sum_duplicates()
        out.append(D)
    return out


def assemble_K_eff(p: Problem) -> sp.csr_matrix:
    """3N x 3N interleaved exchange + anisotropy matrix, ``src/amg_utils.py:741-789``."""
    N = p.N
    g = p.mat_id - 1
    Kex = 2.0 * p.A_lookup[g][:, None, None] * p.volume[:, None, None] * np.einsum(
        "eai,ebi->eab", p.grad_phi, p.grad_phi)
    val = -2.0 * p.K1_lookup[g] * p.volume / 20.0
    Kan = val[:, None, None] * (np.ones((4, 4)) + np.eye(4))
    k = p.k_easy[g]
    kkT = np.einsum("eu,ev->euv", k, k)
    K_block = Kex[:, :, :, None, None] * np.eye(3)[None, None, None] + Kan[:, :, :, None, None] * kkT[:, None, None]
    rn, cn = _pairs(p.conn)
    r = 3 * rn[:, None, None] + np.arange(3)[None, :, None]
    c = 3 * cn[:, None, None] + np.arange(3)[None, None, :]
    r, c = np.broadcast_arrays(r, c)
    K = sp.coo_matrix((K_block.reshape(-1), (r.reshape(-1), c.reshape(-1))), shape=(3 * N, 3 * N)).tocsr()
    K.sum_duplicates()
    return K


def assembled_operators(p: Problem, reg=1e-12, parts=("A", "D", "G", "K_eff")):
    """A, D (blocked N x 3N), G (blocked 3N x N) and K_eff as ``src/loop.py:1089-1166,1199-1201`` builds them.

    ``parts`` limits the work to what a caller needs (the Poisson solve needs A and D only).
    """
    out = {}
    if "A" in parts:
        out["A"] = assemble_poisson(p, reg=reg, with_boundary=p.boundary_mask is not None)
    if "D" in parts or "G" in parts:
        Dx, Dy, Dz = assemble_divergence(p)
        D = sp.hstack([Dx, Dy, Dz]).tocsr()
        out["D"] = D
        if "G" in parts:
            N = p.N
            out["G"] = sp.vstack([2.0 * D[:, :N].T, 2.0 * D[:, N:2 * N].T, 2.0 * D[:, 2 * N:].T]).tocsr()
    if "K_eff" in parts:
        out["K_eff"] = assemble_K_eff(p)
    return out


def energy_and_grad_asm(p: Problem, ops, m, U, B_ext, B_bias=None):
    """Assembled energy and gradient, ``src/energy_kernels.py:147-180``."""
    N = p.N
    g_ex_an = (ops["K_eff"] @ m.reshape(-1)).reshape(N, 3)
    g_dem = (ops["G"] @ U).reshape(3, -1).T
    B_eff = np.asarray(B_ext, np.float64)[None, :] + (0.0 if B_bias is None else B_bias)
    g_z = -2.0 * p.M_nodal[:, None] * B_eff
    g_total = g_ex_an + g_dem + g_z
    E = 0.5 * np.sum(m * (g_total + g_z))
    return E / p.V_mag, g_total / p.V_mag


def local_grad_only_asm(p: Problem, ops, v):
    """``src/energy_kernels.py:190-195``."""
    return (ops["K_eff"] @ v.reshape(-1)).reshape(p.N, 3) / p.V_mag


def rhs_from_m_asm(ops, m, mask=None):
    """``src/poisson_solve.py:173-186`` (the blocked D layout)."""
    y = ops["D"] @ np.concatenate([m[:, 0], m[:, 1], m[:, 2]])
    return y if mask is None else y * mask


def apply_A_asm(ops, U, mask=None):
    """``src/poisson_solve.py:166-171``."""
    y = ops["A"] @ U
    return y if mask is None else y * mask


def spai0_diagonal(A: sp.csr_matrix) -> np.ndarray:
    """M_ii = a_ii / sum_j a_ij^2, ``src/amg_utils.py:87-111``."""
    A2 = sp.csr_matrix((A.data**2, A.indices, A.indptr), shape=A.shape)
    return A.diagonal() / (np.asarray(A2.sum(axis=1)).ravel() + 1e-30)


# --------------------------------------------------------------------------------------------
# Morton reorder (src/reorder_mesh.py:19-30, 85-117)
# --------------------------------------------------------------------------------------------
def morton_encode(q: np.ndarray) -> np.ndarray:
    """Interleave three 10-bit coordinates into a 30-bit key, ``src/reorder_mesh.py:19-30``."""
    x, y, z = (q[:, i].astype(np.int64) for i in range(3))
    code = np.zeros(q.shape[0], dtype=np.int64)
    for i in range(10):
        code |= ((x >> i) & 1) << (3 * i + 2)
        code |= ((y >> i) & 1) << (3 * i + 1)
        code |= ((z >> i) & 1) << (3 * i)
    return code


def morton_order(knt: np.ndarray, conn: np.ndarray):
    """(node_perm, elem_perm) of ``reorder_mesh(target="gpu")``, ``src/reorder_mesh.py:85-100``.

    The reference sorts with numpy's default (unstable) argsort; this restatement uses a stable
    sort, which gives the same permutation whenever the keys are distinct.
    """
    knt = np.asarray(knt, np.float64)
    lo, hi = knt.min(axis=0), knt.max(axis=0)
    den = np.where(hi - lo == 0, 1.0, hi - lo)
    node_perm = np.argsort(morton_encode(((knt - lo) / den * 1023).astype(np.int32)), kind="stable")
    cen = np.mean(knt[np.asarray(conn)[:, :4].astype(np.int64)], axis=1)
    elem_perm = np.argsort(morton_encode(((cen - lo) / den * 1023).astype(np.int32)), kind="stable")
    return node_perm, elem_perm
