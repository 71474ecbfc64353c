"""Mesh containers and host setup, mirroring ``src/fem_utils.py`` and ``src/loop.py:845-939``.

Geometry, the Dirichlet mask and the Morton order are computed by the C++ setup in
libmumag_cuda (``mm_geom_compute``, ``mm_boundary_mask``, ``mm_morton_order``).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _abi


@dataclass
class TetGeom:
    """Same fields as the reference's container (``src/fem_utils.py:22-40``), as numpy arrays."""

    conn: np.ndarray
    volume: np.ndarray
    mat_id: np.ndarray
    grad_phi: np.ndarray | None = None
    JinvT: np.ndarray | None = None
    x_nodes: np.ndarray | None = None


def compute_node_volumes(geom: TetGeom, n_nodes: int | None = None) -> np.ndarray:
    """Lumped nodal volume sum_e Ve/4 (``src/fem_utils.py:174-212``), summed in element order."""
    conn = np.asarray(geom.conn)
    n = int(n_nodes if n_nodes is not None else (geom.x_nodes.shape[0] if geom.x_nodes is not None else conn.max() + 1))
    w = np.repeat(0.25 * np.asarray(geom.volume, np.float64), 4)
    return np.bincount(conn.reshape(-1), weights=w, minlength=n)


@dataclass
class MeshSetup:
    """Everything a problem needs, in reduced units (``src/loop.py:856-939``)."""

    knt: np.ndarray
    geom: TetGeom
    A_lookup: np.ndarray
    K1_lookup: np.ndarray
    Js_lookup: np.ndarray
    k_easy: np.ndarray
    V_mag: float
    M_nodal: np.ndarray
    node_volumes: np.ndarray
    boundary_mask: np.ndarray | None

    @property
    def N(self) -> int:
        return self.knt.shape[0]


def prepare(knt, ijk, A_lookup, K1_lookup, Js_lookup, k_easy, with_boundary: bool = True,
            reorder: bool | str = False) -> MeshSetup:
    """Orient the mesh, compute volumes/gradients, V_mag, M_nodal and the Dirichlet mask.

    With ``reorder`` ("gpu" or True: Morton order, ``src/reorder_mesh.py:85-117``; "cpu": reverse
    Cuthill-McKee, ``:53-83``) the nodes and elements are first renumbered.
    """
    knt = np.ascontiguousarray(knt, dtype=np.float64)
    ijk = np.asarray(ijk)
    mat_id = ijk[:, 4].astype(np.int32) if ijk.shape[1] > 4 else np.ones(ijk.shape[0], np.int32)
    if mat_id.min() == 0:
        mat_id = mat_id + 1
    conn = ijk[:, :4].astype(np.int32)
    if reorder:
        if reorder == "cpu":
            node_perm, elem_perm = _abi.rcm_order(conn, knt.shape[0])
        else:
            node_perm, elem_perm = _abi.morton_order(knt, conn)
        inv = np.empty_like(node_perm)
        inv[node_perm] = np.arange(len(node_perm), dtype=np.int32)
        knt = knt[node_perm]
        conn = inv[conn[elem_perm]]
        mat_id = mat_id[elem_perm]
    conn, volume, JinvT, grad_phi = _abi.geom_compute(knt, conn)
    Js_lookup = np.asarray(Js_lookup, np.float64)
    is_mag = np.isin(mat_id, np.where(Js_lookup > 0)[0] + 1)
    V_mag = float(np.sum(volume[is_mag])) or 1.0
    geom = TetGeom(conn=conn, volume=volume, mat_id=mat_id, grad_phi=grad_phi, JinvT=JinvT, x_nodes=knt)
    N = knt.shape[0]
    node_vols = compute_node_volumes(geom, N)
    M_nodal = compute_node_volumes(TetGeom(conn=conn, volume=volume * Js_lookup[mat_id - 1], mat_id=mat_id), N)
    mask = _abi.boundary_mask(conn, N) if with_boundary else None
    return MeshSetup(knt=knt, geom=geom, A_lookup=np.asarray(A_lookup, np.float64),
                     K1_lookup=np.asarray(K1_lookup, np.float64), Js_lookup=Js_lookup,
                     k_easy=np.asarray(k_easy, np.float64), V_mag=V_mag, M_nodal=M_nodal,
                     node_volumes=node_vols, boundary_mask=mask)


def make_problem(s: MeshSetup):
    """Upload a prepared mesh to the GPU."""
    from .cuda_backend import Problem

    return Problem(s.geom.conn, s.geom.volume, s.geom.grad_phi, s.geom.mat_id, s.A_lookup, s.K1_lookup, s.Js_lookup,
                   s.k_easy, s.V_mag, s.M_nodal, s.boundary_mask, n_nodes=s.N)
