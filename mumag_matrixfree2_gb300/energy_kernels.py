"""``make_energy_kernels`` with the reference's signature (``src/energy_kernels.py:82-142``), on the GPU.

Both reference modes compute the same operators; here both run the assembled per-row operator of
libmumag_cuda (``k_energy_grad``, ``k_local_grad``), including the per-element magnetoelastic terms
``k1me``/``k1me_p`` when given (``mm_set_magnetoelastic``).
"""

from __future__ import annotations

import numpy as np

from .cuda_backend import problem_for_geom


def make_energy_kernels(geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, V_mag, M_nodal, *, B_bias=None,
                        k1me=None, k1me_p=None, chunk_elems: int = 200_000, assembly: str = "segment_sum",
                        grad_backend: str = "stored_grad_phi", mode: str = "matrix_free", Kex_sparse=None,
                        Gx_sparse=None, Gy_sparse=None, Gz_sparse=None, Kan_sparse=None, k_nodes=None,
                        boundary_mask=None):
    """Return (energy_and_grad, energy_only, grad_only, local_grad_only) running on the GPU.

    energy_and_grad(m, U, B_ext, sparse_ops=None) -> (E, g): E = 1/2 m.(g + g_z) / V_mag and
    g = (K m + G U + g_z) / V_mag with g_z = -2 M_nodal (B_ext + B_bias) (``:147-180,340-459``).
    m, U may be numpy arrays or CUDA torch tensors (then g is a CUDA tensor).
    """
    prob = problem_for_geom(geom, A_lookup, K1_lookup, Js_lookup, k_easy_lookup, V_mag, M_nodal, boundary_mask,
                            k1me=k1me, k1me_p=k1me_p)
    bias0 = None if B_bias is None else np.asarray(B_bias, np.float64)

    def energy_and_grad(m, U, B_ext, sparse_ops=None):
        bias = bias0
        if sparse_ops is not None and sparse_ops.get("B_bias") is not None:
            bias = np.asarray(sparse_ops["B_bias"], np.float64)
        if bias is not None and np.ndim(bias) == 1:
            bias = np.broadcast_to(bias, (prob.N, 3))
        if bias is not None and type(m).__module__.startswith("torch"):
            import torch

            bias = torch.as_tensor(np.ascontiguousarray(bias), device=m.device)
        return prob.energy_and_grad(m, U, B_ext, bias)

    def energy_only(m, U, B_ext, sparse_ops=None):
        return energy_and_grad(m, U, B_ext, sparse_ops)[0]

    def grad_only(m, U, B_ext, sparse_ops=None):
        return energy_and_grad(m, U, B_ext, sparse_ops)[1]

    def local_grad_only(v, sparse_ops=None):
        return prob.local_grad(v)

    energy_and_grad.problem = prob
    return energy_and_grad, energy_only, grad_only, local_grad_only


def compute_exchange_diagonal(geom, A_lookup, V_mag, *, chunk_elems: int = 200_000, assembly: str = "segment_sum",
                              grad_backend: str = "stored_grad_phi"):
    """sum_e 2 A Ve |grad phi_a|^2 / V_mag per node (``src/energy_kernels.py:492-566``)."""
    A = np.asarray(A_lookup, np.float64).ravel()
    G = len(A)
    prob = problem_for_geom(geom, A, np.zeros(G), np.zeros(G), np.tile([0.0, 0.0, 1.0], (G, 1)), V_mag,
                            np.zeros(int(np.asarray(geom.conn).max()) + 1))
    return prob.exchange_diagonal()
