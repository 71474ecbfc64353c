"""Shared construction of the same problem for the oracle and the product."""

from __future__ import annotations

import functools

import numpy as np

from mumag_matrixfree2_gb300 import fem_utils
from mumag_matrixfree2_gb300 import synthetic as syn
from oracle import fem as ofem

NDFEB = syn.Material(Js=1.61, A=7.7e-12, K1=4.3e6, axis=(0.0, 0.0, 1.0))


def materials(mats=None):
    mats = mats or [NDFEB, syn.AIR]
    return syn.reduced_materials(mats)


@functools.lru_cache(maxsize=None)
def case(name: str, with_boundary: bool = True, tilt_axis: bool = False):
    """(MeshSetup for the product, oracle Problem) for a named synthetic workload."""
    w = syn.WORKLOADS[name]
    knt, ijk = syn.box_mesh(w)
    mats = None
    if tilt_axis:
        mats = [syn.Material(axis=(np.sin(0.3), 0.0, np.cos(0.3))), syn.AIR]
    A, K1, Js, k, Js_ref = materials(mats)
    s = fem_utils.prepare(knt, ijk, A, K1, Js, k, with_boundary=with_boundary)
    p = ofem.make_problem(knt, ijk, A, K1, Js, k, with_boundary=with_boundary)
    return s, p, Js_ref


def random_state(N, seed=0, amplitude=0.3):
    rng = np.random.default_rng(seed)
    m = np.array([0.0, 0.0, 1.0]) + amplitude * rng.standard_normal((N, 3))
    return m / np.linalg.norm(m, axis=1, keepdims=True)


# ------------------------------------------------------------------------------------------------
# inputs of the fixtures made from the reference's C++ minimizer (tests/golden/make_ref_golden.py)
# ------------------------------------------------------------------------------------------------
REF_CASES = {"cube8_h2_air24": 1, "cube40_h2_air200": 37}  # workload -> node sampling stride
REF_FIELDS_T = (8.0, 2.0, -3.0)  # field steps (Tesla) of the short minimizer sequences
REF_B = (0.01, -0.02, -0.3)  # reduced external field of the energy / inner-solve fixtures


def ref_state(name: str):
    """(m, U, B): a seeded magnetisation, a smooth potential that vanishes on the Dirichlet faces and a
    field, all deterministic, so both sides of a fixture comparison start from the same input."""
    s, p, _ = case(name)
    m = random_state(p.N, seed=11, amplitude=0.3)
    x, y, z = p.knt[:, 0], p.knt[:, 1], p.knt[:, 2]
    U = 0.1 * np.sin(x / 7.0) * np.cos(y / 5.0) + 0.02 * z / np.abs(z).max()
    if p.boundary_mask is not None:
        U = U * p.boundary_mask
    return m, U, np.array(REF_B)


def ref_sample(N: int, stride: int) -> np.ndarray:
    """Node indices stored by a fixture (every ``stride``-th node, the last node included)."""
    idx = np.arange(0, N, stride)
    return idx if idx[-1] == N - 1 else np.append(idx, N - 1)


def ref_min_params():
    """Minimizer parameters of the fixtures: the loop settings of the workloads (tau_f 1e-8, eps_a 1e-6,
    10 inner iterations) with the demag solves at 1e-12, the accuracy of the reference's direct solve."""
    from oracle import minimize as omin

    return omin.Params(tau_f=1e-8, eps_a=1e-6, pc_iters=10, cg_tol=1e-12)
