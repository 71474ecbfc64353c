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
