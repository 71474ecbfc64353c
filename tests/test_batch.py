"""Batched particles: the ellipsoid meshes (CPU) and concurrent sweeps on one GPU (GPU)."""

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import fem_utils
from mumag_matrixfree2_gb300 import synthetic as syn


def test_ellipsoid_mesh_is_valid_and_graded():
    p = syn.Particle(6.0, 9.0, 12.5, syn.Material())
    knt, ijk = syn.ellipsoid_mesh(p)
    A, K1, Js, k, _ = syn.reduced_materials([p.material, syn.AIR])
    s = fem_utils.prepare(knt, ijk, A, K1, Js, k)
    assert np.all(s.geom.volume > 0)
    box = 5.0 * 12.5
    assert np.allclose(knt.min(0), -box / 2) and np.allclose(knt.max(0), box / 2)
    mag = ijk[:, 4] == 1
    V_mag = s.geom.volume[mag].sum()
    V_ell = 4.0 / 3.0 * np.pi * 6.0 * 9.0 * 12.5
    assert abs(V_mag - V_ell) < 0.15 * V_ell  # voxelised at 1.5 nm
    assert s.boundary_mask is not None and (s.boundary_mask == 0).sum() > 0


def test_random_particles_follow_the_stated_distributions():
    ps = syn.random_particles(256, seed=0)
    ax = np.array([[p.a, p.b, p.c] for p in ps])
    assert ax.min() >= 5.0 and ax.max() <= 25.0
    k = np.array([p.material.axis for p in ps])
    assert np.allclose(np.linalg.norm(k, axis=1), 1.0) and abs(k.mean(0)).max() < 0.15
    assert all(1e6 <= p.material.K1 <= 5e6 and 1.0 <= p.material.Js <= 1.6 for p in ps)


@pytest.mark.gpu
def test_concurrent_sweeps_equal_sequential_sweeps(cuda_ok):
    """Four particles swept by four host threads (four problems, four streams) give exactly the
    results of one thread sweeping them in turn: the problems share no device state."""
    from mumag_matrixfree2_gb300 import batch

    ps = syn.random_particles(4, seed=3, semi=(5.0, 7.0))
    B = np.linspace(3.0, -3.0, 13)
    one = batch.run_batch(ps, B, workers=1)
    four = batch.run_batch(ps, B, workers=4)
    for r1, r4 in zip(one["results"], four["results"]):
        assert r1.nodes == r4.nodes and r1.pcg_iters == r4.pcg_iters
        assert np.array_equal(np.asarray(r1.J), np.asarray(r4.J))
    assert one["particles"] == 4 and four["step_latency_ms"]["p99"] > 0
