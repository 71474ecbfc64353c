"""CPU oracle: an FP64 numpy/scipy restatement of the reference's hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this directory; only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use
it, and only as the checker or the timed CPU baseline, never as the thing measured for the GPU.

Every function cites the file:line of the reference (MaMMoS-project/mumag_matrixfree2) it follows.
The reference's own hot path cannot run here (JAX, PyAMG and Intel MKL are absent), so the
restatement is pinned instead by

* the reference's golden mesh ``tests/single_solid.npz`` and outputs of its importable modules
  (``src/mesh.py``, ``src/reorder_mesh.py``) committed under ``tests/golden/``;
* the analytic energies of ``tests/test_energy.py`` and the finite-difference gradients of
  ``tests/test_gradients.py``;
* agreement between the assembled and matrix-free formulations, as ``tests/test_compare_kernels.py``
  checks the reference's two implementations against each other.

The smoothed-aggregation hierarchy is this project's own (PyAMG is not available and no reference
test pins its hierarchy): parity for aggregation and prolongation is unpinned against the reference
and bit-exact against this oracle only.
"""
