"""GB300-native ``cuda`` backend for the micromagnetic hot path of MaMMoS-project/mumag_matrixfree2.

The package mirrors the reference's factory API (``make_energy_kernels``, ``make_solve_U``,
``make_minimizer``, ``run_hysteresis_loop``) and runs every hot operation in hand-written sm_103a
CUDA kernels behind the C-ABI library ``libmumag_cuda.so`` (declared in ``include/mumag_cuda.h``).
"""
