"""The allocation-free energy entry point, for callers that cannot allocate device memory at call
time (an application whose device memory all comes from a fixed pool reserved at start-up, with no
allocation allowed while it runs).  Its reduction scratch lives in a static device array instead of
the problem's workspace; its results must equal those of the allocating entry point.  This file is
collected last on purpose."""

import ctypes as C

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import _abi, fem_utils

from .helpers import case, random_state

pytestmark = pytest.mark.gpu

RTOL = 1e-10  # same FP64 bar as the other energy parity tests


def test_noalloc_energy_matches_the_allocating_entry_point(cuda_ok):
    import torch

    s, p, _ = case("cube16_h2_air48")
    prob = fem_utils.make_problem(s)
    rng = np.random.default_rng(21)
    m = torch.from_numpy(random_state(p.N, seed=21)).cuda()
    U = torch.from_numpy(rng.standard_normal(p.N)).cuda()
    bias = torch.from_numpy(0.01 * rng.standard_normal((p.N, 3))).cuda()
    B = np.array([0.05, -0.1, 0.2])
    lib = _abi.lib()
    for b in (None, bias):
        E_ref, g_ref = prob.energy_and_grad(m, U, B, b)
        g_ref = g_ref.cpu().numpy()
        for _call in range(2):  # the shared scratch must give the same answer call after call
            g = torch.full_like(m, float("nan"))
            E = C.c_double()
            rc = lib.mm_energy_grad_noalloc(prob.h, C.c_void_p(m.data_ptr()), C.c_void_p(U.data_ptr()),
                                            _abi.dptr(B), None if b is None else C.c_void_p(b.data_ptr()),
                                            C.byref(E), C.c_void_p(g.data_ptr()))
            assert rc == 0, lib.mm_last_error(prob.h)
            assert abs(E.value - E_ref) <= RTOL * abs(E_ref)
            gn = g.cpu().numpy()
            assert np.max(np.abs(gn - g_ref)) <= RTOL * np.max(np.abs(g_ref))


def test_noalloc_rejects_missing_arguments(cuda_ok):
    s, p, _ = case("cube8_h2_air24")
    prob = fem_utils.make_problem(s)
    lib = _abi.lib()
    E = C.c_double()
    assert lib.mm_energy_grad_noalloc(prob.h, None, None, None, None, C.byref(E), None) == -1
