"""Learned warm start on the GPU (tcgen05 convolutions, mma.sync weight gradients, Adam) against the
CPU oracle network.  Both round to bf16 at the same points; the GPU accumulates in FP32, the oracle
in FP64, so values agree to a few bf16 ulps (tolerances stated per check)."""

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import learned
from oracle import unet as ou

pytestmark = pytest.mark.gpu

G, NB = 16, 2
ORACLE_NAME = {"x": ("e0a", 0), "e0a": ("e0a", 1), "s0": ("e0b", 1), "p0": ("e1a", 0), "e1a": ("e1a", 1),
               "s1": ("e1b", 1), "p1": ("e2a", 0), "e2a": ("e2a", 1), "s2": ("e2b", 1), "p2": ("b3a", 0),
               "b3a": ("b3a", 1), "b3b": ("b3b", 1), "b3c": ("b3c", 1), "h2": ("d2a", 0), "d2a": ("d2a", 1),
               "d2b": ("d2b", 1), "h1": ("d1a", 0), "d1a": ("d1a", 1), "d1b": ("d1b", 1), "h0": ("d0a", 0),
               "d0a": ("d0a", 1), "out": ("d0b", 1)}


# Relative L2 tolerance of each parameter gradient: 3x the spread between two oracle runs on this
# case that differ only in accumulating the convolutions in FP32 instead of FP64 (bf16-rounded
# gradients passed through ReLU masks; largest on the few-voxel bottleneck level), at least 1 %.
SPREAD = {"d0b": 1e-4, "d0a": 1e-3, "d1b": 1.5e-3, "d1a": 2.7e-3, "d2b": 1.16e-2, "d2a": 1.59e-2, "b3c": 5.05e-2,
          "b3b": 5.61e-2, "b3a": 5.3e-2, "e2b": 2.19e-2, "e2a": 2.36e-2, "e1b": 3.3e-3, "e1a": 3.4e-3,
          "e0b": 1.7e-3, "e0a": 9.4e-3}


def _params(seed):
    rng = np.random.default_rng(seed)
    p = learned.init_params(seed)
    for k in p:
        if k.endswith(".b"):
            p[k] = (0.05 * rng.standard_normal(p[k].shape)).astype(np.float32)
    return p


@pytest.fixture(scope="module")
def case(cuda_ok):
    rng = np.random.default_rng(11)
    p = _params(7)
    x = rng.standard_normal((NB, G, G, G, 4)).astype(np.float32)
    t = rng.standard_normal((NB, G, G, G)).astype(np.float32)
    net = learned.UNet(G, NB, p)
    y = net.forward(x)
    tapes, refs = [], []
    for b in range(NB):
        tape = ou.Tape()
        refs.append(ou.forward(p, x[b], tape))
        tapes.append(tape)
    return net, p, x, t, y, tapes, refs


def test_forward_matches_oracle_layer_by_layer(case):
    net, p, x, t, y, tapes, refs = case
    for b in range(NB):
        for name in learned.TENSORS:
            lay, k = ORACLE_NAME[name]
            ref = tapes[b].acts[lay][k]
            got = net.read(name, b)
            scale = float(np.abs(ref).max()) or 1.0
            err = np.abs(got - ref)
            assert err.max() <= 3e-2 * scale and err.mean() <= 3e-3 * scale, (b, name, err.max() / scale)
        assert np.abs(y[b] - refs[b][..., 0]).max() <= 3e-2 * np.abs(refs[b][..., 0]).max()


def test_gradients_and_loss_match_oracle(case):
    net, p, x, t, y, tapes, refs = case
    loss = net.backward(t)
    n = NB * G ** 3
    gref, lref = None, 0.0
    for b in range(NB):
        r = refs[b][..., 0].astype(np.float64) - t[b]
        lref += float((r * r).sum()) / n
        seed = np.zeros_like(refs[b])
        seed[..., 0] = (2.0 / n) * r
        g = ou.backward(p, tapes[b], ou.bf16(seed))
        gref = g if gref is None else {k: gref[k] + g[k] for k in g}
    assert abs(loss - lref) <= 1e-2 * lref
    gg = net.get_grads()
    for k in gref:
        a, r = gg[k].astype(np.float64).ravel(), gref[k].astype(np.float64).ravel()
        nr = np.linalg.norm(r)
        if nr == 0.0:
            assert np.abs(a).max() == 0.0, k
            continue
        tol = max(1e-2, 3.0 * SPREAD[k.split(".")[0]])
        assert np.linalg.norm(a - r) <= tol * nr, (k, np.linalg.norm(a - r) / nr)
        assert a @ r >= 0.995 * np.linalg.norm(a) * nr, k  # same direction
    assert np.abs(gg["e0a.w"][:, 4:, :]).max() == 0.0  # padded input channels never learn


def test_adam_matches_oracle_update(case):
    net, p, x, t, y, tapes, refs = case
    net.forward(x)
    net.backward(t)
    g = net.get_grads()
    p0 = net.get_params()
    net.adam(1e-3)
    p1 = net.get_params()
    ref = ou.adam_step({k: v.copy() for k, v in p0.items()}, g, {"t": 0, "m": {}, "v": {}}, lr=1e-3)
    for k in p1:
        assert np.allclose(p1[k], ref[k], rtol=1e-5, atol=1e-7), k
    net.set_params(p)  # restore for the other tests


def test_training_reduces_the_loss(cuda_ok):
    rng = np.random.default_rng(3)
    net = learned.UNet(G, NB, _params(5))
    x = rng.standard_normal((NB, G, G, G, 4)).astype(np.float32)
    # a smooth target the network can fit: a blurred linear map of the input
    t = (0.5 * x[..., 0] - 0.25 * x[..., 3]).astype(np.float32)
    losses = []
    for _ in range(30):
        net.forward(x)
        losses.append(net.backward(t))
        net.adam(2e-3)
    assert losses[-1] < 0.75 * losses[0], losses[::5]


# ------------------------------------------------------------------------------------------------
# the warm start on a mesh: data from the plain solver's sweeps, training, and what it gains
# ------------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def sweeps(cuda_ok):
    import torch

    from mumag_matrixfree2_gb300 import fem_utils
    from mumag_matrixfree2_gb300 import synthetic as syn
    from mumag_matrixfree2_gb300.cuda_backend import MinimizerParams

    from .helpers import case

    s, _, Js_ref = case("cube40_h2_air200")
    prob = fem_utils.make_problem(s)
    prob.build_poisson(1e-12, "amgcl")
    ws = learned.WarmStart(s, grid=32, margin=10.0, batch=8, seed=1)
    prm = MinimizerParams(tau_f=1e-8, eps_a=1e-6, cg_tol=1e-10, pc_iters=10)
    B = syn.field_values(8.0 / Js_ref, -8.0 / Js_ref, 0.2 / Js_ref)
    train, pairs = [], []
    for tilt, seed in ((10.0, 1), (30.0, 2), (45.0, 3)):
        st, _, _ = learned.collect_sweep(prob, ws, syn.initial_state(s.N, seed=seed),
                                         syn.tilted_field_direction(tilt), B, prm)
        base = len(train)
        train += st
        pairs += [(base + i, base + i + d) for d in (1, 2) for i in range(len(st) - d)]
    ev, nodal, _ = learned.collect_sweep(prob, ws, syn.initial_state(s.N, seed=0),
                                         syn.tilted_field_direction(1.0), B, prm, keep_nodal=True)
    ws.calibrate(train, pairs)
    torch.cuda.synchronize()
    return prob, ws, train, pairs, ev, nodal


def test_device_transfer_matches_host_transfer(sweeps):
    """mm_unet_voxelise_dev / forward / mm_unet_interp_add_dev (the in-solve path, no normalisation:
    the bias-free network is homogeneous) against the torch gathers and a normalised forward."""
    import torch

    prob, ws, train, pairs, ev, nodal = sweeps
    (ma, Ua), (mb, Ub) = nodal[10], nodal[11]
    U_dev = Ua.clone()
    ws.apply(mb, ma, U_dev)
    fa = ws.fields(ma, Ua)
    mv = ws._vox(mb) * ws.jsf[:, None]
    fb = torch.cat([mv.float(), fa[:, 3:]], 1)
    pred, _ = ws.predict_grid(fa, fb)
    corr = torch.zeros_like(Ua)
    corr[ws.k_nodes.long()] = (pred.double()[ws.k_idx8.long()] * ws.k_w8.double()).sum(1)
    ref = Ua + corr
    d = (U_dev - ref).abs().max().item()
    scale = corr.abs().max().item()
    assert scale > 0 and d <= 2e-2 * scale, (d, scale)  # bf16 activations, different input scaling


def test_trained_warm_start_saves_pcg_iterations(sweeps):
    """Trained on the plain solver's own sweeps, the network's prediction of U_b - U_a on a held-out
    sweep beats U_a alone: median grid error at least 30 % below the untrained network's, the initial
    guess's energy-norm error over the sweep at least 5 % below the previous potential's (the scaled
    prediction cannot increase it step by step), and PCG to the same tolerance needs no more
    iterations from it (with 15-iteration solves the saving can round to zero on this small mesh)."""
    prob, ws, train, pairs, ev, nodal = sweeps
    ev_pairs = [(i, i + 1) for i in range(len(ev) - 1)]
    err0 = np.median([ws.predict_grid(ev[a], ev[b])[1] for a, b in ev_pairs])
    ws.train(train, pairs, steps=1500, lr=1e-3)
    err1 = np.median([ws.predict_grid(ev[a], ev[b])[1] for a, b in ev_pairs])
    assert err1 < 0.7 * err0 and err1 < 1.0, (err0, err1)
    base = learn = 0
    ea0 = ea1 = 0.0

    def a_err(U_star, x):
        e = (U_star - x).cpu().numpy()
        return float(e @ prob.apply_A(e))

    for k in range(len(nodal) - 1):
        (ma, Ua), (mb, Ub) = nodal[k], nodal[k + 1]
        x = Ua.clone()
        ea0 += a_err(Ub, x)
        _, it0, rr0, rc0 = prob.solve_u(mb, x, 1e-10)
        x = Ua.clone()
        ws.apply(mb, ma, x, prob)
        ea1 += a_err(Ub, x)
        _, it1, rr1, rc1 = prob.solve_u(mb, x, 1e-10)
        assert rc0 == 0 and rc1 == 0 and rr1 <= 1e-10
        base += it0
        learn += it1
    assert ea1 < 0.95 * ea0, (ea0, ea1)
    assert learn <= base, (learn, base)


def test_no_wait_apply_equals_waiting_apply(sweeps):
    """The queued chain (network stream after the caller's stream, scaled correction on the problem's
    stream after the network's, alpha on the device) gives the waiting path's corrected U and the same
    PCG iterations; the correction's alpha is the one the waiting path returns."""
    prob, ws, train, pairs, ev, nodal = sweeps
    for k in (3, 9):
        (ma, Ua), (mb, _) = nodal[k], nodal[k + 1]
        x1 = Ua.clone()
        a1 = ws.apply(mb, ma, x1, prob)
        x2 = Ua.clone()
        assert ws.apply(mb, ma, x2, prob, wait=False) is None
        prob.sync()  # before torch reads x2
        ws.net.sync()
        d = (x1 - x2).abs().max().item()
        assert d <= 1e-12 * max(1.0, x1.abs().max().item()), d
        # the solve queued right behind the correction on the problem's stream
        x3 = Ua.clone()
        ws.apply(mb, ma, x3, prob, wait=False)
        _, it3, rr3, rc3 = prob.solve_u(mb, x3, 1e-10)
        _, it1, rr1, rc1 = prob.solve_u(mb, x1, 1e-10)
        assert rc1 == rc3 == 0 and it1 == it3 and rr3 <= 1e-10
        assert a1 > 0
