"""Learned warm start, CPU side: the oracle network against finite differences and torch's bf16,
and the host layout helpers."""

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import learned
from oracle import unet as ou


def test_layer_tables_agree():
    assert [l[:5] for l in learned.LAYERS] == [l[:5] for l in ou.LAYERS]
    p = learned.init_params(3)
    q = ou.init_params(3)
    for k in p:
        assert np.array_equal(p[k], q[k])


def test_flatten_roundtrip():
    p = learned.init_params(1)
    flat = learned.flatten(p)
    assert flat.size == sum(27 * ci * co + co for _, _, ci, co, _ in learned.LAYERS)
    q = learned.unflatten(flat)
    assert all(np.array_equal(p[k], q[k]) for k in p)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 10.0 ** np.random.default_rng(1).integers(-8, 8, 10000)
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(ou.bf16(x), ref)


def test_oracle_gradients_match_finite_differences(monkeypatch):
    """Backward of the unrounded (float64) oracle against central differences of its loss."""
    monkeypatch.setattr(ou, "ROUND", False)
    G = 16
    rng = np.random.default_rng(5)
    p = {k: v.astype(np.float64) for k, v in ou.init_params(2).items()}
    for k in p:
        if k.endswith(".b"):
            p[k] = 0.05 * rng.standard_normal(p[k].shape)
    x = rng.standard_normal((G, G, G, 4))
    t = rng.standard_normal((G, G, G))

    def loss(pp):
        return ou.loss_and_seed(ou.forward(pp, x), t)[0]

    tape = ou.Tape()
    y = ou.forward(p, x, tape)
    _, seed = ou.loss_and_seed(y, t)
    g = ou.backward(p, tape, seed)
    checked = 0
    for name in ("e0a.w", "e1b.w", "b3b.w", "d2a.b", "d0b.w", "d0b.b"):
        flat = p[name].reshape(-1)
        nz = np.flatnonzero(np.abs(g[name].reshape(-1)) > 1e-6)
        idx = rng.choice(nz, size=min(3, nz.size), replace=False)
        for i in idx:
            h = 1e-5 * max(1.0, abs(flat[i]))
            pp = {k: v.copy() for k, v in p.items()}
            pp[name].reshape(-1)[i] += h
            lp = loss(pp)
            pp[name].reshape(-1)[i] -= 2 * h
            lm = loss(pp)
            fd = (lp - lm) / (2 * h)
            an = g[name].reshape(-1)[i]
            assert abs(fd - an) <= 1e-4 * abs(an) + 1e-9, (name, i, fd, an)
            checked += 1
    assert checked == 16  # d0b.b has one non-zero gradient (only output channel 0 enters the loss)
