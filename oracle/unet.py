"""CPU oracle of the learned demag warm start (test infrastructure only: never called by the product).

The network is this project's own (the reference has no learned component): a 3D U-Net over a
G^3 voxel grid that maps the voxelised change of magnetisation (3 channels) and the voxelised
previous potential (1 channel) to the change of the demag potential (channel 0 of the output).
Every convolution is 3x3x3, stride 1, zero padding 1, with bias; hidden convolutions use ReLU.
Levels are joined by 2x2x2 average pooling and nearest-neighbour upsampling; skips are added.

Rounding points follow the GPU kernels exactly: activations, activation gradients and the
convolution weights are bfloat16 (round to nearest even); products are accumulated in float32
(here float64, a stricter reference); biases, weight gradients and the Adam state are float32.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# (name, level, c_in, c_out, relu)
LAYERS = [
    ("e0a", 0, 16, 16, True), ("e0b", 0, 16, 16, True),
    ("e1a", 1, 16, 32, True), ("e1b", 1, 32, 32, True),
    ("e2a", 2, 32, 64, True), ("e2b", 2, 64, 64, True),
    ("b3a", 3, 64, 128, True), ("b3b", 3, 128, 128, True), ("b3c", 3, 128, 64, True),
    ("d2a", 2, 64, 64, True), ("d2b", 2, 64, 32, True),
    ("d1a", 1, 32, 32, True), ("d1b", 1, 32, 16, True),
    ("d0a", 0, 16, 16, True), ("d0b", 0, 16, 16, False),
]
IN_CHANNELS = 4  # dm_x, dm_y, dm_z, U_prev (zero-padded to 16)


ROUND = True  # bf16 rounding at the GPU's storage points; False: plain float64 (finite differences)


def _st(x) -> np.ndarray:
    """A stored tensor: bf16-rounded like the GPU's, or float64 when ROUND is off."""
    return bf16(x) if ROUND else np.asarray(x, np.float64)


def _ft():
    return np.float32 if ROUND else np.float64


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def init_params(seed: int = 0) -> dict[str, np.ndarray]:
    """He-uniform weights [27, c_in, c_out] (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) and zero biases."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, _, ci, co, _ in LAYERS:
        fan_in = 27 * (IN_CHANNELS if name == "e0a" else ci)
        lim = np.sqrt(6.0 / fan_in)
        w = rng.uniform(-lim, lim, size=(27, ci, co)).astype(np.float32)
        if name == "e0a":
            w[:, IN_CHANNELS:, :] = 0.0
        if name == "d0b":
            w *= 0.1
        p[name + ".w"] = w
        p[name + ".b"] = np.zeros(co, np.float32)
    return p


def _pad(x):
    return np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))


def conv3d(x: np.ndarray, w: np.ndarray, b: np.ndarray | None) -> np.ndarray:
    """Same-size 3x3x3 convolution of x [G,G,G,ci] with w [27,ci,co] (float64 accumulation)."""
    G = x.shape[0]
    xp = _pad(x.astype(np.float64))
    out = np.zeros(x.shape[:3] + (w.shape[2],), np.float64)
    t = 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sl = xp[1 + dz:1 + dz + G, 1 + dy:1 + dy + G, 1 + dx:1 + dx + G, :]
                out += sl @ w[t].astype(np.float64)
                t += 1
    if b is not None:
        out += b.astype(np.float64)
    return out


def conv3d_wgrad(x: np.ndarray, dpre: np.ndarray) -> np.ndarray:
    """dW[t, ci, co] = sum_v x[v + s_t, ci] dpre[v, co] (float64)."""
    G = x.shape[0]
    xp = _pad(x.astype(np.float64))
    d = dpre.astype(np.float64).reshape(-1, dpre.shape[3])
    out = np.zeros((27, x.shape[3], dpre.shape[3]), np.float64)
    t = 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sl = xp[1 + dz:1 + dz + G, 1 + dy:1 + dy + G, 1 + dx:1 + dx + G, :].reshape(-1, x.shape[3])
                out[t] = sl.T @ d
                t += 1
    return out


def conv3d_dgrad(dpre: np.ndarray, w: np.ndarray) -> np.ndarray:
    """dX = conv3d(dpre, W') with W'[t] = W[26 - t]^T (the adjoint of a same-size convolution)."""
    wt = np.ascontiguousarray(np.transpose(w[::-1], (0, 2, 1)))
    return conv3d(dpre, wt, None)


def pool(x):
    G = x.shape[0] // 2
    return _st(x.reshape(G, 2, G, 2, G, 2, -1).astype(_ft()).mean(axis=(1, 3, 5), dtype=_ft()))


def pool_bwd(d):
    return _st(np.repeat(np.repeat(np.repeat(d / 8.0, 2, 0), 2, 1), 2, 2))


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_bwd(d):
    G = d.shape[0] // 2
    return d.reshape(G, 2, G, 2, G, 2, -1).astype(_ft()).sum(axis=(1, 3, 5), dtype=_ft())


@dataclass
class Tape:
    acts: dict = field(default_factory=dict)


def _conv_layer(p, name, x, relu, tape):
    w = _st(p[name + ".w"])
    y = conv3d(x, w, p[name + ".b"])
    if relu:
        y = np.maximum(y, 0.0)
    y = _st(y.astype(_ft()))
    tape.acts[name] = (x, y, relu)
    return y


def forward(p: dict, x_in: np.ndarray, tape: Tape | None = None) -> np.ndarray:
    """x_in [G,G,G,4] float32 -> output [G,G,G,16] (bf16 values; channel 0 is the prediction)."""
    tape = tape if tape is not None else Tape()
    G = x_in.shape[0]
    x = np.zeros((G, G, G, 16), _ft())
    x[..., :IN_CHANNELS] = _st(x_in)
    h = _conv_layer(p, "e0a", x, True, tape)
    s0 = _conv_layer(p, "e0b", h, True, tape)
    h = pool(s0)
    h = _conv_layer(p, "e1a", h, True, tape)
    s1 = _conv_layer(p, "e1b", h, True, tape)
    h = pool(s1)
    h = _conv_layer(p, "e2a", h, True, tape)
    s2 = _conv_layer(p, "e2b", h, True, tape)
    h = pool(s2)
    h = _conv_layer(p, "b3a", h, True, tape)
    h = _conv_layer(p, "b3b", h, True, tape)
    h = _conv_layer(p, "b3c", h, True, tape)
    h = _st(up(h) + s2)
    h = _conv_layer(p, "d2a", h, True, tape)
    h = _conv_layer(p, "d2b", h, True, tape)
    h = _st(up(h) + s1)
    h = _conv_layer(p, "d1a", h, True, tape)
    h = _conv_layer(p, "d1b", h, True, tape)
    h = _st(up(h) + s0)
    h = _conv_layer(p, "d0a", h, True, tape)
    return _conv_layer(p, "d0b", h, False, tape)


def loss_and_seed(y: np.ndarray, target: np.ndarray) -> tuple[float, np.ndarray]:
    """Mean squared error of channel 0 over the G^3 voxels and its gradient (bf16, all channels)."""
    n = target.size
    r = y[..., 0].astype(np.float64) - target.astype(np.float64)
    d = np.zeros(y.shape, _ft())
    d[..., 0] = (2.0 / n) * r
    return float(np.mean(r * r)), _st(d)


def _conv_bwd(p, name, dy, grads):
    """dy: gradient w.r.t. the layer's stored output; returns dx (bf16)."""
    x, y, relu = grads["_tape"].acts[name]
    dpre = _st(np.where(y > 0, dy, 0.0).astype(_ft())) if relu else dy
    grads[name + ".w"] = conv3d_wgrad(x, dpre).astype(_ft())
    grads[name + ".b"] = dpre.astype(np.float64).sum(axis=(0, 1, 2)).astype(_ft())
    return _st(conv3d_dgrad(dpre, _st(p[name + ".w"])).astype(_ft()))


def backward(p: dict, tape: Tape, dout: np.ndarray) -> dict[str, np.ndarray]:
    """Parameter gradients of the loss, given dL/d(output) (bf16, [G,G,G,16])."""
    g = {"_tape": tape}
    d = _conv_bwd(p, "d0b", dout, g)
    d = _conv_bwd(p, "d0a", d, g)
    ds0 = d
    d = _st(up_bwd(d))
    d = _conv_bwd(p, "d1b", d, g)
    d = _conv_bwd(p, "d1a", d, g)
    ds1 = d
    d = _st(up_bwd(d))
    d = _conv_bwd(p, "d2b", d, g)
    d = _conv_bwd(p, "d2a", d, g)
    ds2 = d
    d = _st(up_bwd(d))
    d = _conv_bwd(p, "b3c", d, g)
    d = _conv_bwd(p, "b3b", d, g)
    d = _conv_bwd(p, "b3a", d, g)
    d = _st(pool_bwd(d) + ds2)
    d = _conv_bwd(p, "e2b", d, g)
    d = _conv_bwd(p, "e2a", d, g)
    d = _st(pool_bwd(d) + ds1)
    d = _conv_bwd(p, "e1b", d, g)
    d = _conv_bwd(p, "e1a", d, g)
    d = _st(pool_bwd(d) + ds0)
    d = _conv_bwd(p, "e0b", d, g)
    _conv_bwd(p, "e0a", d, g)
    del g["_tape"]
    g["e0a.w"][:, IN_CHANNELS:, :] = 0.0
    return g


def adam_step(p, g, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """Adam (bias-corrected), float32 master weights; state = {"t": int, "m": {}, "v": {}}."""
    state["t"] += 1
    t = state["t"]
    for k, gk in g.items():
        m = state["m"].setdefault(k, np.zeros_like(gk))
        v = state["v"].setdefault(k, np.zeros_like(gk))
        m[...] = b1 * m + (1 - b1) * gk
        v[...] = b2 * v + (1 - b2) * gk * gk
        mh = m / (1 - b1 ** t)
        vh = v / (1 - b2 ** t)
        p[k] = (p[k] - lr * mh / (np.sqrt(vh) + eps)).astype(p[k].dtype)
    return p
