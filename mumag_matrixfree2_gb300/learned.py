"""Learned demag warm start on the GPU (no counterpart in the reference).

A 3D U-Net (``mm_unet_*`` in libmumag_cuda) predicts the change of the demag potential caused by a
change of magnetisation, from the voxelised change of m and the voxelised previous potential.  The
demag solve then starts from ``U_last + interp(prediction)`` instead of ``U_last`` and runs PCG to the
same tolerance, so the plain solver stays the judge of the prediction.

Because the potential is linear in m (A U = D m), the map the network learns is the linear demag
operator applied to dm; inputs and targets are normalised by the largest |dm| so that one network
serves every step size.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi

# (name, level, c_in, c_out, relu) -- the layer table of mm_unet (include/mumag_cuda.h)
LAYERS = [
    ("e0a", 0, 16, 16, True), ("e0b", 0, 16, 16, True),
    ("e1a", 1, 16, 32, True), ("e1b", 1, 32, 32, True),
    ("e2a", 2, 32, 64, True), ("e2b", 2, 64, 64, True),
    ("b3a", 3, 64, 128, True), ("b3b", 3, 128, 128, True), ("b3c", 3, 128, 64, True),
    ("d2a", 2, 64, 64, True), ("d2b", 2, 64, 32, True),
    ("d1a", 1, 32, 32, True), ("d1b", 1, 32, 16, True),
    ("d0a", 0, 16, 16, True), ("d0b", 0, 16, 16, False),
]
IN_CHANNELS = 4
TENSORS = ["x", "e0a", "s0", "p0", "e1a", "s1", "p1", "e2a", "s2", "p2", "b3a", "b3b", "b3c", "h2", "d2a", "d2b",
           "h1", "d1a", "d1b", "h0", "d0a", "out"]

_fp = C.POINTER(C.c_float)


def _f32p(a: np.ndarray):
    return a.ctypes.data_as(_fp)


def flatten(params: dict[str, np.ndarray]) -> np.ndarray:
    """Per layer w[27, c_in, c_out] then b[c_out], in layer order (the library's flat layout)."""
    parts = []
    for name, _, ci, co, _ in LAYERS:
        parts.append(np.asarray(params[name + ".w"], np.float32).reshape(27 * ci * co))
        parts.append(np.asarray(params[name + ".b"], np.float32).reshape(co))
    return np.ascontiguousarray(np.concatenate(parts))


def unflatten(flat: np.ndarray) -> dict[str, np.ndarray]:
    out, k = {}, 0
    for name, _, ci, co, _ in LAYERS:
        n = 27 * ci * co
        out[name + ".w"] = flat[k:k + n].reshape(27, ci, co).copy()
        k += n
        out[name + ".b"] = flat[k:k + co].copy()
        k += co
    return out


def init_params(seed: int = 0) -> dict[str, np.ndarray]:
    """He-uniform weights, zero biases; the last layer scaled by 0.1 (small initial corrections)."""
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


class UNet:
    """The GPU network: BF16 tensor-core forward and backward, FP32 Adam."""

    def __init__(self, grid: int, batch: int, params: dict | None = None, seed: int = 0):
        L = _abi.lib()
        h = C.c_void_p()
        rc = L.mm_unet_create(int(grid), int(batch), C.byref(h))
        if rc != 0:
            raise _abi.MMError("mm_unet_create", rc, (L.mm_unet_last_error(None) or b"").decode())
        self.h, self.G, self.B = h, int(grid), int(batch)
        n = C.c_int64()
        self._check("mm_unet_param_count", L.mm_unet_param_count(h, C.byref(n)))
        self.n_params = int(n.value)
        self.set_params(params if params is not None else init_params(seed))

    def _check(self, fn, rc):
        if rc < 0:
            raise _abi.MMError(fn, rc, (_abi.lib().mm_unet_last_error(self.h) or b"").decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            _abi.lib().mm_unet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        flat = flatten(params) if isinstance(params, dict) else np.ascontiguousarray(params, np.float32)
        assert flat.size == self.n_params
        self._check("mm_unet_set_params", _abi.lib().mm_unet_set_params(self.h, _f32p(flat)))

    def get_params(self) -> dict[str, np.ndarray]:
        flat = np.empty(self.n_params, np.float32)
        self._check("mm_unet_get_params", _abi.lib().mm_unet_get_params(self.h, _f32p(flat)))
        return unflatten(flat)

    def get_grads(self) -> dict[str, np.ndarray]:
        flat = np.empty(self.n_params, np.float32)
        self._check("mm_unet_get_grads", _abi.lib().mm_unet_get_grads(self.h, _f32p(flat)))
        return unflatten(flat)

    def forward(self, x: np.ndarray) -> np.ndarray:
        """x [nb, G, G, G, 4] -> prediction [nb, G, G, G] (output channel 0)."""
        x = np.ascontiguousarray(x, np.float32)
        nb = x.shape[0]
        y = np.empty((nb, self.G, self.G, self.G), np.float32)
        self._check("mm_unet_forward", _abi.lib().mm_unet_forward(self.h, _f32p(x), nb, _f32p(y)))
        return y

    def backward(self, target: np.ndarray) -> float:
        t = np.ascontiguousarray(target, np.float32)
        loss = C.c_double()
        self._check("mm_unet_backward", _abi.lib().mm_unet_backward(self.h, _f32p(t), t.shape[0], C.byref(loss)))
        return float(loss.value)

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self._check("mm_unet_adam", _abi.lib().mm_unet_adam(self.h, lr, beta1, beta2, eps))

    def read(self, name: str, sample: int = 0, grad: bool = False) -> np.ndarray:
        """One sample of an activation (or its gradient) as [G_l, G_l, G_l, C]."""
        which = TENSORS.index(name)
        lvl, ch = C.c_int(), C.c_int()
        _abi.lib().mm_unet_tensor_info(which, C.byref(lvl), C.byref(ch))
        g = self.G >> lvl.value
        out = np.empty((g, g, g, ch.value), np.float32)
        self._check("mm_unet_read_tensor", _abi.lib().mm_unet_read_tensor(self.h, which, int(grad), sample, _f32p(out)))
        return out
