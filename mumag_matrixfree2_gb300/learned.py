"""Learned demag warm start on the GPU (no counterpart in the reference).

A 3D U-Net (``mm_unet_*`` in libmumag_cuda) predicts the change of the demag potential caused by a
change of magnetisation, from the voxelised change of m (and, optionally, the voxelised previous
potential).  The demag solve then starts from ``U_last + interp(prediction)`` instead of ``U_last``
and runs PCG to the same tolerance, so the result does not depend on the prediction's quality.

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

    def forward_dev(self, x, y=None, nb: int | None = None):
        """Device variant: x a CUDA float32 tensor [nb, G^3, 4] (or None: the voxelised input already in
        place), y a CUDA float32 tensor [nb, G^3] for output channel 0 (or None)."""
        nb = int(nb if nb is not None else x.shape[0])
        self._check("mm_unet_forward_dev", _abi.lib().mm_unet_forward_dev(
            self.h, None if x is None else C.c_void_p(x.data_ptr()), nb,
            None if y is None else C.c_void_p(y.data_ptr())))

    def sync(self):
        """Wait for the network's stream (and report a convolution that gave up waiting)."""
        self._check("mm_unet_sync", _abi.lib().mm_unet_sync(self.h))

    def backward_dev(self, target) -> float:
        loss = C.c_double()
        self._check("mm_unet_backward_dev", _abi.lib().mm_unet_backward_dev(
            self.h, C.c_void_p(target.data_ptr()), int(target.shape[0]), C.byref(loss)))
        return float(loss.value)

    def read(self, name: str, sample: int = 0, grad: bool = False) -> np.ndarray:
        """One sample of an activation (or its gradient) as [G_l, G_l, G_l, C]."""
        which = TENSORS.index(name)
        lvl, ch = C.c_int(), C.c_int()
        _abi.lib().mm_unet_tensor_info(which, C.byref(lvl), C.byref(ch))
        g = self.G >> lvl.value
        out = np.empty((g, g, g, ch.value), np.float32)
        self._check("mm_unet_read_tensor", _abi.lib().mm_unet_read_tensor(self.h, which, int(grad), sample, _f32p(out)))
        return out


# ------------------------------------------------------------------------------------------------
# mesh <-> voxel grid
# ------------------------------------------------------------------------------------------------
@dataclass(frozen=True)
class GridSpec:
    """G^3 cubic voxels with centres lo + (i + 1/2) h."""

    lo: tuple
    h: float
    G: int

    def centres(self, i):
        return np.asarray(self.lo) + (np.asarray(i, np.float64) + 0.5) * self.h


def grid_around_magnet(knt, conn, mat_id, Js_lookup, margin: float, G: int) -> GridSpec:
    """The cube around the magnetic elements' bounding box, widened by `margin` on every side."""
    Js_e = np.asarray(Js_lookup, np.float64)[np.asarray(mat_id) - 1]
    nodes = np.unique(np.asarray(conn)[Js_e > 0].reshape(-1))
    lo, hi = knt[nodes].min(0), knt[nodes].max(0)
    c = 0.5 * (lo + hi)
    edge = float((hi - lo).max()) + 2.0 * margin
    return GridSpec(tuple(c - edge / 2), edge / G, int(G))


def locate_voxels(knt, conn, grad_phi, spec: GridSpec, chunk: int = 200_000):
    """Containing tetrahedron and its P1 (barycentric) weights for every voxel centre (-1: none).

    Tetrahedra are bucketed by the voxel centres inside their bounding boxes; a centre belongs to
    the first tetrahedron (in element order) whose barycentric coordinates are all >= -1e-9.
    """
    G, h, lo = spec.G, spec.h, np.asarray(spec.lo)
    V = G ** 3
    tet_of = np.full(V, -1, np.int64)
    lam_of = np.zeros((V, 4))
    conn = np.asarray(conn)
    for e0 in range(0, conn.shape[0], chunk):
        cidx = np.arange(e0, min(e0 + chunk, conn.shape[0]))
        X = knt[conn[cidx]]
        i0 = np.clip(np.ceil((X.min(1) - lo) / h - 0.5 - 1e-9).astype(np.int64), 0, G)
        i1 = np.clip(np.floor((X.max(1) - lo) / h - 0.5 + 1e-9).astype(np.int64), -1, G - 1)
        ext = np.maximum(i1 - i0 + 1, 0)
        n = ext.prod(1)
        sel = np.flatnonzero(n > 0)
        if sel.size == 0:
            continue
        cnt = n[sel]
        loc = np.repeat(sel, cnt)
        k = np.arange(loc.size) - np.repeat(np.cumsum(cnt) - cnt, cnt)
        ex = ext[loc]
        ijk = i0[loc] + np.stack([k % ex[:, 0], (k // ex[:, 0]) % ex[:, 1], k // (ex[:, 0] * ex[:, 1])], 1)
        p = lo + (ijk + 0.5) * h
        lam = 1.0 + np.einsum("pac,pac->pa", grad_phi[cidx[loc]], p[:, None, :] - X[loc])
        ok = lam.min(1) >= -1e-9
        vox = ((ijk[ok, 2] * G + ijk[ok, 1]) * G + ijk[ok, 0])
        tets = cidx[loc[ok]]
        lam = lam[ok]
        order = np.lexsort((tets, vox))
        vox, tets, lam = vox[order], tets[order], lam[order]
        first = np.ones(vox.size, bool)
        first[1:] = vox[1:] != vox[:-1]
        vox, tets, lam = vox[first], tets[first], lam[first]
        new = tet_of[vox] < 0
        tet_of[vox[new]] = tets[new]
        lam_of[vox[new]] = lam[new]
    return tet_of, lam_of


class GridMap:
    """Tables between the mesh nodes and the voxel grid of the warm start.

    mesh -> grid: every voxel centre takes the P1 interpolant of its tetrahedron (idx4, w4); jsf is
    Js_e / max Js of that tetrahedron (0 in air), which masks the magnetisation channels.
    grid -> mesh: every node inside the hull of the voxel centres takes the trilinear interpolant of
    its 8 surrounding centres, multiplied by a taper that falls linearly to 0 over the outermost
    `taper` voxels (the correction is continuous where it ends).
    """

    def __init__(self, knt, conn, grad_phi, mat_id, Js_lookup, spec: GridSpec, taper: float = 3.0):
        self.spec = spec
        G = spec.G
        conn = np.asarray(conn)
        tet, lam = locate_voxels(knt, conn, np.asarray(grad_phi).reshape(-1, 4, 3), spec)
        ok = tet >= 0
        self.idx4 = np.where(ok[:, None], conn[np.maximum(tet, 0)], -1).astype(np.int32)
        self.w4 = np.where(ok[:, None], lam, 0.0).astype(np.float32)
        Js = np.asarray(Js_lookup, np.float64)
        Js_e = Js[np.asarray(mat_id) - 1]
        self.jsf = np.where(ok, Js_e[np.maximum(tet, 0)] / max(Js.max(), 1e-30), 0.0).astype(np.float32)
        f = (np.asarray(knt) - np.asarray(spec.lo)) / spec.h - 0.5
        inside = np.all((f >= 0.0) & (f <= G - 1), axis=1)
        self.nodes = np.flatnonzero(inside).astype(np.int32)
        fi = f[inside]
        i = np.clip(np.floor(fi).astype(np.int64), 0, G - 2)
        t = fi - i
        d = np.minimum(fi, (G - 1) - fi)
        tap = np.clip(d / taper, 0.0, 1.0).prod(1)
        idx, w = [], []
        for c in range(8):
            o = np.array([c & 1, (c >> 1) & 1, c >> 2])
            ii = i + o
            idx.append((ii[:, 2] * G + ii[:, 1]) * G + ii[:, 0])
            w.append(np.prod(np.where(o == 1, t, 1.0 - t), axis=1) * tap)
        self.idx8 = np.stack(idx, 1).astype(np.int32)
        self.w8 = np.stack(w, 1).astype(np.float32)
        self.covered = float(ok.mean())


class WarmStart:
    """The learned initial guess of a demag solve on one mesh.

    The network has no biases (they are held at zero), so it is positively homogeneous,
    f(a x) = a f(x): one trained network serves every step size, and a prediction needs no
    per-sample normalisation on the device.  Input channels: dm * jsf (3) and c_U * U_a * jsf (1).
    The exact change U_b - U_a = A^-1 D (m_b - m_a) depends on dm alone, so c_U is 0 by default (the
    U channel holds zeros); with u_channel=True it is fixed when training starts so that both kinds of
    channel have comparable magnitudes (the ratio then varies by orders of magnitude between pairs
    with large and with tiny dm, which made training much worse on the 80 nm cube);
    output: U_b - U_a.  Training pairs are normalised by 1 / max|dm| (conditioning only).

    State fields on the grid (float32, [G^3, 5]): m * jsf (3), U * jsf (1), U (1).
    """

    def __init__(self, setup, grid: int = 64, margin: float = 20.0, batch: int = 8, params=None, seed: int = 0,
                 u_channel: bool = False):
        import torch

        self.torch = torch
        dev = torch.device("cuda")
        geom = setup.geom
        self.N = setup.N
        self.spec = grid_around_magnet(setup.knt, geom.conn, geom.mat_id, setup.Js_lookup, margin, grid)
        self.map = GridMap(setup.knt, geom.conn, geom.grad_phi, geom.mat_id, setup.Js_lookup, self.spec)
        mp = self.map
        self.idx4 = torch.from_numpy(np.maximum(mp.idx4, 0).astype(np.int64)).to(dev)
        self.w4 = torch.from_numpy(mp.w4.astype(np.float64)).to(dev)
        self.jsf = torch.from_numpy(mp.jsf.astype(np.float64)).to(dev)
        # tables of the device kernels (mm_unet_voxelise_dev / mm_unet_interp_add_dev)
        self.k_idx4 = torch.from_numpy(mp.idx4).to(dev)
        self.k_w4 = torch.from_numpy((mp.w4 * mp.jsf[:, None]).astype(np.float32)).to(dev)
        self.k_nodes = torch.from_numpy(mp.nodes).to(dev)
        self.k_idx8 = torch.from_numpy(mp.idx8).to(dev)
        self.k_w8 = torch.from_numpy(mp.w8).to(dev)
        self.G, self.V = grid, grid ** 3
        if params is None:
            params = init_params(seed)
        params = {k: (np.zeros_like(v) if k.endswith(".b") else v) for k, v in params.items()}
        self.net = UNet(grid, batch, params, seed)
        self.net._check("mm_unet_set_bias_training", _abi.lib().mm_unet_set_bias_training(self.net.h, 0))
        self.batch = batch
        self.u_channel = u_channel
        self.c_U = None
        self._x = torch.zeros((batch, self.V, 4), dtype=torch.float32, device=dev)
        self._t = torch.zeros((batch, self.V), dtype=torch.float32, device=dev)
        self._y = torch.zeros((batch, self.V), dtype=torch.float32, device=dev)
        self._c = torch.zeros(self.N, dtype=torch.float64, device=dev)  # the nodal prediction (no-wait path)

    def _vox(self, f):
        if f.dim() == 1:
            return (f[self.idx4] * self.w4).sum(1)
        return (f[self.idx4] * self.w4[..., None]).sum(1)

    def fields(self, m, U):
        """Grid fields of a solved state (m [N,3], U [N] CUDA float64 tensors)."""
        torch = self.torch
        mv = self._vox(m) * self.jsf[:, None]
        Uv = self._vox(U)
        return torch.cat([mv, (Uv * self.jsf)[:, None], Uv[:, None]], 1).float()

    def _pair(self, fa, fb, out_x, out_t=None):
        dm = fb[:, :3] - fa[:, :3]
        s = 1.0 / max(float(dm.abs().max()), 1e-30)
        out_x[:, :3] = dm * s
        out_x[:, 3] = fa[:, 3] * (self.c_U * s)
        if out_t is not None:
            out_t[:] = (fb[:, 4] - fa[:, 4]) * s
        return s

    def calibrate(self, states, pairs):
        """c_U = median max|dm| / median max|U jsf| over the pairs (0 without the U channel)."""
        if not self.u_channel:
            self.c_U = 0.0
            return self.c_U
        dm = [float((states[b][:, :3] - states[a][:, :3]).abs().max()) for a, b in pairs[:: max(1, len(pairs) // 64)]]
        um = [float(states[a][:, 3].abs().max()) for a, b in pairs[:: max(1, len(pairs) // 64)]]
        self.c_U = float(np.median(dm) / max(np.median(um), 1e-30))
        return self.c_U

    def train(self, states, pairs, steps: int, lr: float = 1e-3, seed: int = 0, log_every: int = 0):
        """Adam on random batches of (a, b) index pairs into `states` (a list of grid fields)."""
        if self.c_U is None:
            self.calibrate(states, pairs)
        rng = np.random.default_rng(seed)
        losses = []
        nb = self.batch
        for it in range(steps):
            sel = rng.integers(0, len(pairs), size=nb)
            for k, j in enumerate(sel):
                a, b = pairs[j]
                self._pair(states[a], states[b], self._x[k], self._t[k])
            self.net.forward_dev(self._x, None, nb)
            losses.append(self.net.backward_dev(self._t))
            self.net.adam(lr)
            if log_every and (it + 1) % log_every == 0:
                print(f"[warm start] step {it + 1}: loss {np.mean(losses[-log_every:]):.4e}", flush=True)
        return losses

    def predict_grid(self, fa, fb):
        """Prediction of U_b - U_a on the grid (float32 [G^3]) and its relative error (fb holds U_b)."""
        s = self._pair(fa, fb, self._x[0])
        self.net.forward_dev(self._x, self._y, 1)
        pred = self._y[0] / s
        true = fb[:, 4] - fa[:, 4]
        rel = float((pred - true).norm() / max(float(true.norm()), 1e-30))
        return pred, rel

    def exact_grid_correction(self, U_a, U_b, U):
        """U += the exact U_b - U_a sampled on the grid and interpolated back (the ceiling of any
        prediction on this grid; used to measure it)."""
        true = self._vox(U_b - U_a)
        U[self.k_nodes.long()] += (true[self.k_idx8.long()] * self.k_w8.double()).sum(1)
        return U

    def apply(self, m_new, m_old, U, prob=None, wait: bool = True):
        """U += the predicted potential change of m_old -> m_new (CUDA float64 tensors; U in place),
        entirely on the device: voxelise dm and U, run the network, interpolate to the nodes.  With
        the solver's `prob`, the prediction c is added as alpha c with alpha = c.(b - A U) / (c.A c)
        (the multiple that minimises the energy-norm error), so a poor prediction cannot hurt.
        Returns alpha (1.0 without `prob`).

        wait=False (with `prob`): the whole chain is queued without a host wait - the network's stream
        waits for the caller's current stream, the problem's stream for the network's, alpha is
        computed on the device - so the next solve on `prob` follows directly; returns None."""
        L = _abi.lib()
        if not wait and prob is not None:
            vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
            st = C.c_void_p()
            after = C.c_void_p(self.torch.cuda.current_stream().cuda_stream)
            self.net._check("mm_unet_predict_dev", L.mm_unet_predict_dev(
                self.net.h, after, 0, self.V, vp(self.k_idx4), vp(self.k_w4), vp(m_new), vp(m_old), vp(U), 1.0,
                float(self.c_U), int(self.k_nodes.numel()), vp(self.k_nodes), vp(self.k_idx8), vp(self.k_w8), 1.0,
                self.N, vp(self._c), C.byref(st)))
            prob._check("mm_scale_correction_async", L.mm_scale_correction_async(prob.h, st, vp(m_new), vp(U),
                                                                                  vp(self._c)))
            return None
        dm = m_new - m_old
        c = self.torch.zeros_like(U)
        self.torch.cuda.current_stream().synchronize()  # dm, U and c are ready before the network's stream reads them
        vp = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        self.net._check("mm_unet_voxelise_dev", L.mm_unet_voxelise_dev(
            self.net.h, 0, self.V, vp(self.k_idx4), vp(self.k_w4), vp(dm), vp(U), 1.0, float(self.c_U)))
        self.net.forward_dev(None, None, 1)
        self.net._check("mm_unet_interp_add_dev", L.mm_unet_interp_add_dev(
            self.net.h, 0, int(self.k_nodes.numel()), vp(self.k_nodes), vp(self.k_idx8), vp(self.k_w8), 1.0, vp(c)))
        if prob is None:
            U += c
            return 1.0
        a = C.c_double()
        prob._check("mm_scale_correction_dev", L.mm_scale_correction_dev(prob.h, vp(m_new), vp(U), vp(c), C.byref(a)))
        return a.value


def collect_sweep(prob, ws: WarmStart, m0, h_dir, B_values, params, keep_nodal: bool = False):
    """Minimise at every field of a sweep with the plain solver and keep each solved state's grid
    fields (and, with keep_nodal, the nodal (m, U) as CUDA tensors).  These are the training pairs'
    raw material: U solves A U = D m to the solver's tolerance at every state."""
    import torch

    m = np.asarray(m0, np.float64)
    U = np.zeros(m.shape[0])
    states, nodal, info_all = [], [], []
    h = np.asarray(h_dir, np.float64)
    for B in B_values:
        m, U, info = prob.minimize(float(B) * h, m, U, params)
        mt = torch.from_numpy(m).cuda()
        Ut = torch.from_numpy(U).cuda()
        states.append(ws.fields(mt, Ut))
        if keep_nodal:
            nodal.append((mt, Ut))
        info_all.append(info)
    return states, nodal, info_all


def time_forward(grid: int = 64, batch: int = 4, reps: int = 10, warmup: int = 3) -> dict:
    """Forward passes of a freshly initialised network on random input, timed with CUDA events."""
    import torch

    net = UNet(grid, batch)
    x = torch.randn(batch, grid ** 3, 4, device="cuda")
    net.forward_dev(x, None, batch)
    for _ in range(warmup):  # the first in-place forwards set the kernels up and capture the graph
        net.forward_dev(None, None, batch)
    net.sync()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        net.forward_dev(None, None, batch)
    net.sync()  # the network runs on its own stream: wait for it before the closing event
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flop = batch * sum(2.0 * 27 * ci * co * (grid >> lvl) ** 3 for _, lvl, ci, co, _ in LAYERS)
    return {"grid": grid, "batch": batch, "ms": ms, "flop": flop, "tflops": flop / (ms * 1e-3) / 1e12}


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="time the warm-start network's forward pass on cuda:0")
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args()
    print(json.dumps(time_forward(args.grid, args.batch, args.reps)))
