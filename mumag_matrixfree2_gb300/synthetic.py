"""Synthetic workloads: graded tensor-product box meshes, materials, initial states, field sweeps.

The reference meshes its bodies with TetGen and adds a graded air shell; neither is available here,
so the workloads are built from one tensor-product grid whose magnet part has uniform spacing ``h``
and whose air part grows geometrically (ratio ``r``) towards the box faces.  Every hexahedron is
split into six tetrahedra exactly like the reference's structured grid mesher
(``src/mesh.py:1246-1262``: A,B,D,H / A,B,F,H / A,C,D,H / A,C,G,H / A,E,F,H / A,E,G,H) with node
index ``i + (nx+1)*(j + (ny+1)*k)`` (``src/mesh.py:1230-1231``), so with no air cells the mesh is
node-for-node the reference's ``mesh_backend_grid_box``.

Material group 1 is the magnet, group 2 the air (Js = K1 = A = 0); the potential is held at zero on
the outer box faces.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

MU0 = 4e-7 * math.pi


@dataclass(frozen=True)
class BoxWorkload:
    """A cube magnet of edge ``L`` (nm) meshed at spacing ``h`` inside a graded air box of edge ``box``."""

    name: str
    L: float
    h: float
    r: float = 1.2
    n_air: int = 0
    box: float | None = None


# The three single-magnet workloads: a 40 nm cube at 2 nm in a 200 nm box (59,319 nodes / 329,232 tets),
# an 80 nm cube at 1.6 nm in a 200 nm box (357,911 nodes / 2,058,000 tets) and a 120 nm cube at 1.2 nm
# in a 240 nm box (1,601,613 nodes / 9,365,376 tets).
WORKLOADS = {
    "cube40_h2_air200": BoxWorkload("cube40_h2_air200", L=40.0, h=2.0, r=1.2, n_air=9, box=200.0),
    "cube80_h1.6_air200": BoxWorkload("cube80_h1.6_air200", L=80.0, h=1.6, r=1.15, n_air=10, box=200.0),
    "cube120_h1.2_air240": BoxWorkload("cube120_h1.2_air240", L=120.0, h=1.2, r=1.2, n_air=8, box=240.0),
    # small cases for tests
    "cube20_h2": BoxWorkload("cube20_h2", L=20.0, h=2.0),
    "cube8_h2_air24": BoxWorkload("cube8_h2_air24", L=8.0, h=2.0, r=1.3, n_air=3, box=24.0),
    "cube16_h2_air48": BoxWorkload("cube16_h2_air48", L=16.0, h=2.0, r=1.25, n_air=5, box=48.0),
}


def graded_axis(L: float, h: float, r: float, n_air: int, box: float | None) -> tuple[np.ndarray, int, int]:
    """Node coordinates along one axis and the index range [c0, c1) of the magnet cells."""
    nc = max(1, int(np.ceil(L / h)))
    core = np.linspace(-L / 2, L / 2, nc + 1)
    if n_air <= 0:
        return core, 0, nc
    if box is None or box <= L:
        raise ValueError("a graded air region needs box > L")
    w = h * r ** np.arange(1, n_air + 1, dtype=np.float64)
    w *= ((box - L) / 2.0) / w.sum()
    right = L / 2 + np.cumsum(w)
    right[-1] = box / 2
    left = -right[::-1]
    xs = np.concatenate([left, core, right])
    return xs, n_air, n_air + nc


def kuhn_box_mesh(xs: np.ndarray, ys: np.ndarray, zs: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Tensor-product grid split into six tetrahedra per hexahedron (reference node/element order)."""
    nx, ny, nz = len(xs) - 1, len(ys) - 1, len(zs) - 1
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    knt = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float64)

    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel().astype(np.int64), j.ravel().astype(np.int64), k.ravel().astype(np.int64)

    def nidx(a, b, c):
        return a + (nx + 1) * (b + (ny + 1) * c)

    A = nidx(i, j, k)
    B = nidx(i + 1, j, k)
    C = nidx(i, j + 1, k)
    D = nidx(i + 1, j + 1, k)
    E = nidx(i, j, k + 1)
    F = nidx(i + 1, j, k + 1)
    G = nidx(i, j + 1, k + 1)
    H = nidx(i + 1, j + 1, k + 1)
    tets = np.stack(
        [
            np.stack([A, B, D, H], 1),
            np.stack([A, B, F, H], 1),
            np.stack([A, C, D, H], 1),
            np.stack([A, C, G, H], 1),
            np.stack([A, E, F, H], 1),
            np.stack([A, E, G, H], 1),
        ],
        axis=1,
    ).reshape(-1, 4)
    return knt, tets.astype(np.int32)


def box_mesh(w: BoxWorkload) -> tuple[np.ndarray, np.ndarray]:
    """(knt (N,3) f64, ijk (E,5) i32) with column 4 the material group (1 magnet, 2 air)."""
    xs, c0, c1 = graded_axis(w.L, w.h, w.r, w.n_air, w.box)
    knt, tets = kuhn_box_mesh(xs, xs, xs)
    n = len(xs) - 1
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    inside = (i >= c0) & (i < c1) & (j >= c0) & (j < c1) & (k >= c0) & (k < c1)
    mat_hex = np.where(inside.ravel(), 1, 2).astype(np.int32)
    mat = np.repeat(mat_hex, 6)
    return knt, np.column_stack([tets, mat]).astype(np.int32)


@dataclass(frozen=True)
class Material:
    """Intrinsic properties of one material group (SI units; axis as a unit vector)."""

    Js: float = 1.61
    A: float = 7.7e-12
    K1: float = 4.3e6
    axis: tuple[float, float, float] = (0.0, 0.0, 1.0)


AIR = Material(Js=0.0, A=0.0, K1=0.0)


def reduced_materials(mats: list[Material], mesh_unit: float = 1e-9):
    """Lookup tables in reduced units, following ``src/loop.py:861-877`` and ``:150-163``.

    Returns (A_red, K1_red, Js_red, k_easy, Js_ref) with A scaled by (1/mesh_unit)^2 and all energy
    densities divided by Kd = Js_ref^2 / (2 mu0), Js_ref the largest Js.
    """
    Js = np.array([m.Js for m in mats], dtype=np.float64)
    A = np.array([m.A for m in mats], dtype=np.float64) * (1.0 / mesh_unit) ** 2
    K1 = np.array([m.K1 for m in mats], dtype=np.float64)
    k = np.array([m.axis for m in mats], dtype=np.float64)
    k /= np.linalg.norm(k, axis=1, keepdims=True)
    Js_ref = float(Js.max()) if Js.max() > 0 else 1.0
    Kd = Js_ref**2 / (2.0 * MU0)
    return A / Kd, K1 / Kd, Js / Js_ref, k, Js_ref


def initial_state(n_nodes: int, seed: int = 0, amplitude: float = 0.01,
                  direction=(0.0, 0.0, 1.0)) -> np.ndarray:
    """m = direction + U(-amplitude, amplitude)^3 from ``numpy.random.default_rng(seed)``, renormalised."""
    rng = np.random.default_rng(seed)
    m = np.asarray(direction, dtype=np.float64)[None, :] + rng.uniform(-amplitude, amplitude, size=(n_nodes, 3))
    return m / np.linalg.norm(m, axis=1, keepdims=True)


def field_values(H_start: float, H_end: float, dH: float, loop: bool = False) -> np.ndarray:
    """Field magnitudes of a sweep, as ``src/hysteresis_loop.py:128-150`` builds them."""
    if dH == 0:
        raise ValueError("dH must be nonzero")
    if (H_end - H_start) * dH < 0:
        dH = -dH
    n = int(np.floor((H_end - H_start) / dH + 1e-12))
    vals = H_start + dH * np.arange(n + 1)
    if abs(vals[-1] - H_end) > 1e-12 * max(1.0, abs(H_end)):
        vals = np.append(vals, H_end)
    if not loop:
        return vals
    return np.concatenate([vals, vals[-2::-1]])


def tilted_field_direction(tilt_deg: float = 1.0) -> np.ndarray:
    """Unit field direction tilted ``tilt_deg`` from +z in the x-z plane."""
    t = math.radians(tilt_deg)
    return np.array([math.sin(t), 0.0, math.cos(t)], dtype=np.float64)


# ------------------------------------------------------------------------------------------------
# batched particles: voxelised ellipsoids, each in its own graded air box
# ------------------------------------------------------------------------------------------------
@dataclass(frozen=True)
class Particle:
    """One tri-axial ellipsoid (semi-axes in nm) and its material."""

    a: float
    b: float
    c: float
    material: Material


def random_particles(n: int, seed: int = 0, semi=(5.0, 25.0)) -> list[Particle]:
    """Semi-axes U(5, 25) nm; easy axis uniform on the sphere; K1 U(1, 5) MJ/m^3; Js U(1.0, 1.6) T;
    A U(5, 12) pJ/m; from numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        a, b, c = rng.uniform(semi[0], semi[1], size=3)
        v = rng.standard_normal(3)
        v /= np.linalg.norm(v)
        mat = Material(Js=float(rng.uniform(1.0, 1.6)), A=float(rng.uniform(5e-12, 12e-12)),
                       K1=float(rng.uniform(1e6, 5e6)), axis=tuple(float(x) for x in v))
        out.append(Particle(float(a), float(b), float(c), mat))
    return out


def _graded_cells(L: float, h: float, r: float, box: float) -> int:
    """Air cells per side so that cells growing by r from h reach the box face."""
    total = 0.5 * (box - L)
    return max(1, int(math.ceil(math.log(1.0 + total * (r - 1.0) / (h * r)) / math.log(r))))


def ellipsoid_mesh(p: Particle, h: float = 1.5, r: float = 1.2, box_factor: float = 5.0):
    """(knt, ijk): hexahedra of edge h whose centre lies inside the ellipsoid are the magnet (group 1);
    the rest of the uniform core and a graded shell (ratio r) up to a cube of edge box_factor * the
    largest semi-axis are air (group 2).  Every hexahedron is split into six tetrahedra."""
    box = box_factor * max(p.a, p.b, p.c)
    axes, ranges = [], []
    for s in (p.a, p.b, p.c):
        nc = int(math.ceil(2.0 * s / h))
        L = nc * h
        xs, c0, c1 = graded_axis(L, h, r, _graded_cells(L, h, r, box), box)
        axes.append(xs)
        ranges.append((c0, c1))
    xs, ys, zs = axes
    knt, tets = kuhn_box_mesh(xs, ys, zs)
    cx, cy, cz = 0.5 * (xs[1:] + xs[:-1]), 0.5 * (ys[1:] + ys[:-1]), 0.5 * (zs[1:] + zs[:-1])
    Z, Y, X = np.meshgrid(cz, cy, cx, indexing="ij")
    inside = (X / p.a) ** 2 + (Y / p.b) ** 2 + (Z / p.c) ** 2 <= 1.0
    mat = np.repeat(np.where(inside.ravel(), 1, 2).astype(np.int32), 6)
    return knt, np.column_stack([tets, mat]).astype(np.int32)
