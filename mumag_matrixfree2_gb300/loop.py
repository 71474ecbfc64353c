"""Command-line hysteresis loop on the GPU backend, with the reference's CLI (``src/loop.py:338-1180``).

    python -m mumag_matrixfree2_gb300.loop MODEL          # MODEL.npz (+ MODEL.krn, MODEL.p2 if present)
    python -m mumag_matrixfree2_gb300.loop --mesh box.npz --materials box.krn --B-start 2 --B-end -2

Same inputs and outputs as the reference: an NPZ mesh (``knt``, ``ijk`` with an optional material
column), a MaMMoS ``.krn`` file (theta, phi, K1, K2, Js, A per material group), an optional ``.p2``
file whose [mesh], [field], [initial state], [minimizer] and [poisson] entries override the defaults, fields in
Tesla, and the CSV / ``.mh`` files of ``run_hysteresis_loop`` in ``--out-dir``.  Values given on the
command line win over the ``.p2`` file, which wins over the defaults (``src/loop.py:940-1062``).

The mesh must already contain its air region: the reference's graded-shell generation
(``--add-shell``) needs TetGen/meshpy and is not part of this backend.
"""

from __future__ import annotations

import argparse
import configparser
import sys
from pathlib import Path

import numpy as np

MU0 = 4e-7 * np.pi
METHODS = ("cohen", "pcg", "pcohen", "pcohen_hs", "pcohen_exact", "pcohen_hs_exact", "lbfgs", "plbfgs", "dplbfgs",
           "tn_split", "wg_np", "tr", "aapg", "aapg_exact", "pnag", "pcohen_lbfgs", "ptr")


def read_krn(path, G: int, mesh_unit: float = 1e-9):
    """(A [J/m * (1/mesh_unit)^2], K1, Js, easy axes) of G material groups from a .krn file
    (columns theta, phi, K1, K2, Js, A, ...; exactly G rows), as ``src/loop.py:105-171`` reads it."""
    data = np.loadtxt(path, ndmin=2)
    if data.shape[0] != G:
        raise ValueError(f"{path}: {data.shape[0]} material rows for a mesh with {G} groups (need exactly {G})")
    theta, phi = data[:, 0], data[:, 1]
    k = np.column_stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)])
    return data[:, 5] * (1.0 / mesh_unit) ** 2, data[:, 2].copy(), data[:, 4].copy(), k


def read_p2(path) -> dict:
    """Overrides from a .p2 file ([mesh] size; [field] h or hx/hy/hz, hstart, hfinal, hstep, mfinal,
    mstep, loop, bias_type, bias_strength; [initial state] mx/my/mz; [minimizer] tol_fun, eps_a,
    max_iter, tau0, method, pc_iters, pc_auto, pc_force_eta, pc_force_alpha, pc_stagnation_nu, memory,
    tn_iters, lr, mu, pc_reg, wg_gamma, phi_extrapolate; [poisson] cg_maxiter, cg_tol, reg), as
    ``src/loop.py:174-288`` reads it.  Fields stay in Tesla."""
    cp = configparser.ConfigParser()
    cp.read(path)
    out: dict = {}
    if "mesh" in cp and "size" in cp["mesh"]:
        out["mesh_unit"] = float(cp["mesh"]["size"])
    if "field" in cp:
        f = cp["field"]
        if "h" in f:
            h = np.array([float(x) for x in f["h"].split(",")])
        elif any(k in f for k in ("hx", "hy", "hz")):
            h = np.array([float(f.get("hx", 0.0)), float(f.get("hy", 0.0)), float(f.get("hz", 0.0))])
        else:
            h = None
        if h is not None:
            out["h_dir"] = h / (np.linalg.norm(h) + 1e-30)
        for key, name in (("hstart", "B_start"), ("hfinal", "B_end"), ("hstep", "dB"), ("mfinal", "mfinal"),
                          ("mstep", "mstep"), ("bias_strength", "bias_strength")):
            if key in f:
                out[name] = float(f[key])
        if "loop" in f:
            out["loop"] = f.getboolean("loop")
        if "bias_type" in f:
            out["bias_type"] = str(f["bias_type"])
    if "initial state" in cp:
        s = cp["initial state"]
        if all(k in s for k in ("mx", "my", "mz")):
            v = np.array([float(s["mx"]), float(s["my"]), float(s["mz"])])
            out["m0_dir"] = v / (np.linalg.norm(v) + 1e-30)
    if "minimizer" in cp:
        mn = cp["minimizer"]
        for key, name, typ in (("tol_fun", "tau_f", float), ("eps_a", "eps_a", float), ("max_iter", "max_iter", int),
                               ("tau0", "tau0", float), ("method", "method", str), ("pc_iters", "pc_iters", int),
                               ("pc_force_eta", "pc_force_eta", float), ("pc_force_alpha", "pc_force_alpha", float),
                               ("pc_stagnation_nu", "pc_stagnation_nu", float), ("memory", "memory", int),
                               ("tn_iters", "tn_iters", int), ("lr", "lr", float), ("mu", "mu", float),
                               ("pc_reg", "pc_reg", float), ("wg_gamma", "wg_gamma", int)):
            if key in mn:
                out[name] = typ(mn[key])
        for key in ("pc_auto", "phi_extrapolate"):
            if key in mn:
                out[key] = mn.getboolean(key)
    if "poisson" in cp:
        po = cp["poisson"]
        for key, name, typ in (("cg_maxiter", "cg_maxiter", int), ("cg_tol", "cg_tol", float),
                               ("reg", "poisson_reg", float)):
            if key in po:
                out[name] = typ(po[key])
    return out


def bias_field(knt, conn, mat_id, bias_type, strength) -> np.ndarray | None:
    """Per-node symmetry-breaking field (``src/loop.py:1064-1083``): "circular" is the unit azimuthal
    field (-y, x) / |(x, y)| around the centre of the magnet's nodes, "random" unit vectors from
    numpy's default_rng(42); both scaled by ``strength`` (reduced units)."""
    if bias_type is None:
        return None
    B = np.zeros((knt.shape[0], 3))
    if bias_type == "circular":
        mag = np.unique(conn[mat_id == 1])
        if mag.size > 0:
            xy = knt - np.mean(knt[mag], axis=0)
            nr = np.sqrt(xy[:, 1] ** 2 + xy[:, 0] ** 2) + 1e-30
            B[:, 0] = -xy[:, 1] / nr
            B[:, 1] = xy[:, 0] / nr
    elif bias_type == "random":
        B = np.random.default_rng(42).standard_normal((knt.shape[0], 3))
        B /= np.linalg.norm(B, axis=1, keepdims=True) + 1e-30
    else:
        raise ValueError(f"bias type {bias_type!r} (circular or random)")
    return B * strength


def parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser(description="hysteresis loop on the GB300 backend (reference CLI)")
    ap.add_argument("modelname", nargs="?", default=None, help="MODEL: MODEL.npz, MODEL.krn, MODEL.p2")
    ap.add_argument("--mesh", help="Input NPZ mesh (knt, ijk).")
    ap.add_argument("--materials", help="Path to a .krn file (theta, phi, K1, K2, Js, A per group).")
    ap.add_argument("--add-shell", action="store_true", help="not available: needs TetGen/meshpy")
    ap.add_argument("--precond-type", default="amgcl", choices=["jacobi", "amg", "amgcl"])
    ap.add_argument("--operator-mode", default="assembled", choices=["matrix_free", "assembled"])
    ap.add_argument("--cg-maxiter", type=int, default=2000)
    ap.add_argument("--cg-tol", type=float, default=1e-8)
    ap.add_argument("--poisson-reg", type=float, default=1e-12)
    ap.add_argument("--h-dir", type=str, default="0,0,1")
    ap.add_argument("--B-start", type=float, default=-1.0)
    ap.add_argument("--B-end", type=float, default=1.0)
    ap.add_argument("--dB", type=float, default=0.05)
    ap.add_argument("--max-iter", type=int, default=2000)
    ap.add_argument("--tau-f", type=float, default=1e-8)
    ap.add_argument("--eps-a", type=float, default=1e-12)
    ap.add_argument("--tau0", type=float, default=1e-2)
    ap.add_argument("--bias-type", default=None, choices=["circular", "random"])
    ap.add_argument("--bias-strength", type=float, default=0.0)
    ap.add_argument("--method", default="pcohen_hs", choices=list(METHODS))
    ap.add_argument("--pc-iters", type=int, default=10)
    ap.add_argument("--pc-auto", action="store_true", default=True)
    ap.add_argument("--pc-no-auto", action="store_false", dest="pc_auto")
    ap.add_argument("--pc-force-eta", type=float, default=0.5)
    ap.add_argument("--pc-force-alpha", type=float, default=0.5)
    ap.add_argument("--pc-stagnation-nu", type=float, default=0.01)
    ap.add_argument("--memory", type=int, default=5)
    ap.add_argument("--tn-iters", type=int, default=5)
    ap.add_argument("--L", type=int, default=None, help="CG restart period (default: the number of nodes)")
    ap.add_argument("--lr", type=float, default=0.1)
    ap.add_argument("--mu", type=float, default=0.9)
    ap.add_argument("--pc-reg", type=float, default=0.0)
    ap.add_argument("--wg-gamma", type=int, default=5)
    ap.add_argument("--phi-extrapolate", action="store_true", default=True)
    ap.add_argument("--no-phi-extrapolate", action="store_false", dest="phi_extrapolate")
    # src/loop.py:697,759-760,977: the reference selects its C++ minimizer with --cpp-mkl (default: on
    # hosts without a GPU).  Here the GPU runs either way; the flag selects that minimizer's conventions
    # for pcohen_hs / pcohen (counting and the lagged energy test of run_cpp_pcohen_hs_minimization).
    ap.add_argument("--cpp-mkl", action=argparse.BooleanOptionalAction, default=None)
    ap.add_argument("--m0-dir", type=str, default="0,0,1")
    ap.add_argument("--out-dir", default="hyst_out")
    ap.add_argument("--snapshot-every", type=int, default=1, help="VTU snapshot every N steps (0: none)")
    ap.add_argument("--verbose", action="store_true")
    # accepted so that the reference's command lines run unchanged; this backend has a single path for
    # each of them (assembled operators on the GPU, one device, no shell generation)
    compat = ap.add_argument_group("accepted for compatibility, no effect")
    compat.add_argument("--geom-backend", default="stored_JinvT", choices=["stored_JinvT", "stored_grad_phi", "on_the_fly"])
    compat.add_argument("--chunk-elems", type=int, default=200_000)
    compat.add_argument("--cpu-spmv-backend", default="persistent_mkl",
                        choices=["persistent_mkl", "dot_product_mkl", "scipy", "jax_default", "custom_jax", "mkl_ffi"])
    compat.add_argument("--poisson-solver", default="auto", choices=["auto", "jax", "pardiso", "jax_mkl"])
    compat.add_argument("--tau-min", type=float, default=1e-6)
    compat.add_argument("--tau-max", type=float, default=1.0)
    compat.add_argument("--wg-threshold", type=float, default=1e-6)
    compat.add_argument("--data-parallel", action="store_true")
    compat.add_argument("--benchmark", action="store_true")
    shell = ap.add_argument_group("shell generation (with --add-shell, which this backend refuses)")
    shell.add_argument("--shell-type", default="hull", choices=["triangles", "hull"])
    shell.add_argument("--layers", type=int, default=None)
    shell.add_argument("--K", type=float, default=1.5)
    shell.add_argument("--KL", type=float, default=10.0)
    shell.add_argument("--auto-layers", action="store_true")
    shell.add_argument("--beta", type=float, default=1.0)
    shell.add_argument("--center", default="0,0,0")
    shell.add_argument("--h0", type=float, default=None)
    shell.add_argument("--hmax", type=float, default=None)
    shell.add_argument("--minratio", type=float, default=1.4)
    shell.add_argument("--max-steiner", type=int, default=None)
    shell.add_argument("--no-exact", action="store_true")
    shell.add_argument("--shell-verbose", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed", "fp32_precond"],
                    help="demag solve precision of this backend (mixed: FP32 inside FP64 refinement)")
    return ap


def _explicit(ap, argv) -> set:
    """Destinations whose flag appears on the command line (they win over the .p2 file)."""
    out = set()
    for act in ap._actions:
        if any(any(a == f or a.startswith(f + "=") for a in argv) for f in act.option_strings):
            out.add(act.dest)
    return out


def main(argv=None) -> dict:
    from . import fem_utils
    from .hysteresis_loop import LoopParams, run_hysteresis_loop
    from .io_utils import write_mh

    argv = list(sys.argv[1:] if argv is None else argv)
    ap = parser()
    args = ap.parse_args(argv)
    if args.add_shell:
        ap.error("--add-shell needs TetGen/meshpy (graded shell generation), which this backend does not include; "
                 "pass a mesh that already contains its air region")
    p2 = {}
    if args.modelname:
        base = Path(args.modelname)
        args.mesh = args.mesh or str(base.with_suffix(".npz"))
        if args.materials is None and base.with_suffix(".krn").exists():
            args.materials = str(base.with_suffix(".krn"))
        if args.out_dir == "hyst_out":
            args.out_dir = f"hyst_{base.name}"
        if base.with_suffix(".p2").exists():
            p2 = read_p2(base.with_suffix(".p2"))
    if args.mesh is None:
        ap.error("the following arguments are required: --mesh or modelname")
    if args.materials is None:
        cand = Path(args.mesh).with_suffix(".krn")
        if not cand.exists():
            ap.error("no .krn materials file given or found next to the mesh")
        args.materials = str(cand)
    data = np.load(args.mesh)
    knt = np.asarray(data["knt"], np.float64)
    ijk = np.asarray(data["ijk"])
    mat_id = ijk[:, 4].astype(np.int32) if ijk.shape[1] == 5 else np.ones(ijk.shape[0], np.int32)
    if mat_id.min() == 0:
        mat_id = mat_id + 1
    G = int(mat_id.max())
    mesh_unit = p2.get("mesh_unit", 1e-9)
    A, K1, Js, k = read_krn(args.materials, G, mesh_unit)
    Js_ref = float(Js.max()) or 1.0
    Kd = Js_ref**2 / (2.0 * MU0)
    s = fem_utils.prepare(knt, np.column_stack([ijk[:, :4], mat_id]), A / Kd, K1 / Kd, Js / Js_ref, k)

    explicit = _explicit(ap, argv)
    prm = dict(h_dir=np.array([float(x) for x in args.h_dir.split(",")]), B_start=args.B_start, B_end=args.B_end,
               dB=args.dB, max_iter=args.max_iter, tau_f=args.tau_f, eps_a=args.eps_a, tau0=args.tau0,
               method=args.method, pc_iters=args.pc_iters, memory=args.memory, cg_tol=args.cg_tol,
               cg_maxiter=args.cg_maxiter, poisson_reg=args.poisson_reg, loop=False, mfinal=None, mstep=None,
               pc_auto=args.pc_auto, pc_force_eta=args.pc_force_eta, pc_force_alpha=args.pc_force_alpha,
               pc_stagnation_nu=args.pc_stagnation_nu, tn_iters=args.tn_iters, lr=args.lr, mu=args.mu,
               pc_reg=args.pc_reg, wg_gamma=args.wg_gamma, phi_extrapolate=args.phi_extrapolate,
               bias_type=args.bias_type, bias_strength=args.bias_strength, L=args.L, cpp_mkl=bool(args.cpp_mkl))
    m0_dir = np.array([float(x) for x in args.m0_dir.split(",")])
    for key, val in p2.items():
        if key == "m0_dir":
            if "m0_dir" not in explicit:
                m0_dir = val
        elif key in prm and key not in explicit:
            prm[key] = val
    for key in ("B_start", "B_end", "dB", "mfinal", "mstep"):  # Tesla -> reduced units
        if prm[key] is not None:
            prm[key] = prm[key] / Js_ref
    params = LoopParams(**prm, out_dir=args.out_dir, verbose=args.verbose, Js_ref=Js_ref,
                        snapshot_every=args.snapshot_every)
    m0 = np.tile(m0_dir / np.linalg.norm(m0_dir), (s.N, 1))
    B_bias = bias_field(s.knt, s.geom.conn, s.geom.mat_id, params.bias_type, params.bias_strength)
    res = run_hysteresis_loop(knt, s.geom, s.A_lookup, s.K1_lookup, s.Js_lookup, s.k_easy, m0, params, s.V_mag,
                              s.node_volumes, s.M_nodal, B_bias=B_bias, boundary_mask=s.boundary_mask,
                              precond_type=args.precond_type, mode=args.operator_mode, precision=args.precision)
    # the mammos-mumag history file is named after the model (src/loop.py:1248-1251)
    mh_name = Path(args.modelname).name if args.modelname else "hysteresis"
    write_mh(Path(args.out_dir) / mh_name, res["history"])
    print(f"[ok] Wrote mammos-mumag compatibility file: {Path(args.out_dir) / mh_name}.mh")
    try:
        import mammos_entity  # noqa: F401
    except ImportError:
        # src/io_utils.py:271-300 skips the mammos_entity CSV the same way when the package is absent
        print("[warning] mammos_entity not found, skipping CSV conversion")
    return res


if __name__ == "__main__":
    main()
