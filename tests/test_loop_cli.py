"""The reference-style command line (python -m mumag_matrixfree2_gb300.loop): its file readers on the
CPU and a loop through it on the GPU, against run_hysteresis_loop called directly."""

import numpy as np
import pytest

from mumag_matrixfree2_gb300 import loop as cli
from mumag_matrixfree2_gb300 import synthetic as syn


def _model(tmp_path):
    knt, ijk = syn.box_mesh(syn.WORKLOADS["cube8_h2_air24"])
    base = tmp_path / "cube"
    np.savez(base.with_suffix(".npz"), knt=knt, ijk=ijk)
    # theta, phi, K1, K2, Js, A: the magnet (easy axis 0.3 rad off z, in x-z) and the air box
    base.with_suffix(".krn").write_text("0.3 0.0 4.3e6 0.0 1.61 7.7e-12\n0.0 0.0 0.0 0.0 0.0 0.0\n")
    base.with_suffix(".p2").write_text(
        "[mesh]\nsize = 1.0e-9\n[field]\nhx = 0.0\nhy = 0.0\nhz = 1.0\nhstart = 4.0\nhfinal = -4.0\nhstep = 2.0\n"
        "[initial state]\nmx = 0\nmy = 0\nmz = 1\n[minimizer]\ntol_fun = 1e-8\neps_a = 1e-5\nmethod = pcohen_hs\n")
    return base


def test_krn_and_p2_readers(tmp_path):
    base = _model(tmp_path)
    A, K1, Js, k = cli.read_krn(base.with_suffix(".krn"), 2, 1e-9)
    assert np.allclose(A, [7.7e-12 * 1e18, 0.0]) and np.allclose(Js, [1.61, 0.0]) and np.allclose(K1, [4.3e6, 0])
    assert np.allclose(k[0], [np.sin(0.3), 0.0, np.cos(0.3)]) and np.allclose(k[1], [0, 0, 1])
    with pytest.raises(ValueError):
        cli.read_krn(base.with_suffix(".krn"), 3)
    p2 = cli.read_p2(base.with_suffix(".p2"))
    assert p2["mesh_unit"] == 1e-9 and p2["B_start"] == 4.0 and p2["B_end"] == -4.0 and p2["dB"] == 2.0
    assert np.allclose(p2["h_dir"], [0, 0, 1]) and np.allclose(p2["m0_dir"], [0, 0, 1])
    assert p2["tau_f"] == 1e-8 and p2["eps_a"] == 1e-5 and p2["method"] == "pcohen_hs"


def test_minimizer_options_and_bias_field(tmp_path):
    """Every method of the reference's --method list parses; the minimizer and bias entries of a .p2
    file are read; the circular bias field is the unit azimuthal field around the magnet's centre."""
    for method in cli.METHODS:
        assert cli.parser().parse_args(["m", "--method", method]).method == method
    a = cli.parser().parse_args(["m", "--pc-no-auto", "--no-phi-extrapolate", "--tn-iters", "7", "--lr", "0.5",
                                 "--mu", "0.8", "--bias-type", "random", "--bias-strength", "0.02"])
    assert (a.pc_auto, a.phi_extrapolate, a.tn_iters, a.lr, a.mu, a.bias_type, a.bias_strength) == \
        (False, False, 7, 0.5, 0.8, "random", 0.02)
    p2 = tmp_path / "x.p2"
    p2.write_text("[field]\nbias_type = circular\nbias_strength = 0.01\n[minimizer]\nmethod = ptr\ntn_iters = 3\n"
                  "pc_auto = false\nmu = 0.7\nphi_extrapolate = no\n[poisson]\ncg_tol = 1e-9\nreg = 1e-11\n")
    o = cli.read_p2(p2)
    assert o == {"bias_type": "circular", "bias_strength": 0.01, "method": "ptr", "tn_iters": 3, "pc_auto": False,
                 "mu": 0.7, "phi_extrapolate": False, "cg_tol": 1e-9, "poisson_reg": 1e-11}
    knt = np.array([[0.0, 0, 0], [2, 0, 0], [0, 2, 0], [0, 0, 2], [5, 5, 5], [1, 3, 0]])
    conn = np.array([[0, 1, 2, 3], [1, 2, 3, 4]])
    B = cli.bias_field(knt, conn, np.array([1, 2]), "circular", 0.5)
    c = knt[:4].mean(axis=0)
    for i in range(6):
        x, y = knt[i, 0] - c[0], knt[i, 1] - c[1]
        assert np.allclose(B[i], 0.5 * np.array([-y, x, 0.0]) / (np.hypot(x, y) + 1e-30))
    R = cli.bias_field(knt, conn, np.array([1, 2]), "random", 2.0)
    assert np.allclose(np.linalg.norm(R, axis=1), 2.0)
    assert cli.bias_field(knt, conn, np.array([1, 2]), None, 1.0) is None


# every option of the reference's command line (src/loop.py:338-740)
REFERENCE_OPTIONS = (
    "--B-end", "--B-start", "--K", "--KL", "--L", "--add-shell", "--auto-layers", "--benchmark", "--beta",
    "--bias-strength", "--bias-type", "--center", "--cg-maxiter", "--cg-tol", "--chunk-elems", "--cpp-mkl",
    "--cpu-spmv-backend", "--dB", "--data-parallel", "--eps-a", "--geom-backend", "--h-dir", "--h0", "--hmax",
    "--layers", "--lr", "--m0-dir", "--materials", "--max-iter", "--max-steiner", "--memory", "--mesh", "--method",
    "--minratio", "--mu", "--no-exact", "--no-phi-extrapolate", "--operator-mode", "--out-dir", "--pc-auto",
    "--pc-force-alpha", "--pc-force-eta", "--pc-iters", "--pc-no-auto", "--pc-reg", "--pc-stagnation-nu",
    "--phi-extrapolate", "--poisson-reg", "--poisson-solver", "--precond-type", "--shell-type", "--shell-verbose",
    "--snapshot-every", "--tau-f", "--tau-max", "--tau-min", "--tau0", "--tn-iters", "--verbose", "--wg-gamma",
    "--wg-threshold")


def test_every_reference_option_is_accepted():
    opts = set()
    for act in cli.parser()._actions:
        opts.update(act.option_strings)
    assert not set(REFERENCE_OPTIONS) - opts
    a = cli.parser().parse_args(["m", "--L", "40", "--no-cpp-mkl", "--geom-backend", "on_the_fly"])
    assert a.L == 40 and a.cpp_mkl is False


def test_cli_rejects_shell_generation_and_missing_mesh():
    with pytest.raises(SystemExit):
        cli.main(["--add-shell", "--mesh", "x.npz"])
    with pytest.raises(SystemExit):
        cli.main([])


@pytest.mark.gpu
def test_cli_loop_equals_direct_loop(cuda_ok, tmp_path):
    from mumag_matrixfree2_gb300 import fem_utils
    from mumag_matrixfree2_gb300.hysteresis_loop import LoopParams, run_hysteresis_loop

    base = _model(tmp_path)
    res = cli.main([str(base), "--out-dir", str(tmp_path / "out"), "--eps-a", "1e-6"])
    assert (tmp_path / "out" / "hysteresis.csv").exists() and (tmp_path / "out" / "hysteresis.mh").exists()
    assert (tmp_path / "out" / "cube.mh").read_text() == (tmp_path / "out" / "hysteresis.mh").read_text()
    # the same loop called directly: CLI value for eps_a wins over the .p2 file
    knt, ijk = syn.box_mesh(syn.WORKLOADS["cube8_h2_air24"])
    A, K1, Js, k, Js_ref = syn.reduced_materials(
        [syn.Material(axis=(np.sin(0.3), 0.0, np.cos(0.3))), syn.AIR])
    s = fem_utils.prepare(knt, ijk, A, K1, Js, k)
    prm = LoopParams(h_dir=np.array([0.0, 0, 1]), B_start=4.0 / Js_ref, B_end=-4.0 / Js_ref, dB=2.0 / Js_ref,
                     loop=False, tau_f=1e-8, eps_a=1e-6, out_dir=str(tmp_path / "direct"), Js_ref=Js_ref)
    ref = run_hysteresis_loop(knt, s.geom, s.A_lookup, s.K1_lookup, s.Js_lookup, s.k_easy,
                              np.tile([0.0, 0.0, 1.0], (s.N, 1)), prm, s.V_mag, s.node_volumes, s.M_nodal,
                              boundary_mask=s.boundary_mask)
    assert res["history"].shape == ref["history"].shape == (5, 6)
    assert np.allclose(res["history"], ref["history"], rtol=1e-12, atol=1e-12)
    # without mstep every step is a saved configuration: one VTU snapshot each, config = step
    snaps = sorted((tmp_path / "out").glob("state_cfg*.vtu"))
    assert len(snaps) == 5 and snaps[0].name.startswith("state_cfg00000_B+4.0000e+00T")
    cfg = np.loadtxt(tmp_path / "out" / "hysteresis.csv", delimiter=",", skiprows=1)[:, 0]
    assert np.array_equal(cfg, np.arange(5))
