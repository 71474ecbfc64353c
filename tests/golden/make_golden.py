"""Generate the golden fixtures of tests/golden/ by running the reference's own importable modules.

Run in a checkout that has the reference next to it (not on the GPU machine):

    python tests/golden/make_golden.py /path/to/mumag_matrixfree2

It imports ``src/mesh.py`` (structured grid mesher) and ``src/reorder_mesh.py`` (Morton reorder)
from the reference, which import with numpy/scipy only, and stores their outputs for small meshes:

* ``grid_box_*.npz``: ``mesh_backend_grid_box`` for three boxes (knt, ijk); the 20 nm box also
  records whether it equals the reference's test mesh ``tests/single_solid.npz``;
* ``morton_*.npz``: ``reorder_mesh(..., target="gpu")`` of a graded box mesh and of a grid box
  (knt, ijk, node_perm, inv_node_perm) together with the input mesh;
* ``io_state.vtu``, ``io_records.mh``, ``io_hysteresis.csv`` and their inputs ``io_inputs.npz``: the
  reference's ``src/io_utils.py`` writers (VTU snapshot with float32 m and U and int32 mat_id, the
  .mh history, the CSV header and rows) on seeded data.
"""

import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))


def main(ref_root: str) -> None:
    sys.path.insert(0, str(Path(ref_root) / "src"))
    import io_utils as ref_io  # noqa: E402
    import mesh as ref_mesh  # noqa: E402
    import reorder_mesh as ref_reorder  # noqa: E402

    from mumag_matrixfree2_gb300 import synthetic as syn

    ex, ey, ez = np.array([1.0, 0, 0]), np.array([0, 1.0, 0]), np.array([0, 0, 1.0])
    for ext, h in [((20.0, 20.0, 20.0), 2.0), ((8.0, 6.0, 4.0), 2.0), ((10.0, 7.0, 5.0), 1.5)]:
        knt, ijk = ref_mesh.mesh_backend_grid_box(ext, ex, ey, ez, h, False)
        name = "grid_box_%gx%gx%g_h%g.npz" % (*ext, h)
        extra = {}
        ss = Path(ref_root) / "tests" / "single_solid.npz"
        if ext == (20.0, 20.0, 20.0) and ss.exists():
            # the reference's own test mesh is this grid box, node for node
            d = np.load(ss)
            extra["equals_reference_single_solid"] = bool(
                np.array_equal(d["knt"], knt) and np.array_equal(d["ijk"], ijk))
        np.savez_compressed(HERE / name, knt=knt, ijk=ijk, extent=np.array(ext), h=h, **extra)
        print("wrote", name, knt.shape, ijk.shape)

    cases = {
        "morton_cube8_h2_air24.npz": syn.box_mesh(syn.WORKLOADS["cube8_h2_air24"]),
        "morton_grid_box_10x7x5_h1.5.npz": ref_mesh.mesh_backend_grid_box((10.0, 7.0, 5.0), ex, ey, ez, 1.5, False),
    }
    for name, (knt, ijk) in cases.items():
        with tempfile.TemporaryDirectory() as td:
            src, dst = Path(td) / "in.npz", Path(td) / "out.npz"
            np.savez(src, knt=knt, ijk=ijk)
            ref_reorder.reorder_mesh(str(src), str(dst), target="gpu")
            out = np.load(dst)
            np.savez_compressed(HERE / name, knt_in=knt, ijk_in=ijk, knt=out["knt"], ijk=out["ijk"],
                                node_perm=out["node_perm"], inv_node_perm=out["inv_node_perm"])
        print("wrote", name)

    rng = np.random.default_rng(7)
    knt, ijk = ref_mesh.mesh_backend_grid_box((8.0, 6.0, 4.0), ex, ey, ez, 2.0, False)
    m = rng.standard_normal((knt.shape[0], 3))
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    U = rng.standard_normal(knt.shape[0])
    mat_id = rng.integers(1, 3, ijk.shape[0]).astype(np.int32)
    records = rng.standard_normal((7, 6))
    rows = [(i, float(rng.standard_normal()), float(rng.standard_normal()), float(rng.standard_normal()),
             float(abs(rng.standard_normal()))) for i in range(4)]
    np.savez_compressed(HERE / "io_inputs.npz", knt=knt, conn=ijk[:, :4], m=m, U=U, mat_id=mat_id, records=records,
                        rows=np.array(rows))
    ref_io.write_vtu_tetra(HERE / "io_state.vtu", knt, ijk[:, :4],
                           point_data={"m": m.astype(np.float32), "U": U.astype(np.float32)},
                           cell_data={"mat_id": mat_id})
    ref_io.write_mh(HERE / "io_records", records)
    ref_io.write_hysteresis_header(HERE / "io_hysteresis.csv")
    for r in rows:
        ref_io.append_hysteresis_row(HERE / "io_hysteresis.csv", int(r[0]), r[1], r[2], r[3], r[4])
    print("wrote io_state.vtu, io_records.mh, io_hysteresis.csv")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the reference checkout>")
    main(sys.argv[1])
