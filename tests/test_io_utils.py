"""The output writers against files written by the reference's own src/io_utils.py
(tests/golden/io_*, made by tests/golden/make_golden.py): byte for byte."""

from pathlib import Path

import numpy as np

from mumag_matrixfree2_gb300 import io_utils

GOLDEN = Path(__file__).parent / "golden"


def test_writers_match_the_reference_files(tmp_path):
    d = np.load(GOLDEN / "io_inputs.npz")
    io_utils.write_vtu_tetra(tmp_path / "s.vtu", d["knt"], d["conn"],
                             point_data={"m": d["m"].astype(np.float32), "U": d["U"].astype(np.float32)},
                             cell_data={"mat_id": d["mat_id"]})
    assert (tmp_path / "s.vtu").read_text() == (GOLDEN / "io_state.vtu").read_text()
    io_utils.write_mh(tmp_path / "r", d["records"])
    assert (tmp_path / "r.mh").read_text() == (GOLDEN / "io_records.mh").read_text()
    io_utils.write_hysteresis_header(tmp_path / "h.csv")
    for r in d["rows"]:
        io_utils.append_hysteresis_row(tmp_path / "h.csv", int(r[0]), r[1], r[2], r[3], r[4])
    assert (tmp_path / "h.csv").read_text() == (GOLDEN / "io_hysteresis.csv").read_text()
    assert io_utils.snapshot_name(12, -0.25) == "state_cfg00012_B-2.5000e-01T.vtu"
