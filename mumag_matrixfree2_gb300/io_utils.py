"""Output files of the hysteresis loop with the reference's formats (``src/io_utils.py``).

* ``hysteresis.csv``: header ``config,B_ext_T,J_par_T,E,gnorm``, one row per field step with the
  numbers in ``%.9e`` (``:31-75``);
* ``hysteresis.mh``: ``# B_ext [T]  J_parallel [T]  mx  my  mz  E [J/m^3]`` then the rows in ``%.9e``
  (``:78-95``);
* ``state_cfgNNNNN_B+x.xxxxe+00T.vtu``: an ASCII VTK UnstructuredGrid of the tetrahedral mesh with the
  nodal fields in float32 and the cell fields in int32 (``:139-268``).  Numbers are written as
  Python's ``str`` of the float32 value widened to a double, as the reference's writer does, so the
  files match it byte for byte.

Host-side I/O, outside the GPU hot path.
"""

from __future__ import annotations

from collections.abc import Sequence
from pathlib import Path

import numpy as np

CSV_COLUMNS = ("config", "B_ext_T", "J_par_T")


def write_hysteresis_header(csv_path, extra_cols: Sequence[str] = ("E", "gnorm")) -> None:
    Path(csv_path).write_text(",".join(list(CSV_COLUMNS) + list(extra_cols)) + "\n", encoding="utf-8")


def append_hysteresis_row(csv_path, config_idx: int, B_T: float, J_par_T: float, E: float | None = None,
                          gnorm: float | None = None) -> None:
    parts = [str(config_idx), f"{B_T:.9e}", f"{J_par_T:.9e}"]
    parts += [f"{v:.9e}" for v in (E, gnorm) if v is not None]
    with Path(csv_path).open("a", encoding="utf-8") as f:
        f.write(",".join(parts) + "\n")


def write_mh(path, records) -> None:
    """``records`` (n, 6): B_ext [T], J_parallel [T], mx, my, mz, E [J/m^3]; the suffix becomes .mh."""
    with open(Path(path).with_suffix(".mh"), "w") as f:
        f.write("# B_ext [T]  J_parallel [T]  mx  my  mz  E [J/m^3] \n")
        np.savetxt(f, np.asarray(records, np.float64).reshape(-1, 6), fmt="%.9e")


_VTK_TYPES = {np.dtype(np.float32): "Float32", np.dtype(np.float64): "Float64", np.dtype(np.int32): "Int32",
              np.dtype(np.int64): "Int64", np.dtype(np.uint8): "UInt8"}


def _numbers(a: np.ndarray) -> str:
    return " ".join(map(str, a.reshape(-1).tolist()))


def _data_array(name: str | None, a: np.ndarray, ncomp: int | None = None) -> list[str]:
    attrs = f'type="{_VTK_TYPES[a.dtype]}"'
    if name is not None:
        attrs += f' Name="{name}"'
    if ncomp is not None:
        attrs += f' NumberOfComponents="{ncomp}"'
    return [f"        <DataArray {attrs} format=\"ascii\">", "          " + _numbers(a), "        </DataArray>"]


def _field_arrays(data: dict, n: int, kind: str) -> list[str]:
    out = []
    for name, arr in data.items():
        a = np.asarray(arr)
        if a.shape[0] != n:
            raise ValueError(f"{kind} '{name}' length mismatch")
        a = a.astype(np.int32 if np.issubdtype(a.dtype, np.integer) else np.float32, copy=False)
        out += _data_array(name, a, 1 if a.ndim == 1 else a.shape[1])
    return out


def write_vtu_tetra(path, points, tets, *, point_data: dict | None = None, cell_data: dict | None = None) -> None:
    """Tetrahedral mesh with nodal and cell fields as an ASCII .vtu file (VTK cell type 10)."""
    pts = np.asarray(points)
    cells = np.asarray(tets)
    if pts.ndim != 2 or pts.shape[1] != 3:
        raise ValueError("points must have shape (N,3)")
    if cells.ndim != 2 or cells.shape[1] != 4:
        raise ValueError("tets must have shape (E,4)")
    N, E = pts.shape[0], cells.shape[0]
    lines = ['<?xml version="1.0"?>', '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">',
             "  <UnstructuredGrid>", f'    <Piece NumberOfPoints="{N}" NumberOfCells="{E}">', "      <Points>"]
    lines += _data_array(None, pts.astype(np.float32, copy=False), 3)
    lines += ["      </Points>", "      <Cells>"]
    lines += _data_array("connectivity", cells.astype(np.int32, copy=False))
    lines += _data_array("offsets", 4 * np.arange(1, E + 1, dtype=np.int32))
    lines += _data_array("types", np.full(E, 10, np.uint8))
    lines += ["      </Cells>", "      <PointData>"]
    lines += _field_arrays(point_data or {}, N, "PointData")
    lines += ["      </PointData>", "      <CellData>"]
    lines += _field_arrays(cell_data or {}, E, "CellData")
    lines += ["      </CellData>", "    </Piece>", "  </UnstructuredGrid>", "</VTKFile>"]
    Path(path).write_text("\n".join(lines), encoding="utf-8")


def snapshot_name(config_idx: int, B_T: float) -> str:
    """File name of a saved state (``src/hysteresis_loop.py:607``)."""
    return f"state_cfg{config_idx:05d}_B{B_T:+.4e}T.vtu"
