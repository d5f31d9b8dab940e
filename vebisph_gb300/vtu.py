"""PART dumps to VTK UnstructuredGrid (.vtu) files, for ParaView: the job of the reference's
offline converter (vtk_conv/PART2VTU_2D.f), written from the VTK XML file format.

A PART line holds r1 r2 u1 u2 theta P conc a_out n_surf vort [tau11 tau12 tau22]
(output.F90:44-51).  Every particle becomes a VTK_VERTEX cell at (r1, r2, 0) with the columns as
point data and u as a 3-vector."""
from __future__ import annotations

import pathlib

import numpy as np

COLUMNS = ["x", "y", "u", "v", "theta", "pressure", "conc", "a_out", "n_surf", "vorticity",
           "tau_xx", "tau_xy", "tau_yy"]


def read_part(path) -> np.ndarray:
    return np.loadtxt(path, ndmin=2)


def _array(name, a, ncomp=1, kind="Float64"):
    body = " ".join(repr(float(v)) if kind == "Float64" else str(int(v)) for v in np.ravel(a))
    return (f'        <DataArray type="{kind}" Name="{name}" NumberOfComponents="{ncomp}" format="ascii">\n'
            f"          {body}\n        </DataArray>\n")


def part_to_vtu(part_path, vtu_path=None) -> pathlib.Path:
    part_path = pathlib.Path(part_path)
    vtu_path = pathlib.Path(vtu_path) if vtu_path else part_path.with_suffix(".vtu")
    a = read_part(part_path)
    n, ncol = a.shape
    if ncol not in (10, 13):
        raise ValueError(f"{part_path}: {ncol} columns, a PART line has 10 or 13")
    pts = np.column_stack([a[:, 0], a[:, 1], np.zeros(n)])
    vel = np.column_stack([a[:, 2], a[:, 3], np.zeros(n)])
    parts = ['<?xml version="1.0"?>\n',
             '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n',
             '  <UnstructuredGrid>\n',
             f'    <Piece NumberOfPoints="{n}" NumberOfCells="{n}">\n',
             '      <PointData Scalars="pressure" Vectors="velocity">\n',
             _array("velocity", vel, 3)]
    for k in range(4, ncol):
        parts.append(_array(COLUMNS[k], a[:, k], 1, "Int32" if COLUMNS[k] == "n_surf" else "Float64"))
    parts += ['      </PointData>\n', '      <Points>\n', _array("Points", pts, 3), '      </Points>\n',
              '      <Cells>\n', _array("connectivity", np.arange(n), 1, "Int32"),
              _array("offsets", np.arange(1, n + 1), 1, "Int32"), _array("types", np.ones(n), 1, "UInt8"),
              '      </Cells>\n', '    </Piece>\n', '  </UnstructuredGrid>\n', '</VTKFile>\n']
    vtu_path.write_text("".join(parts))
    return vtu_path
