"""PART -> VTU conversion (vebisph_gb300/vtu.py): a well-formed VTK XML file whose points and
point data are the PART columns."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from vebisph_gb300.vtu import COLUMNS, part_to_vtu


@pytest.mark.parametrize("ncol", [10, 13])
def test_part_to_vtu_roundtrip(tmp_path, ncol):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((7, ncol))
    a[:, 8] = rng.integers(0, 2, 7)
    np.savetxt(tmp_path / "PART5", a)
    out = part_to_vtu(tmp_path / "PART5")
    root = ET.parse(out).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert piece.get("NumberOfPoints") == "7"
    arrays = {d.get("Name"): np.array(d.text.split(), dtype=float) for d in root.iter("DataArray")}
    assert np.array_equal(arrays["Points"].reshape(7, 3)[:, :2], a[:, :2])
    assert np.array_equal(arrays["velocity"].reshape(7, 3)[:, :2], a[:, 2:4])
    for k in range(4, ncol):
        assert np.array_equal(arrays[COLUMNS[k]], a[:, k]), COLUMNS[k]
    assert np.array_equal(arrays["types"], np.ones(7))
