"""export_grid / export_points of a grid living on the GPU (src/IO.jl:14-59)."""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu


def test_export_device_grid(lv, tmp_path):
    from lvgpu import populate as pop
    flow = W.taylor_green(24)
    g = H.make_gpu(lv, flow, H.seeds(pop, flow))
    g["P"] = np.linspace(0.0, 1.0, g.n)
    f = lv.export_grid(g, str(tmp_path / "c.vtp"), "P", "v")
    root = ET.parse(f).getroot()
    piece = root.find("PolyData/Piece")
    counts, _, _ = g.geometry()
    assert int(piece.attrib["NumberOfPolys"]) == g.n
    assert int(piece.attrib["NumberOfPoints"]) == int(counts.sum())
    P = [da for da in root.iter("DataArray") if da.attrib["Name"] == "P"][0]
    assert np.allclose(np.array(P.text.split(), dtype=float), g["P"], rtol=0, atol=0)
    f2 = lv.export_points(g, str(tmp_path / "p.vtp"), "area")
    piece2 = ET.parse(f2).getroot().find("PolyData/Piece")
    assert int(piece2.attrib["NumberOfVerts"]) == g.n
