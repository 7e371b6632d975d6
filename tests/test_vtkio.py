"""VTK export and run! with file output (src/IO.jl:14-71,
src/simulation.jl:35-94), on host data: a golden mesh stands in for the
device grid (the writers only need geometry() and get())."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from conftest import load_package

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class HostGrid:
    def __init__(self, G):
        self.G = G
        self.fields = {"x": G["x"], "area": G["area"], "centroid": G["centroid"],
                       "P": np.arange(len(G["x"]), dtype=float)}

    def geometry(self):
        return self.G["e_counts"], self.G["e_verts"], self.G["e_labels"]

    def get(self, name):
        return self.fields[name]


def _arrays(path):
    root = ET.parse(path).getroot()
    piece = root.find("PolyData/Piece")
    out = {"piece": piece.attrib}
    for da in root.iter("DataArray"):
        out[da.attrib["Name"]] = np.array([float(v) for v in (da.text or "").split()])
    return out


@pytest.fixture
def grid():
    return HostGrid(dict(np.load(os.path.join(GOLDEN, "mesh_periodic_12.npz"))))


def test_export_grid_polygons_and_cell_data(tmp_path, grid):
    lv = load_package()
    f = lv.export_grid(grid, str(tmp_path / "cells"), "P", "centroid")
    A = _arrays(f)
    n = len(grid.G["x"])
    counts = grid.G["e_counts"]
    assert int(A["piece"]["NumberOfPolys"]) == n
    assert int(A["piece"]["NumberOfPoints"]) == int(counts.sum())
    assert np.array_equal(A["offsets"], np.cumsum(counts))
    # polygon i's points are its sorted edges' first vertices; their shoelace
    # area is the stored area
    pts = A["Points"].reshape(-1, 3)
    off = np.concatenate([[0], np.cumsum(counts)])
    for i in range(n):
        v = pts[off[i]:off[i + 1], :2]
        a = 0.5 * abs(np.dot(v[:, 0], np.roll(v[:, 1], -1)) - np.dot(v[:, 1], np.roll(v[:, 0], -1)))
        assert abs(a - grid.G["area"][i]) <= 1e-13
    assert np.array_equal(A["P"], grid.fields["P"])
    cen = A["centroid"].reshape(-1, 3)
    assert np.array_equal(cen[:, :2], grid.G["centroid"]) and np.all(cen[:, 2] == 0)


def test_export_points_and_unknown_variable(tmp_path, grid):
    lv = load_package()
    f = lv.export_points(grid, str(tmp_path / "pts.vtp"), "area")
    A = _arrays(f)
    assert int(A["piece"]["NumberOfVerts"]) == len(grid.G["x"])
    assert np.array_equal(A["area"], grid.G["area"])
    with pytest.raises(ValueError):
        lv.export_points(grid, str(tmp_path / "bad.vtp"), "nonexistent")


def test_run_writes_frames_pvd_and_csv(tmp_path, grid):
    lv = load_package()

    class Sim:
        pass

    sim = Sim()
    sim.grid = grid
    sim.E = 0.0
    calls = []

    def step(s, t):
        s.E += 1.0

    def post(s, t):
        calls.append(t)

    nf = lv.run(sim, 0.1, 1.0, step, nframes=5, path=str(tmp_path / "res"), save_points=True,
                vtp_vars=("P",), csv_vars=("E",), postproc=post)
    assert nf == 5 and len(calls) == 5
    d = tmp_path / "res"
    assert sorted(os.listdir(d)) == sorted(["cells.pvd", "points.pvd", "simdata.csv"] +
                                           [f"cframe{k}.vtp" for k in range(5)] +
                                           [f"pframe{k}.vtp" for k in range(5)])
    pvd = ET.parse(d / "cells.pvd").getroot()
    files = [ds.attrib["file"] for ds in pvd.iter("DataSet")]
    assert files == [f"cframe{k}.vtp" for k in range(5)]
    rows = (d / "simdata.csv").read_text().strip().splitlines()
    assert rows[0] == "time,E" and len(rows) == 6
    assert [float(r.split(",")[1]) for r in rows[1:]] == [2.0, 4.0, 6.0, 8.0, 10.0]
