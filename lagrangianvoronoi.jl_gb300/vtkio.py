"""VTK export and the run! driver with file output (src/IO.jl:14-71,
src/simulation.jl:35-94).

The grid stays on the GPU; an export downloads the sorted polygon edges
(lv_get_geometry) and the requested per-polygon fields once per frame.  Files
are VTK XML PolyData (.vtp) with ASCII data arrays and a ParaView collection
(.pvd) per series, as the reference writes through WriteVTK.  Any object
with `geometry()` -> (counts, verts, labels) and `get(name)` can be exported,
so the writers are host code only.
"""
import csv
import os
from xml.sax.saxutils import escape

import numpy as np


def _vec3(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        return a
    out = np.zeros((a.shape[0], 3))
    out[:, :min(2, a.shape[1])] = a[:, :2]
    return out


def _data_array(name, a):
    """One <DataArray>: scalars as Float64, 2-vectors as 3-component (Vec3)."""
    a = _vec3(a)
    ncomp = 1 if a.ndim == 1 else 3
    vals = " ".join(repr(float(v)) for v in a.ravel())
    return (f'<DataArray type="Float64" Name="{escape(name)}" NumberOfComponents="{ncomp}" format="ascii">'
            f'{vals}</DataArray>')


def _fields(grid, vars):
    out = []
    for name in vars:
        try:
            a = grid.get(name)
        except KeyError:
            raise ValueError(f"Cannot export variable {name} because it does not exist.")
        a = np.asarray(a, dtype=np.float64)
        if a.ndim == 2 and a.shape[1] > 2:
            raise ValueError(f"Cannot export variable {name}: only numbers and vectors can be exported.")
        out.append((name, a))
    return out


def _write_vtp(filename, points, polys_conn, polys_off, verts_conn, verts_off, celldata, pointdata):
    if not filename.endswith(".vtp"):
        filename = filename + ".vtp"
    npts = len(points)
    npolys, nverts = len(polys_off), len(verts_off)
    with open(filename, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="PolyData" version="1.0" byte_order="LittleEndian">\n<PolyData>\n')
        f.write(f'<Piece NumberOfPoints="{npts}" NumberOfVerts="{nverts}" NumberOfLines="0" NumberOfStrips="0" '
                f'NumberOfPolys="{npolys}">\n')
        f.write("<Points>" + _data_array("Points", points) + "</Points>\n")
        for tag, conn, off in (("Verts", verts_conn, verts_off), ("Polys", polys_conn, polys_off)):
            f.write(f"<{tag}>")
            f.write('<DataArray type="Int64" Name="connectivity" format="ascii">' + " ".join(map(str, conn)) +
                    "</DataArray>")
            f.write('<DataArray type="Int64" Name="offsets" format="ascii">' + " ".join(map(str, off)) +
                    "</DataArray>")
            f.write(f"</{tag}>\n")
        if celldata:
            f.write("<CellData>" + "".join(_data_array(n, a) for n, a in celldata) + "</CellData>\n")
        if pointdata:
            f.write("<PointData>" + "".join(_data_array(n, a) for n, a in pointdata) + "</PointData>\n")
        f.write("</Piece>\n</PolyData>\n</VTKFile>\n")
    return filename


def export_grid(grid, filename, *vars):
    """export_grid(grid, filename, vars...) (src/IO.jl:14-33): every polygon
    as one VTK polygon through its sorted vertices (the first vertex of each
    edge), and the requested per-polygon fields as cell data."""
    counts, verts, _ = grid.geometry()
    counts = np.asarray(counts)
    pts = np.concatenate([verts[i, :counts[i], 0:2] for i in range(len(counts))]) if counts.sum() else \
        np.zeros((0, 2))
    conn = np.arange(int(counts.sum()))
    off = np.cumsum(counts)
    return _write_vtp(filename, _vec3(pts), conn, off, [], [], _fields(grid, vars), [])


def export_points(grid, filename, *vars):
    """export_points(grid, filename, vars...) (src/IO.jl:52-59): the seeds as
    a cloud of VTK vertices with the requested fields."""
    x = np.asarray(grid.get("x"))
    n = len(x)
    return _write_vtp(filename, _vec3(x), [], [], np.arange(n), np.arange(1, n + 1), [], _fields(grid, vars))


class ParaviewCollection:
    """paraview_collection(...) of WriteVTK: a .pvd listing (time, file)."""

    def __init__(self, filename):
        self.filename = filename
        self.entries = []

    def __setitem__(self, t, file):
        self.entries.append((float(t), file))

    def save(self):
        d = os.path.dirname(os.path.abspath(self.filename))
        with open(self.filename, "w") as f:
            f.write('<?xml version="1.0"?>\n<VTKFile type="Collection" version="1.0" byte_order="LittleEndian">\n'
                    "<Collection>\n")
            for t, file in self.entries:
                rel = os.path.relpath(os.path.abspath(file), d)
                f.write(f'<DataSet timestep="{t!r}" part="0" file="{escape(rel)}"/>\n')
            f.write("</Collection>\n</VTKFile>\n")
        return self.filename


def run(sim, dt, t_end, step, nframes=100, path="results", save_points=False, save_grid=True, save_csv=True,
        vtp_vars=(), csv_vars=(), postproc=None, grid=None):
    """run!(sim, dt, t_end, step!; nframes, path, save_points, save_grid,
    save_csv, vtp_vars, csv_vars, postproc!) (src/simulation.jl:35-94).
    `grid` defaults to sim.grid; frames are written every k_frame steps."""
    grid = grid if grid is not None else getattr(sim, "grid", None)
    for var in csv_vars:
        if var == "time":
            raise ValueError("csv_vars cannot be :time")
    if not os.path.isdir(path):
        os.makedirs(path)
    pvd_c = ParaviewCollection(os.path.join(path, "cells.pvd"))
    pvd_p = ParaviewCollection(os.path.join(path, "points.pvd"))
    csv_data = {"time": []}
    for var in csv_vars:
        csv_data[var] = []
    k_frame = max(int(round(t_end / (nframes * dt))) if nframes > 0 else 1 << 62, 1)
    t, k, nframe = 0.0, 0, 0
    while t < t_end:
        k += 1
        step(sim, t)
        if k % k_frame == 0:
            if postproc is not None:
                postproc(sim, t)
            csv_data["time"].append(t)
            for var in csv_vars:
                csv_data[var].append(float(getattr(sim, var)))
            if save_grid:
                pvd_c[t] = export_grid(grid, os.path.join(path, f"cframe{nframe}.vtp"), *vtp_vars)
            if save_points:
                pvd_p[t] = export_points(grid, os.path.join(path, f"pframe{nframe}.vtp"), *vtp_vars)
            nframe += 1
        t += dt
    if save_grid:
        pvd_c.save()
    if save_points:
        pvd_p.save()
    if save_csv:
        with open(os.path.join(path, "simdata.csv"), "w", newline="") as f:
            w = csv.writer(f)
            keys = list(csv_data)
            w.writerow(keys)
            for row in zip(*(csv_data[k] for k in keys)):
                w.writerow(row)
    return nframe
