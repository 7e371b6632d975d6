"""The GPU path on the golden fixtures (tests/golden/): polygons, geometry,
faces, the pressure operator and the right-hand side equal the fixture
bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = {"periodic_12": True, "walls_10": False}


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"mesh_{name}.npz")))


def gpu_mesh(lv, G, periodic):
    x = G["x"]
    n = int(round(np.sqrt(len(x))))
    g = lv.VoronoiGrid(lv.Rectangle((0, 1), (0, 1)), 1.0 / n, xperiodic=periodic, yperiodic=periodic)
    g.push(x)
    lv.remesh(g)
    return g, n


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_mesh_equals_golden(lv, name):
    G = load(name)
    g, _ = gpu_mesh(lv, G, CASES[name])
    counts, verts, labels = g.geometry()
    assert np.array_equal(counts, G["e_counts"])
    for i in range(len(counts)):
        k = counts[i]
        assert np.array_equal(verts[i, :k], G["e_verts"][i, :k]), i
        assert np.array_equal(labels[i, :k], G["e_labels"][i, :k]), i
    assert np.array_equal(g["area"], G["area"])
    assert np.array_equal(g["centroid"], G["centroid"])
    F = g.faces()
    for k in ("rowptr", "nbr", "lrr", "len", "mid", "y"):
        assert np.array_equal(F[k], G["f_" + k]), k


def test_gpu_operator_and_rhs_equal_golden(lv):
    G = load("periodic_12")
    g, n = gpu_mesh(lv, G, True)
    flow = W.taylor_green(n)
    for k, v in W.initial_fields(flow, G["x"], G["area"]).items():
        g[k] = v
    lv.stiffened_eos(g, flow.gamma, flow.P0)
    L = lv._lib.load()
    dt = float(G["dt"][0])
    assert L.lv_pressure_operator(g._ctx, dt) == 0
    vbc = np.zeros(8)
    assert L.lv_pressure_rhs(g._ctx, dt, 0, lv._lib.ptr(vbc)) == 0
    p = lv._lib.ptr
    nnz = C.c_int64()
    assert L.lv_export_system(g._ctx, C.byref(nnz), None, None, None, None, None) == 0
    N = g.n
    diag, rowptr, b = np.zeros(N), np.zeros(N + 1, np.int64), np.zeros(N)
    col, w = np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
    assert L.lv_export_system(g._ctx, None, p(diag), p(rowptr, C.c_int64), p(col, C.c_int32), p(w), p(b)) == 0
    assert np.array_equal(diag, G["op_diag"])
    assert np.array_equal(rowptr, G["op_rowptr"])
    assert np.array_equal(col, G["op_col"])
    assert np.array_equal(w, G["op_w"])
    assert np.array_equal(b, G["rhs_b"])
