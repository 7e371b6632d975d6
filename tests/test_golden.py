"""The committed golden fixtures (tests/golden/, written by make_golden.py):
the CPU oracle reproduces them exactly, and their Voronoi topology and areas
agree with an independent implementation (Qhull) stored in the fixture."""
import os

import numpy as np
import pytest

import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = {"periodic_12": True, "walls_10": False}


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"mesh_{name}.npz")))


def oracle_mesh(oracle, G, periodic):
    x = G["x"]
    n = int(round(np.sqrt(len(x))))
    g = oracle.OracleGrid((0, 1), (0, 1), 1.0 / n, len(x), xperiodic=periodic, yperiodic=periodic, max_edges=20)
    g.set("x", x)
    assert g.remesh() == 0
    return g, n


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_reproduces_golden_mesh(oracle, name):
    G = load(name)
    g, _ = oracle_mesh(oracle, G, CASES[name])
    E = g.edges(maxe=20)
    F = g.faces()
    assert np.array_equal(E["counts"], G["e_counts"])
    assert np.array_equal(E["verts"], G["e_verts"])
    assert np.array_equal(E["labels"], G["e_labels"])
    assert np.array_equal(E["area"], G["area"])
    assert np.array_equal(E["centroid"], G["centroid"])
    for k in ("rowptr", "nbr", "lrr", "len", "mid", "y"):
        assert np.array_equal(F[k], G["f_" + k]), k


def test_golden_mesh_matches_qhull():
    G = load("periodic_12")
    n = len(G["x"])
    rp, nb = G["f_rowptr"], G["f_nbr"]
    got = sorted({(i, int(nb[k])) for i in range(n) for k in range(rp[i], rp[i + 1])})
    assert got == [tuple(p) for p in G["qhull_pairs"].tolist()]
    assert np.max(np.abs(G["area"] - G["qhull_area"])) <= 1e-12
    # the cells tile the unit square
    assert abs(G["area"].sum() - 1.0) <= 1e-13


def test_golden_walls_mesh_labels():
    G = load("walls_10")
    # every boundary label -1..-4 (up, right, down, left) appears, each side
    # covered exactly once by boundary edges
    labs = np.concatenate([G["e_labels"][i, :G["e_counts"][i]] for i in range(len(G["x"]))])
    for lab in (-1, -2, -3, -4):
        assert np.any(labs == lab), lab
    tot = {lab: 0.0 for lab in (-1, -2, -3, -4)}
    for i in range(len(G["x"])):
        for k in range(G["e_counts"][i]):
            lab = int(G["e_labels"][i, k])
            if lab < 0:
                v = G["e_verts"][i, k]
                tot[lab] += np.hypot(v[0] - v[2], v[1] - v[3])
    assert all(abs(t - 1.0) <= 1e-13 for t in tot.values()), tot


def test_oracle_reproduces_golden_operator(oracle):
    G = load("periodic_12")
    g, n = oracle_mesh(oracle, G, True)
    flow = W.taylor_green(n)
    f = W.initial_fields(flow, G["x"], G["area"])
    for k, v in f.items():
        g.set(k, v)
    g.stiffened_eos(flow.gamma, flow.P0)
    op = g.pressure_operator(float(G["dt"][0]))
    b, gp = g.pressure_rhs(float(G["dt"][0]), 0)
    assert np.array_equal(op["diag"], G["op_diag"])
    assert np.array_equal(op["rowptr"], G["op_rowptr"])
    assert np.array_equal(op["col"], G["op_col"])
    assert np.array_equal(op["w"], G["op_w"])
    assert np.array_equal(b, G["rhs_b"])
    assert np.array_equal(gp, G["rhs_gp"])
