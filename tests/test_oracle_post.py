"""Moving least squares, point values and nearest polygons (movingls.jl,
voronoigrid.jl:154-178) in the CPU oracle: exact on polynomial fields, and
the host helpers (power_vector, poly_eval, integral) of the package."""
import os

import numpy as np
import pytest

from conftest import load_package


def _mesh(oracle, n=32, periodic=False, seed=5):
    import importlib.util
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location(
        "populate_post", os.path.join(here, "..", "lagrangianvoronoi.jl_gb300", "populate.py"))
    pop = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pop)
    x = pop.jittered_lattice((0, 1), (0, 1), n, n, 0.2, seed)
    g = oracle.OracleGrid((0, 1), (0, 1), 1.0 / n, n * n, xperiodic=periodic, yperiodic=periodic, max_edges=20)
    g.set("x", x)
    assert g.remesh() == 0
    return g, x


def test_movingls_reproduces_polynomials(oracle):
    g, x = _mesh(oracle)
    n = 32
    inner = np.all((x > 0.25) & (x < 0.75), axis=1)
    f1 = 2.0 * x[:, 0] - 3.0 * x[:, 1]
    L = g.movingls(1, f1, 2.0 / n)
    assert np.max(np.abs(L[inner] - [2.0, -3.0])) < 1e-11
    f2 = x[:, 0] ** 2 + x[:, 0] * x[:, 1] - 0.5 * x[:, 1] ** 2
    Q = g.movingls(2, f2, 3.0 / n)
    px, py = x[inner, 0], x[inner, 1]
    want = np.stack([2 * px + py, px - py, np.ones_like(px), np.ones_like(px), -0.5 * np.ones_like(px)], axis=1)
    assert np.max(np.abs(Q[inner] - want)) < 1e-9
    f3 = x[:, 0] ** 3 - 2 * x[:, 1] ** 3
    Cc = g.movingls(3, f3, 4.0 / n)
    assert np.max(np.abs(Cc[inner][:, 5] - 1.0)) < 1e-6 and np.max(np.abs(Cc[inner][:, 8] + 2.0)) < 1e-6


def test_point_value_and_nearest(oracle):
    g, x = _mesh(oracle)
    rng = np.random.default_rng(3)
    pts = 0.2 + 0.6 * rng.random((50, 2))
    near = g.nearest_polygon(pts)
    brute = np.argmin(((x[None, :, :] - pts[:, None, :]) ** 2).sum(-1), axis=1)
    assert np.array_equal(near, brute)
    f = 2.0 * x[:, 0] - 3.0 * x[:, 1] + 1.0
    pv = g.point_value(pts, f)
    assert np.max(np.abs(pv - (2.0 * pts[:, 0] - 3.0 * pts[:, 1] + 1.0))) < 1e-12


class _HostGrid:
    def __init__(self, E, x):
        self.E, self.x = E, x

    def geometry(self):
        return self.E["counts"], self.E["verts"], self.E["labels"]

    def get(self, name):
        return {"x": self.x}[name]


def test_host_helpers_power_vector_poly_eval_integral(oracle):
    lv = load_package()
    assert np.array_equal(lv.power_vector(lv.QuadraticExpansion, (2.0, 3.0)), [2, 3, 4, 6, 9])
    assert lv.poly_eval(1.0, np.array([1.0, 2.0]), (0.5, 0.25)) == 2.0
    g, x = _mesh(oracle, n=12)
    E = g.edges(maxe=20)
    hg = _HostGrid(E, x)
    # the linear expansion of f = 1 + 2x + 3y integrates to area * f(centroid)
    for i in (0, 17, 77):
        fi = 1 + 2 * x[i, 0] + 3 * x[i, 1]
        got = lv.integral(hg, i, fi, np.array([2.0, 3.0]), geometry=hg.geometry())
        c = E["centroid"][i]
        assert abs(got - E["area"][i] * (1 + 2 * c[0] + 3 * c[1])) < 1e-14
        # quadratic and cubic rules integrate x^2 and x^3 exactly
        q = lv.integral(hg, i, x[i, 0] ** 2, np.array([2 * x[i, 0], 0, 1.0, 0, 0]), geometry=hg.geometry())
        cu = lv.integral(hg, i, x[i, 0] ** 2, np.array([2 * x[i, 0], 0, 1.0, 0, 0, 0, 0, 0, 0]),
                         geometry=hg.geometry())
        assert abs(q - cu) < 1e-15
