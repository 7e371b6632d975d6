"""Known-answer tests of the CPU oracle (no GPU): hand-computed clips, the
cell path order, minimum-image arrows, a hand-assembled two-cell operator,
and the Voronoi topology/areas of periodic jittered lattices against an
independent implementation (scipy.spatial / Qhull)."""
import numpy as np
import pytest


def _square_edges():
    # reset! (polygon.jl:37-47) of the unit square: B->A, A->D, D->C, C->B
    A, B, C, D = (0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)
    edges = [B + A, A + D, D + C, C + B]
    return edges, [-3, -4, -1, -2]


def test_clip_unit_square_by_bisector(oracle):
    edges, labels = _square_edges()
    verts, labs, cut = oracle.clip_polygon((0.25, 0.5), (0.75, 0.5), 7, edges, labels)
    assert cut
    expected = np.array([[0.5, 0.0, 0.0, 0.0],   # B->A cut at x = 1/2, keeps v2
                         [0.0, 0.0, 0.0, 1.0],   # A->D untouched
                         [0.0, 1.0, 0.5, 1.0],   # D->C cut, keeps v1
                         [0.5, 1.0, 0.5, 0.0]])  # new edge, same (clockwise) orientation
    assert np.array_equal(verts, expected)
    assert list(labs) == [-3, -4, -1, 7]


def test_clip_no_cut_and_full_cut(oracle):
    edges, labels = _square_edges()
    # bisector outside the square: nothing changes
    verts, labs, cut = oracle.clip_polygon((0.5, 0.5), (3.0, 0.5), 9, edges, labels)
    assert not cut
    assert np.array_equal(verts, np.array(edges, dtype=float))
    # a vertex exactly on the bisector is kept exactly (polygon.jl:73-74)
    verts, labs, cut = oracle.clip_polygon((0.0, 0.0), (1.0, 1.0), 4, edges, labels)
    assert cut
    pts = {tuple(v[:2]) for v in verts} | {tuple(v[2:]) for v in verts}
    assert (1.0, 0.0) in pts and (0.0, 1.0) in pts and (1.0, 1.0) not in pts
    assert len(verts) == 3


def test_path_order(oracle):
    g = oracle.OracleGrid((0, 1), (0, 1), 0.01, 1)
    i1, i2, rr = g.path()
    first = list(zip(i1[:9], i2[:9]))
    assert first == [(0, 0), (0, -1), (-1, 0), (1, 0), (0, 1), (-1, -1), (1, -1), (-1, 1), (1, 1)]
    assert np.all(rr[:9] == 0.0)
    assert np.all(np.diff(rr) >= 0)
    h = 0.02
    k = np.maximum(0, np.abs(i1) - 1) ** 2 + np.maximum(0, np.abs(i2) - 1) ** 2
    assert np.array_equal(rr, (h * h) * k.astype(float))
    # the prefix ends with the first node beyond r_max = 10 dr
    assert rr[-1] > (10 * 0.01) ** 2 and np.all(rr[:-1] <= (10 * 0.01) ** 2)
    # ties broken by |key|^2
    for a in range(len(rr) - 1):
        if rr[a] == rr[a + 1]:
            assert i1[a] ** 2 + i2[a] ** 2 <= i1[a + 1] ** 2 + i2[a + 1] ** 2


def test_two_cell_operator(oracle):
    """Two unit squares side by side: one face of length 1 at distance 1, so
    lr_ratio = 1 and w = 1*(0.5/rho + 0.5/rho) (pressure.jl:104-117)."""
    g = oracle.OracleGrid((0, 2), (0, 1), 1.0, 2)
    g.set("x", np.array([[0.5, 0.5], [1.5, 0.5]]))
    assert g.remesh() == 0
    E = g.edges()
    assert np.array_equal(E["area"], [1.0, 1.0])
    assert np.array_equal(E["centroid"], [[0.5, 0.5], [1.5, 0.5]])
    rho, c2, dt = 2.0, 4.0, 0.5
    g.set("rho", [rho, rho])
    g.set("mass", [rho, rho])
    g.set("c2", [c2, c2])
    A = g.pressure_operator(dt)
    assert list(A["rowptr"]) == [0, 1, 2] and list(A["col"]) == [1, 0]
    assert np.array_equal(A["w"], [0.5, 0.5])
    assert np.array_equal(A["diag"], [rho / (rho * rho * c2 * dt * dt)] * 2)
    y = g.operator_apply(np.array([1.0, 3.0]))
    d = A["diag"][0]
    assert np.allclose(y, [d * 1.0 + 0.5 * (1 - 3), d * 3.0 + 0.5 * (3 - 1)], rtol=0, atol=1e-15)


def test_minimum_image_faces(oracle):
    """Across a periodic boundary the face position y is x + get_arrow(q.x, x)
    (voronoigrid.jl:116-125, iterators.jl:23-33)."""
    n = 8
    g = oracle.OracleGrid((0, 1), (0, 1), 1.0 / n, n * n, xperiodic=True, yperiodic=True)
    xs = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(xs, xs)
    x = np.stack([X.ravel(), Y.ravel()], axis=1)
    g.set("x", x)
    assert g.remesh() == 0
    F = g.faces()
    for i in range(n * n):
        for k in range(F["rowptr"][i], F["rowptr"][i + 1]):
            d = F["y"][k] - x[i]
            assert np.all(np.abs(d) <= 0.5 + 1e-12)
            assert np.allclose(np.mod(F["y"][k], 1.0), x[F["nbr"][k]], atol=1e-12)
    # square lattice: 4 faces each (the diagonal neighbours touch at a point only)
    counts = np.diff(F["rowptr"])
    assert np.all(counts == 4)
    assert np.allclose(F["lrr"], 1.0)


@pytest.mark.parametrize("n,jitter,seed", [(12, 0.1, 1), (16, 0.3, 2), (20, 0.45, 3)])
def test_periodic_voronoi_against_qhull(oracle, n, jitter, seed):
    spatial = pytest.importorskip("scipy.spatial")
    import importlib.util, os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location(
        "populate_kat", os.path.join(here, "..", "lagrangianvoronoi.jl_gb300", "populate.py"))
    pop = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(pop)
    x = pop.jittered_lattice((0, 1), (0, 1), n, n, jitter, seed)
    g = oracle.OracleGrid((0, 1), (0, 1), 1.0 / n, n * n, xperiodic=True, yperiodic=True)
    g.set("x", x)
    assert g.remesh() == 0
    F = g.faces()
    E = g.edges()
    # 3x3 tiling, Voronoi of all, ridges touching the central tile
    shifts = np.array([(a, b) for b in (-1, 0, 1) for a in (-1, 0, 1)], dtype=float)
    pts = np.concatenate([x + s for s in shifts])
    vor = spatial.Voronoi(pts)
    N = n * n
    centre = 4 * N
    ref = set()
    for (p, q), rv in zip(vor.ridge_points, vor.ridge_vertices):
        if centre <= p < centre + N or centre <= q < centre + N:
            if -1 in rv:
                continue
            a = vor.vertices[rv[0]]
            b = vor.vertices[rv[1]]
            if np.linalg.norm(a - b) < 1e-12:
                continue  # zero-length ridge: degenerate contact
            if centre <= p < centre + N:
                ref.add((p - centre, q % N))
            if centre <= q < centre + N:
                ref.add((q - centre, p % N))
    got = {(i, int(F["nbr"][k])) for i in range(N) for k in range(F["rowptr"][i], F["rowptr"][i + 1])}
    assert got == ref
    for i in range(N):
        region = vor.regions[vor.point_region[centre + i]]
        poly = vor.vertices[region]
        xs_, ys_ = poly[:, 0], poly[:, 1]
        area = 0.5 * abs(np.dot(xs_, np.roll(ys_, 1)) - np.dot(ys_, np.roll(xs_, 1)))
        assert abs(area - E["area"][i]) <= 1e-12 * area
    assert abs(E["area"].sum() - 1.0) < 1e-12
