"""remesh! on the GPU against the oracle: cell lists, polygons, geometry and
faces must be bit-identical on jittered inputs (src/voronoigrid.jl:89-108)."""
import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

SMALL = {
    "gresho": lambda: W.gresho(50),
    "taylor_green": lambda: W.taylor_green(64),
    "rayleigh_taylor": lambda: W.rayleigh_taylor(32, 64),
    "cavity": lambda: W.cavity(64),
    "double_shear": lambda: W.double_shear(64),
}


def _pair(lv, oracle, flow, seed=12345, jitter=0.1):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, seed, jitter)
    return x, H.make_gpu(lv, flow, x), H.make_oracle(oracle, flow, x)


@pytest.mark.parametrize("name", list(SMALL))
def test_cell_list_bit_exact(lv, oracle, name):
    flow = SMALL[name]()
    x, g, og = _pair(lv, oracle, flow)
    s_gpu, items_gpu = g.cell_list()
    s_ref, items_ref = og.cell_items()
    assert np.array_equal(s_gpu.astype(np.int64), s_ref)
    assert np.array_equal(items_gpu, items_ref)


@pytest.mark.parametrize("name", list(SMALL))
@pytest.mark.parametrize("jitter", [0.0, 0.1, 0.3])
def test_polygons_bit_exact(lv, oracle, name, jitter):
    """jitter 0: the unperturbed lattice, where four seeds share every
    vertex and the clipping meets vertices on the bisector (signum 0)."""
    flow = SMALL[name]()
    x, g, og = _pair(lv, oracle, flow, seed=7, jitter=jitter)
    counts, verts, labels = g.geometry()
    E = og.edges(maxe=20)
    assert E["status"] == 0
    assert np.array_equal(counts, E["counts"])
    for i in range(len(x)):
        k = counts[i]
        assert np.array_equal(labels[i, :k], E["labels"][i, :k]), i
        assert np.array_equal(verts[i, :k], E["verts"][i, :k]), i
    assert np.array_equal(g["area"], E["area"])
    assert np.array_equal(g["centroid"], E["centroid"])
    # the cells tile the domain
    dom = (flow.xlims[1] - flow.xlims[0]) * (flow.ylims[1] - flow.ylims[0])
    assert abs(g["area"].sum() - dom) < 1e-12 * dom


@pytest.mark.parametrize("name", list(SMALL))
def test_faces_bit_exact(lv, oracle, name):
    flow = SMALL[name]()
    x, g, og = _pair(lv, oracle, flow)
    F = g.faces()
    R = og.faces()
    assert np.array_equal(F["rowptr"], R["rowptr"])
    assert np.array_equal(F["nbr"], R["nbr"])
    for key in ("lrr", "mid", "y", "len"):
        assert np.array_equal(F[key], R[key]), key
    # neighbour relation is symmetric on non-degenerate input
    rp, nb = F["rowptr"], F["nbr"]
    pairs = {(i, int(nb[k])) for i in range(len(x)) for k in range(rp[i], rp[i + 1])}
    assert all((j, i) in pairs for (i, j) in pairs)


@pytest.mark.parametrize("periodic", [True, False])
def test_hex_lattice_bit_exact(lv, oracle, periodic):
    """populate_hex! seeds (src/populate.jl:155-179): three cells meet at every
    vertex and the rows are offset by half a spacing."""
    from lvgpu import populate as pop
    flow = W.taylor_green(40) if periodic else W.cavity(40)
    x = pop.hex_seeds(flow.xlims, flow.ylims, flow.dr)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    counts, verts, labels = g.geometry()
    E = og.edges(maxe=20)
    assert E["status"] == 0
    assert np.array_equal(counts, E["counts"])
    for i in range(len(x)):
        k = counts[i]
        assert np.array_equal(labels[i, :k], E["labels"][i, :k]), i
        assert np.array_equal(verts[i, :k], E["verts"][i, :k]), i
    assert np.array_equal(g["area"], E["area"])
    F, R = g.faces(), og.faces()
    for key in ("rowptr", "nbr", "lrr", "mid", "y", "len"):
        assert np.array_equal(F[key], R[key]), key


def test_remesh_after_motion(lv, oracle):
    """Seeds moved by a smooth field (no longer a lattice) still mesh identically."""
    flow = W.taylor_green(48)
    x, g, og = _pair(lv, oracle, flow)
    y = x + 0.3 * flow.dr * np.stack([np.sin(6.0 * x[:, 1]), np.cos(5.0 * x[:, 0])], axis=1)
    y = np.mod(y, 1.0)
    g["x"] = y
    lv.remesh(g)
    og.set("x", y)
    assert og.remesh() == 0
    counts, verts, labels = g.geometry()
    E = og.edges(maxe=20)
    assert np.array_equal(counts, E["counts"])
    assert np.array_equal(g["area"], E["area"])
    assert np.array_equal(g.faces()["nbr"], og.faces()["nbr"])


@pytest.mark.parametrize("name", list(SMALL))
def test_resumed_polygons_bit_exact(lv, oracle, name, monkeypatch):
    """Polygons that outgrow the first clipping pass's edge slots are captured
    and finished by the second pass from the capture.  With a first pass of 5
    slots nearly every polygon takes that route; the mesh must still equal the
    oracle's bit for bit."""
    monkeypatch.setenv("LVGPU_CLIP_SLOTS", "5")
    flow = SMALL[name]()
    x, g, og = _pair(lv, oracle, flow, seed=7, jitter=0.3)
    assert g.clip_captures() > len(x) // 4
    counts, verts, labels = g.geometry()
    E = og.edges(maxe=20)
    assert E["status"] == 0
    assert np.array_equal(counts, E["counts"])
    for i in range(len(x)):
        k = counts[i]
        assert np.array_equal(labels[i, :k], E["labels"][i, :k]), i
        assert np.array_equal(verts[i, :k], E["verts"][i, :k]), i
    F, R = g.faces(), og.faces()
    for key in ("rowptr", "nbr", "lrr", "mid", "y", "len"):
        assert np.array_equal(F[key], R[key]), key
    assert np.array_equal(g["area"], E["area"])
    assert np.array_equal(g["centroid"], E["centroid"])
