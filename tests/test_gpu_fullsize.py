"""Every benchmark flow at its full size (2,500 to 4,194,304 particles), one
reference step! on the GPU, checked through properties that hold at any
size: the cells tile the domain, every face lies on the bisector of its two
seeds, the neighbour relation is symmetric, relaxation conserves mass, the
pressure sweeps meet the FP64 residual 1e-8, and the state stays finite.
(The oracle finishes these sizes too slowly; the reduced sizes of
test_gpu_step.py compare against it directly.)"""
import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

FULL = [
    ("gresho", lambda: W.gresho(50)),
    ("taylor_green", lambda: W.taylor_green(256)),
    ("rayleigh_taylor", lambda: W.rayleigh_taylor(512, 1024)),
    ("cavity", lambda: W.cavity(1024)),
    ("double_shear", lambda: W.double_shear(2048)),
]


def _mesh_properties(g, flow, rng, samples=2000):
    x = g["x"]
    n = len(x)
    area = g["area"]
    dom = (flow.xlims[1] - flow.xlims[0]) * (flow.ylims[1] - flow.ylims[0])
    assert np.all(area > 0)
    assert abs(area.sum() - dom) <= 1e-10 * dom
    F = g.faces()
    rp, nb = F["rowptr"], F["nbr"]
    counts = np.diff(rp)
    # interior faces: at least 3 per cell of a periodic domain, 2 in a corner of a walled one
    assert counts.min() >= (3 if flow.periodic else 2) and counts.max() <= 20
    # symmetric neighbour relation: the (i, j) pairs equal the (j, i) pairs
    rows = np.repeat(np.arange(n, dtype=np.int64), counts)
    a = rows * n + nb.astype(np.int64)
    b = nb.astype(np.int64) * n + rows
    assert np.array_equal(np.sort(a), np.sort(b))
    # each face of a sample lies on the perpendicular bisector of x_i and its
    # neighbour image y: the face midpoint is equidistant from both
    idx = rng.choice(len(nb), size=min(samples, len(nb)), replace=False)
    xi = x[rows[idx]]
    y = F["y"][idx]
    m = F["mid"][idx]
    d1 = np.linalg.norm(m - xi, axis=1)
    d2 = np.linalg.norm(m - y, axis=1)
    assert np.max(np.abs(d1 - d2)) <= 1e-10 * flow.dr + 1e-14
    # and y is the neighbour's seed, up to a period shift
    xj = x[nb[idx]]
    shift = y - xj
    if flow.periodic:
        per = np.array([flow.xlims[1] - flow.xlims[0], flow.ylims[1] - flow.ylims[0]])
        shift = shift - per * np.round(shift / per)
    assert np.max(np.abs(shift)) <= 1e-12


@pytest.mark.parametrize("name,mk", FULL)
def test_full_size_step(lv, name, mk):
    from lvgpu import populate as pop
    flow = mk()
    rng = np.random.default_rng(0)
    x = H.seeds(pop, flow)
    g = H.make_gpu(lv, flow, x)
    for k, v in W.initial_fields(flow, g["x"], g["area"]).items():
        g[k] = v
    _mesh_properties(g, flow, rng)
    mass0 = g["mass"].sum()
    solver = lv.PressureSolver(g, method="mixed_ir", tol=1e-8, itmax=40000)
    dt, seq = W.step_sequence(flow)
    stats = None
    for op, kw in seq:
        r = H.apply(lv, flow, g, op, kw, True, solver=solver)
        if op == "find_pressure":
            stats = r
    g.synchronize()
    assert stats is not None and len(stats) == 10
    for it, conv, rel, method, outer in stats:
        assert conv and rel <= 1e-8, (it, rel, outer)
    for k in ("x", "v", "e", "P", "mass"):
        assert np.all(np.isfinite(g[k])), k
    # relaxation_step! remaps conservatively (relaxation.jl:36-73)
    assert abs(g["mass"].sum() - mass0) <= 1e-12 * abs(mass0)
    _mesh_properties(g, flow, rng)
