"""Failure statuses of the C ABI, each made to happen without faulting the GPU:

* LV_ERR_BARRIER_TIMEOUT: the solvers' waits on other blocks are bounded;
  lv_set_wait_limit lowers the bound to one clock cycle so the first wait
  runs out, the call reports the timeout, and the next call (default bound)
  converges as usual.  Every persistent solver is driven this way: the FP64
  register-resident and streaming Jacobi-PCG, the register-resident mixed
  and learned solvers, and the streaming mixed solver.
* LV_ERR_CG_MAXITER: itmax = 1.
* LV_ERR_EDGE_OVERFLOW: a seed ringed by 24 seeds has a 24-gon for a cell,
  beyond LV_MAX_EDGES = 20 (the reference's FastVector would grow; this
  layout reports it; the oracle with 20 slots reports it too).
* LV_ERR_CELL_OVERFLOW: the cell list normally holds every seed's periodic
  copies exactly, so it cannot overflow; LVGPU_CELL_ITEMS lowers its
  capacity at context creation to inject the overflow from the host.
NaN velocity (move.jl:24-26) and the destroyed mesh (voronoigrid.jl:63-65)
are covered in test_gpu_ops.py."""
import ctypes as C

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

BARRIER_TIMEOUT, CG_MAXITER, EDGE_OVERFLOW, CELL_OVERFLOW = 11, 5, 3, 4


def _grid(lv, flow, seed=5):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, seed)
    g = H.make_gpu(lv, flow, x)
    for k, v in W.initial_fields(flow, g["x"], g["area"]).items():
        g[k] = v
    if flow.eos == "stiffened":
        lv.stiffened_eos(g, flow.gamma, flow.P0)
    elif flow.eos == "ideal":
        lv.ideal_eos(g, flow.gamma)
    return g


SOLVERS = [
    ("jacobi_pcg", lambda: W.taylor_green(64)),     # k_pcg_reg (FP64, registers)
    ("jacobi_pcg", lambda: W.cavity(300)),          # k_pcg (FP64, streaming)
    ("mixed_ir", lambda: W.taylor_green(64)),       # k_fcg
    ("learned_pcg", lambda: W.taylor_green(128)),   # k_fcg, staged learned mode
    ("mixed_ir", lambda: W.cavity(420)),            # k_big (streaming)
    ("learned_pcg", lambda: W.double_shear(420)),   # k_big, learned
]


@pytest.mark.parametrize("method,mk", SOLVERS)
def test_barrier_timeout_is_reported_and_recovered(lv, method, mk):
    flow = mk()
    g = _grid(lv, flow)
    L = lv._lib.load()
    if method == "learned_pcg":
        assert L.lv_learn_init(g._ctx, 3) == 0
    solver = lv.PressureSolver(g, method=method, tol=1e-8)
    assert L.lv_set_wait_limit(g._ctx, 1) == 0
    with pytest.raises(lv.LvError) as ei:
        lv.find_pressure(solver, flow.dt, 2)
    assert ei.value.code == BARRIER_TIMEOUT
    # the default bound again: the same call converges
    assert L.lv_set_wait_limit(g._ctx, 0) == 0
    g["P"] = np.zeros(g.n)
    st = lv.find_pressure(solver, flow.dt, 2)
    assert all(conv and rel <= 1.5e-8 for _, conv, rel, _, _ in st), st
    assert all(np.isfinite(g["P"]))


@pytest.mark.parametrize("method", ["jacobi_pcg", "mixed_ir"])
def test_cg_maxiter(lv, method):
    flow = W.gresho(48)  # a vortex: the sweeps have work to do (the cavity at rest has b = 0)
    g = _grid(lv, flow)
    L = lv._lib.load()
    n0 = C.c_int64()
    assert L.lv_solver_unconverged(g._ctx, C.byref(n0)) == 0
    solver = lv.PressureSolver(g, method=method, tol=1e-8, itmax=1)
    st = lv.find_pressure(solver, flow.dt, 3)
    # find_pressure! does not throw (the reference leaves Krylov's stats
    # unread): the sweeps report it, and so does the device-side count
    assert not any(conv for _, conv, _, _, _ in st), st
    n1 = C.c_int64()
    assert L.lv_solver_unconverged(g._ctx, C.byref(n1)) == 0
    assert n1.value - n0.value == 3
    # a plain solve reports it as its status
    b = np.random.default_rng(1).standard_normal(g.n)
    b -= b.mean()
    x = np.zeros(g.n)
    stt = lv.LvSolveStats()
    assert L.lv_solve(g._ctx, lv._lib.ptr(b), lv._lib.ptr(x), C.byref(stt)) == CG_MAXITER
    assert stt.converged == 0 and stt.iterations <= 1


def _fan(k=24, r=0.1):
    t = 2.0 * np.pi * np.arange(k) / k
    ring = np.stack([0.5 + r * np.cos(t), 0.5 + r * np.sin(t)], axis=1)
    return np.ascontiguousarray(np.vstack([[0.5, 0.5], ring]))


def test_edge_overflow(lv, oracle):
    # dr = 0.15: r_max = 1.5 covers the large outer cells (their security
    # radius), so the mesh is not reported destroyed
    dr = 0.15
    x = _fan()
    g = lv.VoronoiGrid(lv.Rectangle((0.0, 1.0), (0.0, 1.0)), dr)
    g.push(x)
    with pytest.raises(lv.LvError) as ei:
        lv.remesh(g)
    assert ei.value.code == EDGE_OVERFLOW
    og = oracle.OracleGrid((0.0, 1.0), (0.0, 1.0), dr, len(x), max_edges=20)
    og.set("x", x)
    assert og.remesh() == EDGE_OVERFLOW
    # with fewer seeds on the ring the centre cell fits
    x = _fan(16)
    g = lv.VoronoiGrid(lv.Rectangle((0.0, 1.0), (0.0, 1.0)), dr)
    g.push(x)
    lv.remesh(g)
    counts, _, _ = g.geometry()
    assert counts[0] == 16


def test_cell_overflow(lv, monkeypatch):
    from lvgpu import populate as pop
    flow = W.taylor_green(32)
    x = H.seeds(pop, flow)
    monkeypatch.setenv("LVGPU_CELL_ITEMS", str(len(x) // 2))
    g = lv.VoronoiGrid(lv.Rectangle(flow.xlims, flow.ylims), flow.dr, xperiodic=True, yperiodic=True)
    g.push(x)
    with pytest.raises(lv.LvError) as ei:
        lv.remesh(g)
    assert ei.value.code == CELL_OVERFLOW
    monkeypatch.delenv("LVGPU_CELL_ITEMS")
    g2 = H.make_gpu(lv, flow, x)
    assert abs(g2["area"].sum() - 1.0) < 1e-12
