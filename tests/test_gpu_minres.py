"""The reference's own pressure solve on the GPU: unpreconditioned FP64
MINRES with atol = rtol = 1e-6 and itmax = 1000, warm-started from P in
every sweep (pressure.jl:215-224; Krylov.jl 0.9.8 minres!).  It is the
default PressureSolver, and it is compared sweep by sweep with the oracle's
MINRES (oracle/lvref.cpp minres_solve, Paige & Saunders 1975).

Tolerances: the two differ only in the summation order of their dot
products, so a sweep's iteration count agrees within max(2, 3 %) (a stopping
test that lands within rounding of the bound can move by one), P agrees to
1e-5 relative after the ten sweeps, and fields after five full steps agree
to 1e-5 relative (the solves stop at an absolute-plus-relative residual of
1e-6, so a sweep that stops one iteration apart moves P by that much).  The
pressure of the incompressible flows is compared modulo its mean."""
import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

FLOWS = [
    ("gresho", lambda: W.gresho(50)),
    ("taylor_green", lambda: W.taylor_green(64)),
    ("rayleigh_taylor", lambda: W.rayleigh_taylor(32, 64)),
    ("cavity", lambda: W.cavity(64)),
    ("double_shear", lambda: W.double_shear(64)),
]


def _pair(lv, oracle, flow):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    return g, og


def _eos(lv, flow, g, og):
    if flow.eos == "stiffened":
        lv.stiffened_eos(g, flow.gamma, flow.P0)
        og.stiffened_eos(flow.gamma, flow.P0)
    elif flow.eos == "ideal":
        lv.ideal_eos(g, flow.gamma)
        og.ideal_eos(flow.gamma)


@pytest.mark.parametrize("name,mk", FLOWS)
def test_minres_sweeps_match_oracle(lv, oracle, name, mk):
    flow = mk()
    g, og = _pair(lv, oracle, flow)
    _eos(lv, flow, g, og)
    # a velocity kick so that every flow's sweeps have work to do
    v = g["v"] + 0.1 * np.sin(7.0 * g["x"][:, ::-1])
    g["v"] = v
    og.set("v", v)
    solver = lv.PressureSolver(g)  # the reference's: MINRES, 1e-6, 1000
    assert (solver.method, solver.tol, solver.itmax) == ("minres", 1e-6, 1000)
    st = lv.find_pressure(solver, flow.dt, 10)
    ref = og.find_pressure(flow.dt, 10, None, method="minres", tol=1e-6, itmax=1000)
    assert all(s[1] for s in st), st
    assert all(s[3] == 3 for s in st), st  # method actually used
    for rec, rr in zip(st, ref):
        assert abs(rec[0] - rr[0]) <= max(2, 0.03 * rr[0]), (st, ref)
    P, Pr = g["P"], og.get("P")
    if flow.eos is None:
        P, Pr = P - P.mean(), Pr - Pr.mean()
    assert np.linalg.norm(P - Pr) <= 1e-5 * max(np.linalg.norm(Pr), 1e-30), np.linalg.norm(P - Pr)


@pytest.mark.parametrize("name,mk", FLOWS)
def test_minres_steps_match_oracle(lv, oracle, name, mk):
    """Five reference step!s with the default solver on both sides."""
    flow = mk()
    g, og = _pair(lv, oracle, flow)
    solver = lv.PressureSolver(g)
    dt, seq = W.step_sequence(flow)
    for _ in range(5):
        for op, kw in seq:
            if op == "find_pressure":
                st = lv.find_pressure(solver, dt, 10, boundary_velocity=flow.walls or None)
                assert all(s[1] for s in st), st
                og.find_pressure(dt, 10, H.wall_table(flow), method="minres", tol=1e-6, itmax=1000)
            else:
                H.apply(lv, flow, g, op, kw, True, solver=solver)
                H.apply(lv, flow, og, op, kw, False)
    g.synchronize()
    tol = 1e-4 if flow.name == "rayleigh_taylor" else 1e-5  # its projection stops at 1e-4 (relaxation.jl:180-206)
    for k in ("x", "v", "P", "mass"):
        a, b = g[k], og.get(k)
        if k == "P" and flow.eos is None:
            a, b = a - a.mean(), b - b.mean()
        scale = flow.dr if k == "x" else max(np.max(np.abs(b)), 1e-30)
        err = np.max(np.abs(a - b)) / scale
        assert err < tol, (k, err)
    assert np.array_equal(g.faces()["nbr"], og.faces()["nbr"])


def test_minres_large_system(lv, oracle):
    """A system above every register-resident solver's size: the same kernel."""
    flow = W.taylor_green(420)
    g, og = _pair(lv, oracle, flow)
    _eos(lv, flow, g, og)
    solver = lv.PressureSolver(g)
    st = lv.find_pressure(solver, flow.dt, 2)
    ref = og.find_pressure(flow.dt, 2, None, method="minres", tol=1e-6, itmax=1000)
    for rec, rr in zip(st, ref):
        assert rec[1] and abs(rec[0] - rr[0]) <= max(2, 0.03 * rr[0]), (st, ref)
