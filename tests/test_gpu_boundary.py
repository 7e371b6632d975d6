"""Boundary closures evaluated per boundary edge, as the reference does:
find_pressure!'s boundary_velocity(midpoint(e), e.label) (pressure.jl:182)
and bdary_friction!'s vDirichlet(m) with charfun(m) (diffusion.jl:64-79).
The host evaluates the closure at the midpoints lv_get_boundary_edges lists
and passes one value per edge; the oracle takes the same values.  Fields
after the steps agree to 1e-6 relative (Jacobi-PCG at 1e-8 on both sides),
the pressure modulo its mean (incompressible)."""
import math

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu


def _pair(lv, oracle, flow):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    return g, og


def test_boundary_edges_match_oracle(lv, oracle):
    flow = W.cavity(40)
    g, og = _pair(lv, oracle, flow)
    mid, lab = g.boundary_edges()
    rmid, rlab = og.boundary_edges()
    assert len(mid) > 4 * 40 - 8
    assert np.array_equal(mid, rmid) and np.array_equal(lab, rlab)
    assert set(np.unique(lab)) == {-1, -2, -3, -4}


def test_per_edge_table_equivalence(lv, oracle):
    """A closure that returns the label table's value per edge gives the
    label-table result bit for bit."""
    flow = W.cavity(40)
    table = {-1: (1.0, 0.0), -3: (0.0, 0.25)}
    res = []
    for per_edge in (False, True):
        g, og = _pair(lv, oracle, flow)
        g["v"] = 0.1 * np.sin(5.0 * g["x"])
        solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)
        bv = (lambda x, label: table.get(label, (0.0, 0.0))) if per_edge else table
        lv.find_pressure(solver, flow.dt, 3, boundary_velocity=bv)
        vd = (lambda x: (1.0, 0.0) if x[1] > 0.999 else (0.0, 0.0)) if per_edge else {-1: (1.0, 0.0)}
        lv.bdary_friction(g, vd, flow.dt)
        res.append((g["P"], g["v"], g["e"]))
    for a, b in zip(res[0], res[1]):
        assert np.array_equal(a, b)


def _lid(dr):
    # examples/cavity.jl:41-44
    return lambda x: (1.0, 0.0) if math.isclose(x[1], 1.0, abs_tol=0.1 * dr) else (0.0, 0.0)


def test_cavity_lid_rule_and_piston(lv, oracle):
    """The cavity's lid as its example writes it (a rule on the position), a
    time-dependent piston on the bottom wall varying along it, and a charfun
    that limits the friction to the left half."""
    flow = W.cavity(48)
    g, og = _pair(lv, oracle, flow)
    solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)
    lid = _lid(flow.dr)
    charfun = lambda x: x[0] < 0.5
    dt, seq = W.step_sequence(flow)
    for step in range(5):
        t = step * dt

        def piston(x, label, t=t):
            return (0.0, 0.2 * math.sin(40.0 * t + 1.0) * math.sin(math.pi * x[0])) if label == -3 else (0.0, 0.0)

        for op, kw in seq:
            if op == "find_pressure":
                st = lv.find_pressure(solver, dt, 10, boundary_velocity=piston)
                assert all(s[1] for s in st), st
                mid, lab = og.boundary_edges()
                og.set_edge_values([piston(m, int(l)) for m, l in zip(mid, lab)])
                og.find_pressure(dt, 10, None, method="pcg", tol=1e-8, guess=H.sweep_guess_on())
                og.set_edge_values(None)
            elif op == "bdary_friction":
                lv.bdary_friction(g, lid, dt, charfun=charfun)
                mid, _ = og.boundary_edges()
                og.set_edge_values([lid(m) for m in mid], [charfun(m) for m in mid])
                og.bdary_friction(np.zeros(8), dt)
                og.set_edge_values(None)
            else:
                H.apply(lv, flow, g, op, kw, True, solver=solver)
                H.apply(lv, flow, og, op, kw, False)
    g.synchronize()
    for k in ("x", "v", "P", "mass", "e"):
        a, b = g[k], og.get(k)
        if k == "P":
            a, b = a - a.mean(), b - b.mean()
        scale = flow.dr if k == "x" else max(np.max(np.abs(b)), 1e-30)
        err = np.max(np.abs(a - b)) / scale
        assert err < 1e-6, (k, err)
    assert np.array_equal(g.faces()["nbr"], og.faces()["nbr"])


def test_per_edge_count_is_checked(lv):
    flow = W.cavity(24)
    from lvgpu import populate as pop
    g = H.make_gpu(lv, flow, H.seeds(pop, flow))
    L = lv._lib.load()
    mid, _ = g.boundary_edges()
    vb = np.zeros((len(mid) + 1, 2))
    assert L.lv_bdary_friction_edges(g._ctx, len(mid) + 1, lv._lib.ptr(vb), None, 1e-3) == 6
