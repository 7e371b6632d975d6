"""The other implicit and explicit physics of the reference: the implicit
ViscousSolver (viscous_solver.jl:43-129) and Fourier heat conduction
(fourier.jl: ideal_temperature!, fourier_step!, heat_from_bdary!), against
the oracle.

Tolerances: the Fourier operators are explicit FP64 in the reference's
order, so T and e are bit-identical.  The viscous step is a MINRES solve to
atol = rtol = 1e-6 on both sides, whose dot products sum in different
orders: the iteration counts agree within max(2, 3 %) and the velocities to
1e-5 relative."""
import math

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

BAD_ARGUMENT = 6


def _pair(lv, oracle, flow, seed=12345):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, seed)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    return g, og


def _both(g, og, name, values):
    g[name] = values
    og.set(name, values)


@pytest.mark.parametrize("mk", [lambda: W.cavity(48), lambda: W.taylor_green(48)])
def test_viscous_solver_matches_oracle(lv, oracle, mk):
    flow = mk()
    g, og = _pair(lv, oracle, flow)
    n = g.n
    rng = np.random.default_rng(4)
    v0 = rng.standard_normal((n, 2))
    _both(g, og, "v", v0)
    _both(g, og, "mu", 0.05 + 0.05 * rng.random(n))  # a viscosity large enough for the implicit step
    solver = lv.ViscousSolver(g)
    for step in range(3):
        it, conv = lv.viscous_step(solver, flow.dt * 10)
        rit, rconv, _ = og.viscous_solve(flow.dt * 10)
        assert conv and rconv
        assert abs(it - rit) <= max(2, 0.03 * rit), (step, it, rit)
        a, b = g["v"], og.get("v")
        assert np.max(np.abs(a - b)) <= 1e-5 * np.max(np.abs(b)), step
    # the implicit step damps the velocity (a check of the solve, not of parity)
    assert np.linalg.norm(g["v"]) < np.linalg.norm(v0)


def _heat_fields(g, og):
    n = g.n
    x = g["x"]
    rng = np.random.default_rng(9)
    _both(g, og, "cV", 1.0 + 0.5 * rng.random(n))
    _both(g, og, "k", 0.01 * (1.0 + np.sin(3.0 * x[:, 0])))
    _both(g, og, "e", 2.0 + np.cos(4.0 * x[:, 1]) + rng.random(n))
    _both(g, og, "v", 0.3 * rng.standard_normal((n, 2)))
    _both(g, og, "rho", 1.0 + 0.1 * rng.random(n))


def _T_bc(m, label):
    # heated bottom wall varying along it, adiabatic elsewhere (examples/heat.jl's kind of rule)
    return 1.0 + 0.5 * math.sin(3.0 * m[0]) if label == -3 else float("nan")


def test_fourier_bit_exact(lv, oracle):
    flow = W.cavity(40)
    g, og = _pair(lv, oracle, flow)
    _heat_fields(g, og)
    dt = 1e-3
    mid, lab = og.boundary_edges()
    Tb = [_T_bc(m, int(l)) for m, l in zip(mid, lab)]
    for _ in range(10):  # examples/heat.jl:94-96, repeated
        lv.ideal_temperature(g)
        og.ideal_temperature()
        assert np.array_equal(g["T"], og.get("T"))
        lv.fourier_step(g, dt)
        og.fourier_step(dt)
        assert np.array_equal(g["e"], og.get("e"))
        lv.heat_from_bdary(g, dt, _T_bc, 1.4)
        assert og.heat_from_bdary(dt, Tb) == 0
        assert np.array_equal(g["T"], og.get("T"))
        assert np.array_equal(g["e"], og.get("e"))
    assert np.any(g["T"] != 0.0)


def test_heat_from_bdary_asserts_cV(lv, oracle):
    flow = W.cavity(24)
    g, og = _pair(lv, oracle, flow)
    _heat_fields(g, og)
    cV = g["cV"]
    cV[0] = 0.0  # polygon 0 sits in a corner: a boundary polygon
    _both(g, og, "cV", cV)
    with pytest.raises(lv.LvError) as ei:
        lv.heat_from_bdary(g, 1e-3, _T_bc)
        g.synchronize()
    assert ei.value.code == BAD_ARGUMENT
    mid, lab = og.boundary_edges()
    assert og.heat_from_bdary(1e-3, [_T_bc(m, int(l)) for m, l in zip(mid, lab)]) == BAD_ARGUMENT
