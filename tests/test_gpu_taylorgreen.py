"""The reference's own test (tests/taylorgreen.jl:112-114) run through the GPU
path: E_err < 1e-8, v_err < 0.01, P_err < 0.01 after t = 0.1, with the FP64
Jacobi-PCG at 1e-8."""
import pytest

import tg_reference as TG

pytestmark = pytest.mark.gpu


def test_taylorgreen_thresholds_gpu(lv):
    from lvgpu import populate as pop
    x = pop.hex_seeds((0.0, 1.0), (0.0, 1.0), TG.dr)
    g = lv.VoronoiGrid(lv.Rectangle((0, 1), (0, 1)), TG.dr, xperiodic=True, yperiodic=True)
    g.push(x)
    lv.remesh(g)
    for k, v in TG.initial_state(x, g["area"]).items():
        g[k] = v
    solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)

    def step(t):
        lv.move(g, TG.dt)
        lv.stiffened_eos(g, TG.gamma, TG.P0)
        lv.find_pressure(solver, TG.dt, 10, stats=False)
        lv.pressure_step(g, TG.dt)
        lv.find_D(g)
        lv.viscous_step(g, TG.dt, False)
        lv.find_dv(g, TG.dt)
        lv.relaxation_step(g, TG.dt)

    def fields():
        g.synchronize()
        return g["x"], g["area"], g["v"], g["P"], g["mass"], g["e"]

    E_err, v_err, P_err, steps = TG.run(step, fields)
    print("GPU TG:", E_err, v_err, P_err)
    assert steps == 80
    assert E_err < 1e-8 and abs(E_err) < 1e-10
    assert v_err < 0.01
    assert P_err < 0.01
