"""The oracle reproduces the reference's own test (tests/taylorgreen.jl) with
the reference's solver settings (MINRES, atol = rtol = 1e-6, itmax = 1000)."""
import os
import importlib.util

import tg_reference as TG

HERE = os.path.dirname(os.path.abspath(__file__))


def _pop():
    spec = importlib.util.spec_from_file_location("populate_tg", os.path.join(HERE, "..", "lagrangianvoronoi.jl_gb300",
                                                                             "populate.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_taylorgreen_thresholds(oracle):
    x = _pop().hex_seeds((0.0, 1.0), (0.0, 1.0), TG.dr)
    g = oracle.OracleGrid((0, 1), (0, 1), TG.dr, len(x), xperiodic=True, yperiodic=True)
    g.set("x", x)
    assert g.remesh() == 0
    for k, v in TG.initial_state(x, g.edges()["area"]).items():
        g.set(k, v)

    def step(t):
        assert g.move(TG.dt) == 0
        g.stiffened_eos(TG.gamma, TG.P0)
        g.find_pressure(TG.dt, 10, None, method="minres", tol=1e-6, itmax=1000)
        g.pressure_step(TG.dt)
        g.find_D()
        g.viscous_step(TG.dt, False)
        g.find_dv(TG.dt)
        assert g.relaxation_step(TG.dt) == 0

    def fields():
        return g.get("x"), g.edges()["area"], g.get("v"), g.get("P"), g.get("mass"), g.get("e")

    E_err, v_err, P_err, steps = TG.run(step, fields)
    assert steps == 80
    assert E_err < 1e-8
    assert v_err < 0.01
    assert P_err < 0.01
    print("oracle TG:", E_err, v_err, P_err)
