"""The oracle's per-edge boundary values (the reference's closures evaluated
at each boundary edge's midpoint) against its label table: the same values
give the same right-hand side and friction bit for bit, and a charfun that
excludes every edge leaves the friction a no-op."""
import numpy as np

import harness as H
import workloads as W


def _grid(oracle):
    from importlib import util
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = util.spec_from_file_location("pop_o", os.path.join(root, "lagrangianvoronoi.jl_gb300", "populate.py"))
    pop = util.module_from_spec(spec)
    spec.loader.exec_module(pop)
    flow = W.cavity(24)
    og = H.make_oracle(oracle, flow, H.seeds(pop, flow))
    for k, v in W.initial_fields(flow, og.get("x"), og.edges()["area"]).items():
        og.set(k, v)
    og.set("v", 0.1 * np.sin(5.0 * og.get("x")))
    og.set("mu", np.full(len(og.get("e")), 1e-3))
    return flow, og


def test_per_edge_values_match_the_label_table(oracle):
    table = np.array([1.0, 0.0, 0.0, 0.0, 0.0, 0.3, 0.0, 0.0])  # UP (1, 0), DOWN (0, 0.3)
    out = []
    for per_edge in (False, True):
        flow, og = _grid(oracle)
        og.pressure_operator(flow.dt)
        if per_edge:
            mid, lab = og.boundary_edges()
            assert len(mid) > 0 and np.all(lab < 0)
            og.set_edge_values(table.reshape(4, 2)[-lab - 1])
            b, _ = og.pressure_rhs(flow.dt, 0, None)
            og.bdary_friction(np.zeros(8), flow.dt)
        else:
            b, _ = og.pressure_rhs(flow.dt, 0, table)
            og.bdary_friction(table, flow.dt)
        out.append((b, og.get("v"), og.get("e")))
    for a, c in zip(*out):
        assert np.array_equal(a, c)


def test_charfun_excluding_every_edge(oracle):
    flow, og = _grid(oracle)
    v0, e0 = og.get("v"), og.get("e")
    mid, _ = og.boundary_edges()
    og.set_edge_values(np.ones((len(mid), 2)), np.zeros(len(mid), np.uint8))
    og.bdary_friction(np.zeros(8), flow.dt)
    assert np.array_equal(og.get("v"), v0) and np.array_equal(og.get("e"), e0)
