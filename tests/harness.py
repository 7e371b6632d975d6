"""Builds matched GPU / oracle grids from the same seeds and applies the
reference's operations to both."""
import os

import numpy as np

import workloads as W

ORDER_FIELDS = ["x", "v", "e", "P", "rho", "c2", "dv", "mass", "momentum", "energy", "phase", "quality", "D", "mu"]


def seeds(pop, flow, seed=12345, jitter=0.1):
    return pop.jittered_lattice(flow.xlims, flow.ylims, flow.nx, flow.ny, jitter, seed)


def sweep_guess_on():
    """Whether the GPU's find_pressure starts sweeps from the line-searched guess."""
    return os.environ.get("LVGPU_SWEEP_GUESS", "1") != "0"


def make_gpu(lv, flow, x):
    grid = lv.VoronoiGrid(lv.Rectangle(flow.xlims, flow.ylims), flow.dr, xperiodic=flow.periodic,
                          yperiodic=flow.periodic)
    grid.push(x)
    lv.remesh(grid)
    return grid


def make_oracle(oracle, flow, x):
    og = oracle.OracleGrid(flow.xlims, flow.ylims, flow.dr, len(x), xperiodic=flow.periodic,
                           yperiodic=flow.periodic, max_edges=20)
    og.set("x", x)
    st = og.remesh()
    assert st == 0, st
    return og


def init_both(flow, grid, og):
    area = grid["area"]
    x = grid["x"]
    f = W.initial_fields(flow, x, area)
    for k, v in f.items():
        grid[k] = v
        og.set(k, v)
    return f


def copy_state(src_get, dst_set, names=ORDER_FIELDS):
    for k in names:
        dst_set(k, src_get(k))


def apply(lv, flow, target, op, kw, is_gpu, solver=None, tol=1e-8):
    dt = flow.dt
    if op == "move":
        return lv.move(target, dt) if is_gpu else target.move(dt)
    if op == "gravity_step":
        return lv.gravity_step(target, kw["g"], dt) if is_gpu else target.gravity_step(kw["g"], dt)
    if op == "stiffened_eos":
        return (lv.stiffened_eos(target, kw["gamma"], kw["P0"]) if is_gpu
                else target.stiffened_eos(kw["gamma"], kw["P0"]))
    if op == "ideal_eos":
        return lv.ideal_eos(target, kw["gamma"]) if is_gpu else target.ideal_eos(kw["gamma"])
    if op == "find_pressure":
        vbc = wall_table(flow)
        if is_gpu:
            return lv.find_pressure(solver, dt, 10, boundary_velocity=flow.walls or None)
        # the oracle starts the sweeps as the GPU does (line-searched guess
        # unless LVGPU_SWEEP_GUESS=0)
        return target.find_pressure(dt, 10, vbc, method="pcg", tol=tol, guess=sweep_guess_on())
    if op == "pressure_step":
        return lv.pressure_step(target, dt) if is_gpu else target.pressure_step(dt)
    if op == "find_D":
        return lv.find_D(target) if is_gpu else target.find_D()
    if op == "viscous_step":
        av = kw["artificial_viscosity"]
        return lv.viscous_step(target, dt, av) if is_gpu else target.viscous_step(dt, av)
    if op == "bdary_friction":
        if is_gpu:
            return lv.bdary_friction(target, kw["walls"], dt)
        return target.bdary_friction(wall_table(flow, zero_default=True), dt)
    if op == "find_dv":
        return lv.find_dv(target, dt) if is_gpu else target.find_dv(dt)
    if op == "multiphase_projection":
        if is_gpu:
            return lv.multiphase_projection(lv.MultiphaseSolver(target))
        return target.multiphase_projection()
    if op == "relaxation_step":
        return lv.relaxation_step(target, dt) if is_gpu else target.relaxation_step(dt)
    raise ValueError(op)


def wall_table(flow, zero_default=False):
    t = np.zeros((4, 2))
    if not flow.walls:
        return t.reshape(8) if zero_default else None
    for lab, v in flow.walls.items():
        t[-lab - 1] = v
    return t.reshape(8)
