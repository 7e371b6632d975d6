"""Seeded workloads shared by the tests: the five benchmark flows at reduced
particle counts, with initial conditions set the way each reference example's
`ic!` does (mass = rho * area after the first remesh)."""
import math

import numpy as np


class Flow:
    """Domain, periodicity, step constants and the analytic initial fields."""

    def __init__(self, name, xlims, ylims, periodic, nx, ny, dt, **kw):
        self.name, self.xlims, self.ylims, self.periodic = name, xlims, ylims, periodic
        self.nx, self.ny, self.dt = nx, ny, dt
        self.dr = (xlims[1] - xlims[0]) / nx
        self.__dict__.update(kw)


def gresho(n=50):
    # periodic unit square centred vortex (examples/gresho.jl:46-62), incompressible
    return Flow("gresho", (0.0, 1.0), (0.0, 1.0), True, n, n, 1e-3, eos=None, gamma=1.4, mu=0.0,
                artificial_viscosity=True, walls=None)


def taylor_green(n=256):
    # stiffened EOS with c0 = 50 as in tests/taylorgreen.jl:9-20
    c0, gamma = 50.0, 1.4
    return Flow("taylor_green", (0.0, 1.0), (0.0, 1.0), True, n, n, 5e-4, eos="stiffened", gamma=gamma,
                P0=c0 * c0 / gamma, mu=0.01, artificial_viscosity=False, walls=None)


def rayleigh_taylor(nx=512, ny=1024):
    return Flow("rayleigh_taylor", (0.0, 0.5), (0.0, 1.0), False, nx, ny, 0.1 * (0.5 / nx), eos="ideal",
                gamma=1.4, c=20.0, g=1.0, Re=420.0, artificial_viscosity=True, walls={})


def cavity(n=1024):
    dr = 1.0 / n
    Re = 1000.0
    return Flow("cavity", (0.0, 1.0), (0.0, 1.0), False, n, n, min(0.1 * dr, 0.1 * Re * dr * dr), eos=None,
                gamma=1.4, mu=1.0 / Re, artificial_viscosity=False, walls={-1: (1.0, 0.0)})


def double_shear(n=2048):
    gamma = 1.4
    dr = 1.0 / n
    return Flow("double_shear", (0.0, 1.0), (0.0, 1.0), True, n, n, 0.1 * dr / 2.0, eos="ideal", gamma=gamma,
                P0=100.0 / gamma, mu=1e-4, artificial_viscosity=True, walls=None)


FLOWS = {"gresho": gresho, "taylor_green": taylor_green, "rayleigh_taylor": rayleigh_taylor, "cavity": cavity,
         "double_shear": double_shear}


def initial_fields(flow, x, area):
    """Initial state arrays given seed positions x[n][2] and cell areas."""
    n = len(x)
    X, Y = x[:, 0], x[:, 1]
    f = {}
    rho = np.ones(n)
    v = np.zeros((n, 2))
    P = np.zeros(n)
    phase = np.zeros(n)
    mu = np.full(n, getattr(flow, "mu", 0.0))
    c2 = np.zeros(n)
    if flow.name == "gresho":
        dx, dy = X - 0.5, Y - 0.5
        r = np.sqrt(dx * dx + dy * dy)
        om = np.where(r < 0.2, 5.0, np.where(r < 0.4, 2.0 / np.maximum(r, 1e-300) - 5.0, 0.0))
        v = np.stack([-om * dy, om * dx], axis=1)
        P = np.where(r < 0.2, 12.5 * r * r,
                     np.where(r < 0.4, 4.0 + 4.0 * np.log(5.0 * np.maximum(r, 1e-300)) - 20.0 * r + 12.5 * r * r,
                              -2.0 + 4.0 * math.log(2.0)))
        c2[:] = np.inf
    elif flow.name == "taylor_green":
        tp = 2.0 * math.pi
        v = np.stack([np.sin(tp * X) * np.cos(tp * Y), -np.cos(tp * X) * np.sin(tp * Y)], axis=1)
        P = flow.P0 + 0.25 * (np.cos(2 * tp * X) + np.cos(2 * tp * Y))
    elif flow.name == "rayleigh_taylor":
        dy = 0.5 + 0.01 * np.cos(4.0 * math.pi * X)
        phase = np.where(Y > dy, 0.0, 1.0)
        rho = np.where(phase == 0.0, 2.0, 1.0)
        mu = rho / flow.Re
        P = 1.0 * flow.c ** 2 / flow.gamma - np.maximum(Y, dy) * 1.0 * flow.g - np.minimum(0.0, Y - dy) * 2.0 * flow.g
    elif flow.name == "cavity":
        c2[:] = np.inf
    elif flow.name == "double_shear":
        u = np.where(Y <= 0.5, np.tanh(80.0 * (Y - 0.25)), np.tanh(80.0 * (0.75 - Y)))
        v = np.stack([u, 0.05 * np.sin(2.0 * math.pi * X)], axis=1)
        P = np.full(n, flow.P0)
    g = flow.gamma
    e = 0.5 * np.sum(v * v, axis=1) + (P / (rho * (g - 1.0)) if flow.eos else 0.0)
    if flow.name == "rayleigh_taylor":
        e = P / (rho * (g - 1.0)) + flow.g * Y
    f.update(v=v, rho=rho, mass=rho * area, P=P, e=e, mu=mu, phase=phase)
    if flow.eos is None:
        f["c2"] = c2
    return f


def step_sequence(flow):
    """The reference's step! for each flow, as (operation, kwargs) pairs:
    gresho.jl:100-114, tests/taylorgreen.jl:61-71, rayleightaylor.jl:90-102,
    cavity.jl:70-80, doubleshear.jl:48-58."""
    dt = flow.dt
    seq = [("move", {})]
    if flow.name == "rayleigh_taylor":
        seq.append(("gravity_step", {"g": (0.0, -flow.g)}))
    if flow.eos == "stiffened":
        seq.append(("stiffened_eos", {"gamma": flow.gamma, "P0": flow.P0}))
    elif flow.eos == "ideal":
        seq.append(("ideal_eos", {"gamma": flow.gamma}))
    seq += [("find_pressure", {}), ("pressure_step", {}), ("find_D", {}),
            ("viscous_step", {"artificial_viscosity": flow.artificial_viscosity})]
    if flow.walls is not None and flow.name in ("cavity", "rayleigh_taylor"):
        seq.append(("bdary_friction", {"walls": flow.walls}))
    seq.append(("find_dv", {}))
    if flow.name == "rayleigh_taylor" and getattr(flow, "multiphase", True):
        seq.append(("multiphase_projection", {}))
    seq.append(("relaxation_step", {}))
    return dt, seq
