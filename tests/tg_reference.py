"""The reference's own test, tests/taylorgreen.jl: periodic Taylor-Green
vortex, N = 80, hexagonal seeds (populate_hex!), Re = 400, dt = 0.1 dr,
stiffened gas c0 = 50, t_end = 0.1, run! with nframes = 20; it asserts
E_err < 1e-8, v_err < 0.01 and P_err < 0.01 after the last frame
(tests/taylorgreen.jl:112-114)."""
import math

import numpy as np

rho0, N, Re, c0, gamma = 1.0, 80, 400.0, 50.0, 1.4
dr = 1.0 / N
dt = 0.1 * dr
t_end = 0.1
P0 = rho0 * c0 ** 2 / gamma
nframes = 20


def v_max(t):
    return math.exp(-8.0 * math.pi ** 2 * t / Re)


def v_exact(x, t):
    tp = 2.0 * math.pi
    u0 = np.cos(tp * x[:, 0]) * np.sin(tp * x[:, 1])
    v0 = -np.sin(tp * x[:, 0]) * np.cos(tp * x[:, 1])
    return v_max(t) * np.stack([u0, v0], axis=1)


def P_exact(x, t):
    tp = 2.0 * math.pi
    return 0.5 * v_max(t) ** 2 * (np.sin(tp * x[:, 0]) ** 2 + np.sin(tp * x[:, 1]) ** 2 - 1.0)


def initial_state(x, area):
    v = v_exact(x, 0.0)
    P = P_exact(x, 0.0)
    return dict(v=v, rho=np.full(len(x), rho0), mass=rho0 * area, P=P,
                e=0.5 * np.sum(v * v, axis=1) + P / (rho0 * (gamma - 1.0)), mu=np.full(len(x), 1.0 / Re))


def errors(x, area, v, P, mass, e, t):
    p_avg = np.sum(area * P)
    E = np.sum(mass * e)
    v_err = math.sqrt(np.sum(area * np.sum((v - v_exact(x, t)) ** 2, axis=1)))
    P_err = math.sqrt(np.sum(area * (P - p_avg - P_exact(x, t)) ** 2))
    return E, v_err, P_err


def run(step, fields):
    """run!(sim, dt, t_end, step!; nframes) with the reference's frame logic
    (simulation.jl:59-89); fields() returns (x, area, v, P, mass, e).
    Returns (E_err, v_err, P_err, steps)."""
    k_frame = max(int(round(t_end / (nframes * dt))), 1)
    t, k = 0.0, 0
    E0 = None
    out = None
    while t < t_end:
        k += 1
        step(t)
        if k % k_frame == 0:
            x, area, v, P, mass, e = fields()
            E, v_err, P_err = errors(x, area, v, P, mass, e, t)
            if E0 is None:
                E0 = E
            out = (E - E0, v_err, P_err, k)
        t += dt
    return out
