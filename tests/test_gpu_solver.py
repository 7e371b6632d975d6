"""Pressure operator assembly (CSR) and the FP64 Jacobi-PCG on the GPU
against the oracle (src/pressure.jl:104-224)."""
import ctypes as C

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu


def _setup(lv, oracle, flow, seed=5):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, seed)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    if flow.eos == "stiffened":
        lv.stiffened_eos(g, flow.gamma, flow.P0)
        og.stiffened_eos(flow.gamma, flow.P0)
    elif flow.eos == "ideal":
        lv.ideal_eos(g, flow.gamma)
        og.ideal_eos(flow.gamma)
    return g, og


def _export(lv, g):
    L = lv._lib.load()
    nnz = C.c_int64()
    assert L.lv_export_system(g._ctx, C.byref(nnz), None, None, None, None, None) == 0
    n = g.n
    diag = np.zeros(n)
    rowptr = np.zeros(n + 1, np.int64)
    col = np.zeros(nnz.value, np.int32)
    w = np.zeros(nnz.value)
    b = np.zeros(n)
    p = lv._lib.ptr
    assert L.lv_export_system(g._ctx, None, p(diag), p(rowptr, C.c_int64), p(col, C.c_int32), p(w), p(b)) == 0
    return dict(diag=diag, rowptr=rowptr, col=col, w=w, b=b)


FLOWS = [lambda: W.taylor_green(64), lambda: W.cavity(48), lambda: W.double_shear(64), lambda: W.gresho(50)]


@pytest.mark.parametrize("mk", FLOWS)
def test_operator_csr_bit_exact(lv, oracle, mk):
    flow = mk()
    g, og = _setup(lv, oracle, flow)
    L = lv._lib.load()
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    S = _export(lv, g)
    R = og.pressure_operator(flow.dt)
    assert np.array_equal(S["rowptr"], R["rowptr"])
    assert np.array_equal(S["col"], R["col"])
    assert np.array_equal(S["w"], R["w"])
    assert np.array_equal(S["diag"], R["diag"])


@pytest.mark.parametrize("mk", FLOWS)
@pytest.mark.parametrize("gp", [0, 1])
def test_rhs_bit_exact(lv, oracle, mk, gp):
    flow = mk()
    g, og = _setup(lv, oracle, flow)
    L = lv._lib.load()
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    vbc = H.wall_table(flow)
    p = lv._lib.ptr
    assert L.lv_pressure_rhs(g._ctx, flow.dt, gp, p(vbc)) == 0
    S = _export(lv, g)
    og.pressure_operator(flow.dt)
    b, gpv = og.pressure_rhs(flow.dt, gp, vbc)
    assert np.array_equal(S["b"], b)


@pytest.mark.parametrize("mk", FLOWS)
def test_operator_apply(lv, oracle, mk):
    """CSR form adiag x - sum w x_j equals the reference's diag x + sum w (x_i - x_j)
    up to rounding of the row's terms."""
    flow = mk()
    g, og = _setup(lv, oracle, flow)
    L = lv._lib.load()
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    A = og.pressure_operator(flow.dt)
    xv = np.random.default_rng(1).standard_normal(g.n)
    y = np.zeros(g.n)
    p = lv._lib.ptr
    assert L.lv_operator_apply(g._ctx, p(xv), p(y)) == 0
    yr = og.operator_apply(xv)
    rp = A["rowptr"]
    scale = np.abs(A["diag"] * xv)
    for i in range(g.n):
        ws, cs = A["w"][rp[i]:rp[i + 1]], A["col"][rp[i]:rp[i + 1]]
        scale[i] += np.sum(np.abs(ws) * (np.abs(xv[i]) + np.abs(xv[cs])))
    assert np.all(np.abs(y - yr) <= 1e-14 * scale * 16)


@pytest.mark.parametrize("mk", FLOWS)
def test_pcg_solution(lv, oracle, mk):
    """GPU Jacobi-PCG reaches ||b - A x|| <= 1e-8 ||b|| (checked with the
    oracle's operator in FP64) in about as many iterations as the oracle's PCG."""
    flow = mk()
    g, og = _setup(lv, oracle, flow)
    L = lv._lib.load()
    dt = flow.dt
    assert L.lv_pressure_operator(g._ctx, dt) == 0
    og.pressure_operator(dt)
    b, _ = og.pressure_rhs(dt, 0, H.wall_table(flow))
    singular = not np.any(og.pressure_operator(dt)["diag"] != 0)
    bp = b - b.mean() if singular else b
    x0 = og.get("P").copy()
    solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)
    solver.configure()
    xg = x0.copy()
    st = lv.LvSolveStats()
    p = lv._lib.ptr
    assert L.lv_solve(g._ctx, p(b), p(xg), C.byref(st)) == 0
    r = bp - og.operator_apply(xg)
    rel = np.linalg.norm(r) / np.linalg.norm(bp)
    assert st.converged == 1
    assert rel <= 1.5e-8, rel
    assert abs(st.rel_residual - rel) <= 1e-9
    xr, (it_ref, conv_ref, rel_ref) = og.solve(b, x0, method="pcg", tol=1e-8)
    assert abs(st.iterations - it_ref) <= 3, (st.iterations, it_ref)
    d = xg - xr
    if singular:
        d = d - d.mean()
    assert np.linalg.norm(d) <= 1e-5 * max(np.linalg.norm(xr - (xr.mean() if singular else 0)), 1e-30)


@pytest.mark.parametrize("guess", ["0", "1"])
@pytest.mark.parametrize("mk", FLOWS)
def test_find_pressure_sweeps(lv, oracle, mk, guess, monkeypatch):
    """The sweeps match the oracle's sweep for sweep, iteration counts
    included: with the plain warm start (the previous sweep's P) and with the
    line-searched guess."""
    monkeypatch.setenv("LVGPU_SWEEP_GUESS", guess)
    flow = mk()
    g, og = _setup(lv, oracle, flow)
    solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)
    st = lv.find_pressure(solver, flow.dt, 10, boundary_velocity=flow.walls or None)
    ref = og.find_pressure(flow.dt, 10, H.wall_table(flow), method="pcg", tol=1e-8, guess=guess == "1")
    assert all(s[1] for s in st), st
    assert all(s[2] <= 1.5e-8 for s in st), st
    P, Pr = g["P"], og.get("P")
    singular = flow.name in ("gresho", "cavity")
    if singular:
        P, Pr = P - P.mean(), Pr - Pr.mean()
    assert np.linalg.norm(P - Pr) <= 1e-5 * np.linalg.norm(Pr)
    for rec, refrec in zip(st, ref):
        assert abs(rec[0] - refrec[0]) <= max(3, 0.05 * refrec[0]), (st, ref)


@pytest.mark.parametrize("mk", FLOWS)
def test_find_pressure_sweep_guess(lv, oracle, mk, monkeypatch):
    """With the line-searched initial guess (the default) every sweep still
    meets the FP64 residual 1e-8, P agrees with the oracle's plain sweeps to
    the solver tolerance, and the sweeps need no more CG iterations in total
    than with the plain warm start (the guess never increases the A-norm of
    the initial error; CG's count can still move by an iteration or two)."""
    flow = mk()
    runs = {}
    for guess in ("0", "1"):
        monkeypatch.setenv("LVGPU_SWEEP_GUESS", guess)
        g, og = _setup(lv, oracle, flow)
        solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)
        runs[guess] = (g, og, lv.find_pressure(solver, flow.dt, 10, boundary_velocity=flow.walls or None))
    g, og, st = runs["1"]
    ref = og.find_pressure(flow.dt, 10, H.wall_table(flow), method="pcg", tol=1e-8)
    assert all(s[1] for s in st), st
    assert all(s[2] <= 1.5e-8 for s in st), st
    P, Pr = g["P"], og.get("P")
    if flow.name in ("gresho", "cavity"):
        P, Pr = P - P.mean(), Pr - Pr.mean()
    assert np.linalg.norm(P - Pr) <= 1e-5 * np.linalg.norm(Pr)
    it_guess = sum(s[0] for s in st)
    it_plain = sum(s[0] for s in runs["0"][2])
    assert it_guess <= 1.02 * it_plain + 2, (it_guess, it_plain, st, runs["0"][2])
