"""The allocation-free solve, lv_pcg_solve_noalloc.

Some callers of this library cannot allocate device memory: a host that
reserves all device memory for its own allocator up front, or a time-step
loop that must not stall on cudaMalloc (it synchronises the device).  For
them, lv_pcg_solve_noalloc solves a pressure system they already hold in
device memory, keeping the solver's scratch in a static device array.  This
test checks it against the regular solve (lv_solve) on the same system and
against the oracle's solution of that system, two calls in a row, at the
tolerance the other solver tests use.  The operator is the one
lv_export_system returns, with its int64 rowptr narrowed to the int32 this
entry point takes.  It lives in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu


def _system(lv, oracle, flow):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, 11)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    if flow.eos == "stiffened":
        lv.stiffened_eos(g, flow.gamma, flow.P0)
        og.stiffened_eos(flow.gamma, flow.P0)
    L = lv._lib.load()
    p = lv._lib.ptr
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    assert L.lv_pressure_rhs(g._ctx, flow.dt, 0, p(H.wall_table(flow))) == 0
    nnz = C.c_int64()
    assert L.lv_export_system(g._ctx, C.byref(nnz), None, None, None, None, None) == 0
    n = g.n
    diag, rowptr, b = np.zeros(n), np.zeros(n + 1, np.int64), np.zeros(n)
    col, w = np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
    assert L.lv_export_system(g._ctx, None, p(diag), p(rowptr, C.c_int64), p(col, C.c_int32), p(w), p(b)) == 0
    return g, og, dict(diag=diag, rowptr=rowptr, col=col, w=w, b=b, x0=g["P"].copy())


@pytest.mark.parametrize("mk", [lambda: W.taylor_green(64), lambda: W.cavity(48)])
def test_noalloc_solve_matches_regular_solve(lv, oracle, mk):
    import torch
    flow = mk()
    g, og, S = _system(lv, oracle, flow)
    L = lv._lib.load()
    p = lv._lib.ptr
    # the regular entry point on the same system
    solver = lv.PressureSolver(g, method="jacobi_pcg", tol=1e-8)
    solver.configure()
    x_reg = S["x0"].copy()
    st = lv.LvSolveStats()
    assert L.lv_solve(g._ctx, p(S["b"]), p(x_reg), C.byref(st)) == 0
    assert st.converged == 1
    # the caller's device buffers (allocated by the caller, not by the entry point)
    dev = "cuda:0"
    d = {k: torch.from_numpy(S[k]).to(dev) for k in ("diag", "col", "w", "b")}
    d["rowptr"] = torch.from_numpy(S["rowptr"].astype(np.int32)).to(dev)
    xd = torch.empty(g.n, dtype=torch.float64, device=dev)
    singular = not np.any(S["diag"] != 0)
    ref = x_reg - x_reg.mean() if singular else x_reg
    # the oracle's solution of the same system (bit-identical operator and b)
    og.pressure_operator(flow.dt)
    xo, _ = og.solve(S["b"], S["x0"], method="pcg", tol=1e-11)
    ref_o = xo - xo.mean() if singular else xo
    for call in range(2):
        xd.copy_(torch.from_numpy(S["x0"]))
        torch.cuda.synchronize()
        it, rel = C.c_int32(), C.c_double()
        rc = L.lv_pcg_solve_noalloc(g.n, d["diag"].data_ptr(), d["rowptr"].data_ptr(), d["col"].data_ptr(),
                                    d["w"].data_ptr(), d["b"].data_ptr(), xd.data_ptr(), 1e-8, 10000, None,
                                    C.byref(it), C.byref(rel))
        assert rc == 0, (call, rc)
        x = xd.cpu().numpy()
        got = x - x.mean() if singular else x
        assert np.linalg.norm(got - ref) <= 1e-6 * np.linalg.norm(ref), call
        assert np.linalg.norm(got - ref_o) <= 1e-6 * np.linalg.norm(ref_o), call
        # LV_OK means the true residual met the tolerance
        assert rel.value <= 1e-8, (call, rel.value)
        assert abs(it.value - st.iterations) <= 3, (call, it.value, st.iterations)


def test_noalloc_rejects_oversized_system(lv):
    L = lv._lib.load()
    big = 524288 + 1
    rc = L.lv_pcg_solve_noalloc(big, 1, 1, 1, 1, 1, 1, 1e-8, 10, None, None, None)
    assert rc == 6
