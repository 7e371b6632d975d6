"""Learned preconditioner: forward values and gradients of the hand-written
tensor-core kernels against a CPU autograd reference (tests/learned_ref.py),
and training on systems the solver produced, then the learned solve on a
held-out system against the Jacobi mixed-precision solve."""
import ctypes as C

import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
import learned_ref as LR  # noqa: E402


def _grid(lv, oracle, flow, seed=3):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, seed)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    if flow.eos == "stiffened":
        lv.stiffened_eos(g, flow.gamma, flow.P0)
    elif flow.eos == "ideal":
        lv.ideal_eos(g, flow.gamma)
    L = lv._lib.load()
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    return g, L


def _export(lv, g, L):
    p = lv._lib.ptr
    nnz = C.c_int64()
    assert L.lv_export_system(g._ctx, C.byref(nnz), None, None, None, None, None) == 0
    n = g.n
    diag, rowptr, b = np.zeros(n), np.zeros(n + 1, np.int64), np.zeros(n)
    col, w = np.zeros(nnz.value, np.int32), np.zeros(nnz.value)
    assert L.lv_export_system(g._ctx, None, p(diag), p(rowptr, C.c_int64), p(col, C.c_int32), p(w), p(b)) == 0
    adiag = diag.copy()
    for i in range(n):
        for k in range(rowptr[i], rowptr[i + 1]):
            adiag[i] += w[k]
    return rowptr, col, w, diag, adiag, b


def _params(L, g, seed, scale=1.0):
    assert L.lv_learn_init(g._ctx, seed) == 0
    npar = L.lv_learn_num_params()
    pr = np.zeros(npar, np.float32)
    assert L.lv_learn_get_params(g._ctx, pr.ctypes.data_as(C.POINTER(C.c_float))) == 0
    # make the readout non-trivial so every parameter gets a gradient
    o, s = LR.OFF["rd"]
    pr[o:o + s] *= 30.0 * scale
    for name in ("ro", "ro2"):
        o, s = LR.OFF[name]
        pr[o:o + s] *= 30.0 * scale
    assert L.lv_learn_set_params(g._ctx, pr.ctypes.data_as(C.POINTER(C.c_float))) == 0
    return pr


@pytest.mark.parametrize("mk", [lambda: W.taylor_green(32), lambda: W.cavity(32)])
def test_forward_matches_reference(lv, oracle, mk):
    flow = mk()
    g, L = _grid(lv, oracle, flow)
    pr = _params(L, g, 11)
    rowptr, col, w, diag, adiag, _ = _export(lv, g, L)
    n, nnz = g.n, len(col)
    gd = np.zeros(n, np.float32)
    gl = np.zeros(nnz, np.float32)
    X = np.zeros((n, 16), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lv_learn_factor(g._ctx, fp(gd), fp(gl), fp(X)) == 0
    rgd, rgl, rX = LR.forward_values(rowptr, col, w, diag, adiag, pr)
    assert np.allclose(X, rX, rtol=1e-6, atol=1e-7)
    assert np.max(np.abs(gd - rgd)) <= 2e-3 * max(1.0, np.max(np.abs(rgd)))
    assert np.max(np.abs(gl - rgl)) <= 2e-3 * max(1e-3, np.max(np.abs(rgl)))
    assert np.max(np.abs(rgl)) > 1e-4  # the off-diagonal readout is exercised


@pytest.mark.parametrize("mk", [lambda: W.taylor_green(32), lambda: W.cavity(32)])
def test_gradient_matches_autograd(lv, oracle, mk):
    flow = mk()
    g, L = _grid(lv, oracle, flow)
    pr = _params(L, g, 5)
    rowptr, col, w, diag, adiag, _ = _export(lv, g, L)
    K = 3
    rng = np.random.default_rng(4)
    probes = np.where(rng.random((K, g.n)) < 0.5, -1.0, 1.0).astype(np.float32)
    loss = C.c_double()
    grad = np.zeros(len(pr), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lv_learn_loss_grad(g._ctx, -1, fp(probes), K, 0, C.byref(loss), fp(grad)) == 0
    rl, rg = LR.loss_and_grad(rowptr, col, w, diag, adiag, pr, probes)
    assert abs(loss.value - rl) <= 1e-3 * abs(rl)
    for name, (o, s) in LR.OFF.items():
        a, b = grad[o:o + s].astype(np.float64), rg[o:o + s]
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 3e-2 * nb + 1e-7, (name, np.linalg.norm(a - b), nb)
    cos = grad.astype(np.float64) @ rg / (np.linalg.norm(grad) * np.linalg.norm(rg))
    assert cos > 0.999, cos


@pytest.mark.parametrize("mk", [lambda: W.taylor_green(32), lambda: W.cavity(32)])
def test_kaporin_gradient_matches_autograd(lv, oracle, mk):
    """The exact FSAI (Kaporin) objective (probes = 0) and its gradient."""
    flow = mk()
    g, L = _grid(lv, oracle, flow)
    pr = _params(L, g, 6, scale=0.3)
    rowptr, col, w, diag, adiag, _ = _export(lv, g, L)
    loss = C.c_double()
    grad = np.zeros(len(pr), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lv_learn_loss_grad(g._ctx, -1, None, 0, 0, C.byref(loss), fp(grad)) == 0
    rl, rg = LR.loss_and_grad(rowptr, col, w, diag, adiag, pr, None)
    assert abs(loss.value - rl) <= 1e-4 * max(1.0, abs(rl)), (loss.value, rl)
    for name, (o, s) in LR.OFF.items():
        a, b = grad[o:o + s].astype(np.float64), rg[o:o + s]
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 3e-2 * nb + 1e-6, (name, np.linalg.norm(a - b), nb)
    cos = grad.astype(np.float64) @ rg / (np.linalg.norm(grad) * np.linalg.norm(rg))
    assert cos > 0.999, cos


def test_kaporin_gradient_many_tiles_is_deterministic(lv, oracle):
    """Above 608 x 128 rows a block of the backward layer accumulates dW over
    several 128-row tiles in tensor memory (Taylor-Green 300 x 300: 704 tiles).
    The gradient still matches autograd, and two evaluations are bit-identical:
    every partial sum of the backward adds in a fixed order."""
    flow = W.taylor_green(300)
    g, L = _grid(lv, oracle, flow)
    assert g.n > 608 * 128
    pr = _params(L, g, 6, scale=0.3)
    rowptr, col, w, diag, adiag, _ = _export(lv, g, L)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    out = []
    for _ in range(2):
        loss = C.c_double()
        grad = np.zeros(len(pr), np.float32)
        assert L.lv_learn_loss_grad(g._ctx, -1, None, 0, 0, C.byref(loss), fp(grad)) == 0
        out.append((loss.value, grad))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    loss, grad = out[0]
    rl, rg = LR.loss_and_grad(rowptr, col, w, diag, adiag, pr, None)
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl)), (loss, rl)
    for name, (o, s) in LR.OFF.items():
        a, b = grad[o:o + s].astype(np.float64), rg[o:o + s]
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 3e-2 * nb + 1e-6, (name, np.linalg.norm(a - b), nb)
    cos = grad.astype(np.float64) @ rg / (np.linalg.norm(grad) * np.linalg.norm(rg))
    assert cos > 0.999, cos


def _factor2(lv, g, L):
    nnz2 = C.c_int64()
    assert L.lv_learn_factor2(g._ctx, C.byref(nnz2), None, None, None) == 0
    rp2 = np.zeros(g.n + 1, np.int64)
    col2 = np.zeros(nnz2.value, np.int32)
    g2 = np.zeros(nnz2.value, np.float32)
    assert L.lv_learn_factor2(g._ctx, None, lv._lib.ptr(rp2, C.c_int64), lv._lib.ptr(col2, C.c_int32),
                              g2.ctypes.data_as(C.POINTER(C.c_float))) == 0
    return rp2, col2, g2


@pytest.mark.parametrize("mk", [lambda: W.taylor_green(24), lambda: W.cavity(24)])
def test_two_hop_forward_matches_reference(lv, oracle, mk):
    """The two-hop pattern (enumeration order, path weights) and its readout."""
    flow = mk()
    g, L = _grid(lv, oracle, flow)
    assert L.lv_learn_set_pattern(g._ctx, 2) == 0
    pr = _params(L, g, 12)
    rowptr, col, w, diag, adiag, _ = _export(lv, g, L)
    n, nnz = g.n, len(col)
    gd = np.zeros(n, np.float32)
    gl = np.zeros(nnz, np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lv_learn_factor(g._ctx, fp(gd), fp(gl), None) == 0
    rp2, col2, g2 = _factor2(lv, g, L)
    rgd, rgl, _, (rrp2, rcol2, rg2) = LR.forward_values(rowptr, col, w, diag, adiag, pr, hops=2)
    assert np.array_equal(rp2, rrp2) and np.array_equal(col2, rcol2)
    assert np.max(np.abs(gd - rgd)) <= 2e-3 * max(1.0, np.max(np.abs(rgd)))
    assert np.max(np.abs(g2 - rg2)) <= 2e-3 * max(1e-3, np.max(np.abs(rg2)))
    assert np.max(np.abs(rg2)) > 1e-5  # the two-hop readout is exercised
    # symmetric pattern: (i, j) present iff (j, i) is
    rows = np.repeat(np.arange(n), np.diff(rp2))
    assert set(zip(rows.tolist(), col2.tolist())) == set(zip(col2.tolist(), rows.tolist()))


@pytest.mark.parametrize("mk", [lambda: W.taylor_green(24), lambda: W.cavity(24)])
def test_two_hop_kaporin_gradient_matches_autograd(lv, oracle, mk):
    flow = mk()
    g, L = _grid(lv, oracle, flow)
    assert L.lv_learn_set_pattern(g._ctx, 2) == 0
    pr = _params(L, g, 6, scale=0.3)
    rowptr, col, w, diag, adiag, _ = _export(lv, g, L)
    loss = C.c_double()
    grad = np.zeros(len(pr), np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lv_learn_loss_grad(g._ctx, -1, None, 0, 0, C.byref(loss), fp(grad)) == 0
    rl, rg = LR.loss_and_grad(rowptr, col, w, diag, adiag, pr, None, hops=2)
    assert abs(loss.value - rl) <= 1e-4 * max(1.0, abs(rl)), (loss.value, rl)
    for name, (o, s) in LR.OFF.items():
        a, b = grad[o:o + s].astype(np.float64), rg[o:o + s]
        nb = np.linalg.norm(b)
        assert np.linalg.norm(a - b) <= 3e-2 * nb + 1e-6, (name, np.linalg.norm(a - b), nb)
    # the Hutchinson objective is refused with the two-hop pattern
    assert L.lv_learn_loss_grad(g._ctx, -1, None, 2, 1, C.byref(loss), None) != 0


def _harvest(lv, oracle, flow, seeds):
    """A grid per seed, operator assembled and snapshot for training; returns the last grid."""
    from lvgpu import populate as pop
    grids = []
    for s in seeds:
        x = H.seeds(pop, flow, s, jitter=0.25)
        g = H.make_gpu(lv, flow, x)
        og = H.make_oracle(oracle, flow, x)
        H.init_both(flow, g, og)
        grids.append((g, og))
    return grids


def test_training_lowers_loss_and_iterations(lv, oracle):
    """Train on operators of one flow, then solve a held-out one: the trained
    factor needs fewer inner CG iterations than Jacobi, and the FP64 residual
    meets 1e-8 either way."""
    flow = W.cavity(64)
    grids = _harvest(lv, oracle, flow, [21, 22, 23, 24, 25, 26])
    L = lv._lib.load()
    trainer, _ = grids[0]
    assert L.lv_learn_init(trainer._ctx, 7) == 0
    # snapshot the training operators into the first grid's set
    for g, og in grids[:-1]:
        assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    # systems are snapshot per context: use the first grid's own operator and
    # those of the others through parameter sharing
    assert L.lv_pressure_operator(trainer._ctx, flow.dt) == 0
    assert L.lv_learn_add_system(trainer._ctx) == 0
    steps = 400
    losses = np.zeros(steps, np.float32)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    assert L.lv_learn_train(trainer._ctx, steps, 3e-3, 4, 1, fp(losses)) == 0
    assert losses[-20:].mean() < 0.8 * losses[:5].mean(), (losses[:5], losses[-20:])
    npar = L.lv_learn_num_params()
    pr = np.zeros(npar, np.float32)
    assert L.lv_learn_get_params(trainer._ctx, fp(pr)) == 0
    # held-out system
    g, og = grids[-1]
    assert L.lv_learn_set_params(g._ctx, fp(pr)) == 0
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    og.pressure_operator(flow.dt)
    rng = np.random.default_rng(0)
    b = rng.standard_normal(g.n)
    b -= b.mean()
    res = {}
    for m in ("mixed_ir", "learned_pcg"):
        lv.PressureSolver(g, method=m, tol=1e-8).configure()
        xg = np.zeros(g.n)
        st = lv.LvSolveStats()
        assert L.lv_solve(g._ctx, lv._lib.ptr(b), lv._lib.ptr(xg), C.byref(st)) == 0
        rel = np.linalg.norm(b - og.operator_apply(xg)) / np.linalg.norm(b)
        assert st.converged == 1 and rel <= 1.5e-8, (m, rel)
        res[m] = (st.iterations, st.method)
    print("jacobi mixed vs learned inner iterations:", res)
    it_j, _ = res["mixed_ir"]
    it_l, meth = res["learned_pcg"]
    assert meth == 2, "the trained factor fell back to Jacobi"
    assert it_l < it_j, res
    # the two-hop pattern, trained the same way, needs fewer still
    assert L.lv_learn_set_pattern(trainer._ctx, 2) == 0
    assert L.lv_learn_init(trainer._ctx, 7) == 0
    assert L.lv_learn_train(trainer._ctx, steps, 3e-3, 0, 1, fp(losses)) == 0
    assert L.lv_learn_get_params(trainer._ctx, fp(pr)) == 0
    assert L.lv_learn_set_pattern(g._ctx, 2) == 0
    assert L.lv_learn_set_params(g._ctx, fp(pr)) == 0
    lv.PressureSolver(g, method="learned_pcg", tol=1e-8).configure()
    xg = np.zeros(g.n)
    st = lv.LvSolveStats()
    assert L.lv_solve(g._ctx, lv._lib.ptr(b), lv._lib.ptr(xg), C.byref(st)) == 0
    rel = np.linalg.norm(b - og.operator_apply(xg)) / np.linalg.norm(b)
    assert st.converged == 1 and rel <= 1.5e-8, rel
    print("two-hop learned inner iterations:", st.iterations, st.method)
    assert st.method == 2 and st.iterations < it_l, (st.iterations, it_l)


@pytest.mark.parametrize("nx", [64, 256, 300])
def test_halo_mode_is_bit_identical(lv, monkeypatch, nx):
    """The learned one-block-per-SM solve in its staged mode (each block
    computes M^-1 r on its halo from shared memory: one neighbour exchange per
    iteration) gives the same iterate, bit for bit, and the same iteration
    count as with u exchanged between blocks (two exchanges): every halo value
    is computed exactly as its owner computes it.  64^2, 256^2 (one row per
    thread, halos above 512 rows) and 300^2 (two rows per thread); an
    untrained and a perturbed network; and a learned solve that falls back to
    Jacobi (the reference count from a loose mixed solve is exceeded)."""
    from lvgpu import populate as pop
    flow = W.taylor_green(nx)
    x = H.seeds(pop, flow, 5, jitter=0.25)
    g = H.make_gpu(lv, flow, x)
    for k, v in W.initial_fields(flow, g["x"], g["area"]).items():
        g[k] = v
    lv.stiffened_eos(g, flow.gamma, flow.P0)
    L = lv._lib.load()
    assert L.lv_pressure_operator(g._ctx, flow.dt) == 0
    rng = np.random.default_rng(1)
    b = rng.standard_normal(g.n)
    b -= b.mean()

    def solve(method, tol):
        lv.PressureSolver(g, method=method, tol=tol).configure()
        xg = np.zeros(g.n)
        st = lv.LvSolveStats()
        assert L.lv_solve(g._ctx, lv._lib.ptr(b), lv._lib.ptr(xg), C.byref(st)) == 0
        return xg, st

    for scale, prior_tol in ((None, None), (0.3, None), (0.3, 1e-2)):
        out = {}
        for halo in ("0", "1"):
            monkeypatch.setenv("LVGPU_FCG_HALO", halo)
            if prior_tol is not None:
                solve("mixed_ir", prior_tol)  # sets the Jacobi reference count
            else:
                solve("mixed_ir", 1e-8)
            if scale is None:
                assert L.lv_learn_init(g._ctx, 5) == 0  # invalidates the factor: rebuilt in this mode
            else:
                _params(L, g, 5, scale=scale)
            xg, st = solve("learned_pcg", 1e-8)
            assert st.converged == 1, (scale, prior_tol, halo, st.iterations)
            hr = C.c_int32()
            assert L.lv_solver_halo(g._ctx, C.byref(hr)) == 0
            if halo == "0":
                assert hr.value == 0
            else:
                assert hr.value > (512 if nx >= 256 else 0), hr.value
            out[halo] = (xg, st.iterations, st.method)
        if prior_tol is not None:
            assert out["1"][2] == 1, "expected the fallback to Jacobi"
        assert out["0"][1:] == out["1"][1:], (scale, prior_tol, out["0"][1:], out["1"][1:])
        assert np.array_equal(out["0"][0], out["1"][0]), (scale, prior_tol)
