"""Rayleigh-Taylor over its full 300 steps (128 x 256 particles, so that the
oracle runs alongside): the GPU's mixed precision (FP32 inner CG in FP64
refinement, 1e-8) against the oracle's FP64 PCG (1e-8), both with the
reference's multiphase MINRES at 1e-4 (relaxation.jl:180-206).  The fields
stay within the solvers' tolerances of each other over the whole run
(largest difference relative to the field's largest value, x relative to
dr): velocity 1e-3 (the multiphase projection's tolerance), the rest 1e-4."""
import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

TOL = {"x": 1e-4, "v": 1e-3, "P": 1e-4, "rho": 1e-4, "e": 1e-4, "mass": 1e-4}


def test_rayleigh_taylor_300_steps_mixed_against_oracle(lv, oracle):
    from lvgpu import populate as pop
    fl = W.rayleigh_taylor(128, 256)
    x = H.seeds(pop, fl)
    g = H.make_gpu(lv, fl, x)
    og = H.make_oracle(oracle, fl, x)
    H.init_both(fl, g, og)
    solver = lv.PressureSolver(g, method="mixed_ir", tol=1e-8)
    dt, seq = W.step_sequence(fl)
    for step in range(1, 301):
        for op, kw in seq:
            H.apply(lv, fl, g, op, kw, True, solver=solver)
            H.apply(lv, fl, og, op, kw, False)
        if step % 100 == 0:
            g.synchronize()
            for k, tol in TOL.items():
                a, b = g[k], og.get(k)
                scale = fl.dr if k == "x" else max(np.max(np.abs(b)), 1e-30)
                err = np.max(np.abs(a - b)) / scale
                assert err < tol, (step, k, err)
