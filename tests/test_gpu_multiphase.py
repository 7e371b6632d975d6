"""multiphase_projection! (src/relaxation.jl:80-206) on the GPU against the
oracle: same MINRES (Paige & Saunders, atol = rtol = 1e-4, itmax = 200), so
the projected repair velocity agrees to the solver's tolerance."""
import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nx,ny", [(24, 48), (48, 96)])
def test_multiphase_projection_matches_oracle(lv, oracle, nx, ny):
    from lvgpu import populate as pop
    flow = W.rayleigh_taylor(nx, ny)
    x = H.seeds(pop, flow, 9)
    g = H.make_gpu(lv, flow, x)
    og = H.make_oracle(oracle, flow, x)
    H.init_both(flow, g, og)
    rng = np.random.default_rng(2)
    D = 5.0 * rng.standard_normal((len(x), 4))
    g["D"] = D
    og.set("D", D)
    lv.find_dv(g, flow.dt)
    og.find_dv(flow.dt)
    dv0 = g["dv"]
    assert np.array_equal(dv0, og.get("dv"))
    it_gpu, conv_gpu = lv.multiphase_projection(lv.MultiphaseSolver(g))
    it_ref, conv_ref = og.multiphase_projection()
    assert abs(it_gpu - it_ref) <= 2, (it_gpu, it_ref)
    corr_gpu = g["dv"] - dv0
    corr_ref = og.get("dv") - dv0
    assert np.linalg.norm(corr_ref) > 0
    assert np.linalg.norm(corr_gpu - corr_ref) <= 1e-3 * np.linalg.norm(corr_ref)
    # untouched where the projection does not apply (same-phase neighbourhoods)
    same = np.all(np.abs(corr_ref) == 0.0, axis=1)
    assert np.all(corr_gpu[same] == 0.0)
