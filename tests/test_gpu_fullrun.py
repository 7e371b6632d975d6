"""bench.py --full-run on small workloads: the run completes with every
pressure sweep converged, finite fields, and the conserved totals held
(mass to rounding; momentum in a periodic domain to rounding)."""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _args(solver, steps):
    return type("Args", (), dict(train_steps=40, train_lr=5e-3, train_probes=0, learn_hops=1, solver=solver,
                                 no_compare=True, warmup=3, full_steps=steps))()


@pytest.mark.parametrize("solver", ["learned_pcg", "jacobi_pcg"])
def test_full_run_taylor_green(solver):
    sys.path.insert(0, ROOT)
    import bench
    r = bench.full_run(_args(solver, 40), bench.Workload("taylor_green", 64))
    assert r["failure"] is None and r["steps"] == 40
    assert r["unconverged_sweeps"] == 0 and r["all_finite"]
    assert abs(r["drift"]["mass"]) < 1e-13
    assert max(abs(m) for m in r["drift"]["momentum_abs"]) < 1e-12
    assert r["drift"]["kinetic"] < 0.0  # viscous decay of the vortex
