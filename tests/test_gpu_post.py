"""nearest_polygon, movingls and point_value on the GPU against the oracle
(movingls.jl:52-146, voronoigrid.jl:154-178)."""
import numpy as np
import pytest

import harness as H
import workloads as W

pytestmark = pytest.mark.gpu

FLOWS = {"periodic": lambda: W.taylor_green(32), "walls": lambda: W.cavity(32)}


def _pair(lv, oracle, flow):
    from lvgpu import populate as pop
    x = H.seeds(pop, flow, 9, jitter=0.2)
    return x, H.make_gpu(lv, flow, x), H.make_oracle(oracle, flow, x)


@pytest.mark.parametrize("name", list(FLOWS))
@pytest.mark.parametrize("order", [1, 2, 3])
def test_movingls_matches_oracle(lv, oracle, name, order):
    flow = FLOWS[name]()
    x, g, og = _pair(lv, oracle, flow)
    f = np.sin(6.0 * x[:, 0]) * np.cos(4.0 * x[:, 1])
    h = (1.5 + order) * flow.dr
    got = lv.movingls(order, g, f, h=h)
    ref = og.movingls(order, f, h)
    scale = np.maximum(1.0, np.abs(ref))
    assert np.max(np.abs(got - ref) / scale) < 1e-9, np.max(np.abs(got - ref) / scale)
    sub = np.array([0, 5, 100, len(x) - 1], dtype=np.int32)
    assert np.allclose(lv.movingls(order, g, f, polys=sub, h=h), ref[sub], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("name", list(FLOWS))
def test_point_value_and_nearest_match_oracle(lv, oracle, name):
    flow = FLOWS[name]()
    x, g, og = _pair(lv, oracle, flow)
    rng = np.random.default_rng(1)
    pts = 0.05 + 0.9 * rng.random((200, 2))
    assert np.array_equal(lv.nearest_polygon(g, pts), og.nearest_polygon(pts))
    f = np.sin(6.0 * x[:, 0]) * np.cos(4.0 * x[:, 1])
    got = lv.point_value(g, pts, f)
    ref = og.point_value(pts, f)
    assert np.max(np.abs(got - ref)) < 1e-12
    assert abs(lv.point_value(g, pts[0], f) - ref[0]) < 1e-12
