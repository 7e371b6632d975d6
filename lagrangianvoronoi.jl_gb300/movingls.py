"""Moving least squares and point values on the device mesh
(src/movingls.jl, src/voronoigrid.jl:154-178).

The reference passes a Julia function of the polygon (`fun(p)`); here the
function is given by its per-polygon values (an array of n numbers, e.g.
grid["P"]).  movingls, point_value and nearest_polygon run as CUDA kernels
(csrc/lv_post.cu); power_vector, poly_eval and integral are host arithmetic
on the downloaded geometry, as in the reference.
"""
import ctypes as C

import numpy as np

from . import _lib

LinearExpansion, QuadraticExpansion, CubicExpansion = 1, 2, 3
_NC = {1: 2, 2: 5, 3: 9}


def _check(grid, rc):
    if rc != 0:
        L = _lib.load()
        msg = L.lv_last_error(grid._ctx)
        raise _lib.LvError(rc, msg.decode() if msg else "")


def gaussian_kernel(h, r):
    """gaussian_kernel (movingls.jl:22-24)."""
    return np.exp(-0.5 * (r / h) ** 2) / np.sqrt(2 * np.pi * h ** 2)


def power_vector(T, x):
    """power_vector (movingls.jl:26-36) for T = 1, 2, 3 (linear, quadratic, cubic)."""
    a, b = float(x[0]), float(x[1])
    v = [a, b]
    if T >= 2:
        v += [a * a, a * b, b * b]
    if T >= 3:
        v += [a * a * a, a * a * b, a * b * b, b * b * b]
    return np.array(v)


def poly_eval(val, taylor, dx):
    """poly_eval (movingls.jl:95-97): val + taylor . power_vector(dx)."""
    T = {2: 1, 5: 2, 9: 3}[len(taylor)]
    return float(val) + float(np.dot(taylor, power_vector(T, dx)))


def nearest_polygon(grid, x):
    """Index of the nearest seed of each point (voronoigrid.jl:154-178)."""
    grid._flush()
    pts = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 2))
    out = np.zeros(len(pts), np.int32)
    _check(grid, _lib.load().lv_nearest_polygon(grid._ctx, len(pts), _lib.ptr(pts), _lib.ptr(out, C.c_int32)))
    return out if np.ndim(x) > 1 else int(out[0])


def movingls(T, grid, values, polys=None, h=None):
    """movingls(T, grid, p, fun; h) (movingls.jl:52-86) for polygons `polys`
    (an index, a list, or None for all); returns coefficients [m][2|5|9]."""
    grid._flush()
    f = np.ascontiguousarray(values, dtype=np.float64)
    single = np.isscalar(polys)
    pl = None if polys is None else np.ascontiguousarray(np.atleast_1d(polys), dtype=np.int32)
    m = grid.n if pl is None else len(pl)
    out = np.zeros((m, _NC[T]))
    hh = float(h) if h is not None else float(grid.h)
    _check(grid, _lib.load().lv_movingls(grid._ctx, int(T), m, _lib.ptr(pl, C.c_int32) if pl is not None else None,
                                         _lib.ptr(f), hh, _lib.ptr(out)))
    return out[0] if single else out


def point_value(grid, x, values):
    """point_value(grid, x, fun) (movingls.jl:140-146) at one point or an array of points."""
    grid._flush()
    pts = np.ascontiguousarray(np.asarray(x, np.float64).reshape(-1, 2))
    f = np.ascontiguousarray(values, dtype=np.float64)
    out = np.zeros(len(pts))
    _check(grid, _lib.load().lv_point_value(grid._ctx, len(pts), _lib.ptr(pts), _lib.ptr(f), _lib.ptr(out)))
    return out if np.ndim(x) > 1 else float(out[0])


# integral (movingls.jl:105-138): quadrature of the expansion over the triangles (x, v1, v2)
_RULES = {
    1: [(1.0, (-2 / 3, 1 / 3, 1 / 3))],
    2: [(1 / 3, (-1 / 3, 1 / 6, 1 / 6)), (1 / 3, (-5 / 6, 2 / 3, 1 / 6)), (1 / 3, (-5 / 6, 1 / 6, 2 / 3))],
    3: [(-9 / 16, (-2 / 3, 1 / 3, 1 / 3)), (25 / 48, (-2 / 5, 1 / 5, 1 / 5)), (25 / 48, (-4 / 5, 3 / 5, 1 / 5)),
        (25 / 48, (-4 / 5, 1 / 5, 3 / 5))],
}


def integral(grid, i, val, taylor, geometry=None):
    """integral(p, val, taylor) (movingls.jl:105-138) over polygon i."""
    counts, verts, _ = geometry if geometry is not None else grid.geometry()
    T = {2: 1, 5: 2, 9: 3}[len(taylor)]
    x = np.asarray(grid.get("x")[i])
    tot = 0.0
    for k in range(counts[i]):
        v1, v2 = verts[i, k, 0:2], verts[i, k, 2:4]
        a = v1 - x
        b = v2 - x
        A = 0.5 * abs(a[0] * b[1] - a[1] * b[0])
        for wgt, (cx, c1, c2) in _RULES[T]:
            tot += wgt * A * poly_eval(val, taylor, cx * x + c1 * v1 + c2 * v2)
    return tot
