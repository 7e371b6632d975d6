"""ctypes wrapper of the CPU oracle (oracle/liblvref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
CPU-baseline leg of bench.py, never by the product package.  The oracle
restates LagrangianVoronoi.jl's per-timestep path in plain C++ (see
lvref.cpp for the per-function citations of the reference).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

F_X, F_V, F_E, F_P, F_RHO, F_C2, F_DV, F_MASS, F_MOMENTUM, F_ENERGY, F_PHASE, F_QUALITY, F_D, F_MU, F_T, F_K, F_CV = range(17)
NCOMP = {F_X: 2, F_V: 2, F_DV: 2, F_MOMENTUM: 2, F_D: 4}
FIELD_NAMES = {"x": F_X, "v": F_V, "e": F_E, "P": F_P, "rho": F_RHO, "c2": F_C2, "dv": F_DV, "mass": F_MASS,
               "momentum": F_MOMENTUM, "energy": F_ENERGY, "phase": F_PHASE, "quality": F_QUALITY, "D": F_D,
               "mu": F_MU, "T": F_T, "k": F_K, "cV": F_CV}


class GridParams(C.Structure):
    _fields_ = [("xmin", C.c_double * 2), ("xmax", C.c_double * 2), ("dr", C.c_double), ("h", C.c_double),
                ("r_max", C.c_double), ("xperiodic", C.c_int32), ("yperiodic", C.c_int32),
                ("max_edges", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("rel_residual", C.c_double)]


def build(force=False):
    """Compile liblvref.so with the committed Makefile (gcc, OpenMP)."""
    so = os.path.join(_HERE, "liblvref.so")
    src = os.path.join(_HERE, "lvref.cpp")
    if force or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B", "liblvref.so"], check=True)
    return so


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(build())
        vp, d, i32, i64 = C.c_void_p, C.c_double, C.c_int32, C.c_int64
        pd, pi32, pi64 = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
        sig = {
            "lvref_ideal_temperature": (C.c_int, [vp]),
            "lvref_fourier_step": (C.c_int, [vp, d]),
            "lvref_heat_from_bdary": (C.c_int, [vp, d, pd]),
            "lvref_viscous_solve": (C.c_int, [vp, d, d, C.c_int, C.POINTER(SolveStats)]),
            "lvref_boundary_edges": (i64, [vp, pd, pi32, i64]),
            "lvref_set_edge_values": (C.c_int, [vp, i64, pd, C.POINTER(C.c_uint8)]),
            "lvref_create": (vp, [C.POINTER(GridParams), C.c_int]),
            "lvref_destroy": (None, [vp]),
            "lvref_num_threads": (C.c_int, [C.c_int]),
            "lvref_cell_dims": (C.c_int, [vp, pi64, pi64]),
            "lvref_path": (C.c_int, [vp, pi64, pi64, pd, C.c_int]),
            "lvref_set_field": (C.c_int, [vp, C.c_int, pd]),
            "lvref_get_field": (C.c_int, [vp, C.c_int, pd]),
            "lvref_remesh": (C.c_int, [vp]),
            "lvref_cell_items": (i64, [vp, pi64, pi32, i64]),
            "lvref_get_edges": (C.c_int, [vp, C.c_int, pi32, pd, pi32, pd, pd]),
            "lvref_get_faces": (i64, [vp, pi64, pi32, pd, pd, pd, pd, i64]),
            "lvref_clip_polygon": (C.c_int, [pd, pd, i64, C.c_int, pd, pi32, C.c_int, C.POINTER(C.c_int)]),
            "lvref_ideal_eos": (C.c_int, [vp, d, d]),
            "lvref_stiffened_eos": (C.c_int, [vp, d, d]),
            "lvref_find_rho": (C.c_int, [vp]),
            "lvref_gravity_step": (C.c_int, [vp, d, d, d]),
            "lvref_pressure_step": (C.c_int, [vp, d]),
            "lvref_find_D": (C.c_int, [vp]),
            "lvref_viscous_step": (C.c_int, [vp, d, C.c_int]),
            "lvref_bdary_friction": (C.c_int, [vp, pd, d]),
            "lvref_find_dv": (C.c_int, [vp, d, d]),
            "lvref_relaxation_step": (C.c_int, [vp, d, C.c_int]),
            "lvref_relax_no_remesh": (C.c_int, [vp, d, C.c_int]),
            "lvref_move": (C.c_int, [vp, d]),
            "lvref_move_no_remesh": (C.c_int, [vp, d]),
            "lvref_pressure_operator": (i64, [vp, d, pd, pi64, pi32, pd, i64]),
            "lvref_pressure_rhs": (C.c_int, [vp, d, C.c_int, pd, pd, pd]),
            "lvref_operator_apply": (C.c_int, [vp, pd, pd]),
            "lvref_find_pressure": (C.c_int, [vp, d, C.c_int, pd, C.c_int, d, C.c_int, C.POINTER(SolveStats)]),
            "lvref_solve": (C.c_int, [vp, pd, pd, C.c_int, d, C.c_int, C.POINTER(SolveStats)]),
            "lvref_multiphase_projection": (C.c_int, [vp, d, d, C.c_int, C.POINTER(SolveStats)]),
            "lvref_nearest_polygon": (C.c_int, [vp, C.c_int, pd, pi32]),
            "lvref_movingls": (C.c_int, [vp, C.c_int, C.c_int, pi32, pd, d, pd]),
            "lvref_point_value": (C.c_int, [vp, C.c_int, pd, pd, pd]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


class OracleGrid:
    """A VoronoiGrid of the oracle: domain [xmin,xmax], resolution dr, cell
    size h (default 2dr) and r_max (default 10dr), as VoronoiGrid{T}
    (src/voronoigrid.jl:14-50)."""

    def __init__(self, xlims, ylims, dr, n, h=None, r_max=None, xperiodic=False, yperiodic=False, max_edges=64):
        L = lib()
        p = GridParams()
        p.xmin[0], p.xmin[1] = float(xlims[0]), float(ylims[0])
        p.xmax[0], p.xmax[1] = float(xlims[1]), float(ylims[1])
        p.dr = float(dr)
        p.h = float(2.0 * dr if h is None else h)
        p.r_max = float(10.0 * dr if r_max is None else r_max)
        p.xperiodic, p.yperiodic, p.max_edges = int(xperiodic), int(yperiodic), int(max_edges)
        self.params = p
        self.n = int(n)
        self.h = L.lvref_create(C.byref(p), self.n)
        self.max_edges = max_edges

    def __del__(self):
        if getattr(self, "h", None) and _LIB is not None:
            _LIB.lvref_destroy(self.h)
            self.h = None

    def set(self, name, arr):
        f = FIELD_NAMES[name]
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64).reshape(self.n * NCOMP.get(f, 1)))
        st = lib().lvref_set_field(self.h, f, _p(a))
        assert st == 0

    def get(self, name):
        if name in ("area", "centroid"):
            return self.edges()[name]
        f = FIELD_NAMES[name]
        k = NCOMP.get(f, 1)
        a = np.empty(self.n * k, dtype=np.float64)
        lib().lvref_get_field(self.h, f, _p(a))
        return a.reshape(self.n, k) if k > 1 else a

    def cell_dims(self):
        n1, n2 = C.c_int64(), C.c_int64()
        lib().lvref_cell_dims(self.h, C.byref(n1), C.byref(n2))
        return n1.value, n2.value

    def path(self):
        cap = 4096
        i1 = np.zeros(cap, np.int64)
        i2 = np.zeros(cap, np.int64)
        rr = np.zeros(cap)
        n = lib().lvref_path(self.h, _p(i1, C.c_int64), _p(i2, C.c_int64), _p(rr), cap)
        return i1[:n], i2[:n], rr[:n]

    def remesh(self):
        return lib().lvref_remesh(self.h)

    def cell_items(self):
        n1, n2 = self.cell_dims()
        starts = np.zeros(n1 * n2 + 1, np.int64)
        tot = lib().lvref_cell_items(self.h, _p(starts, C.c_int64), None, 0)
        items = np.zeros(max(tot, 1), np.int32)
        lib().lvref_cell_items(self.h, _p(starts, C.c_int64), _p(items, C.c_int32), tot)
        return starts, items[:tot]

    def edges(self, maxe=None):
        maxe = maxe or self.max_edges
        counts = np.zeros(self.n, np.int32)
        verts = np.zeros((self.n, maxe, 4))
        labels = np.zeros((self.n, maxe), np.int32)
        area = np.zeros(self.n)
        cen = np.zeros((self.n, 2))
        st = lib().lvref_get_edges(self.h, maxe, _p(counts, C.c_int32), _p(verts), _p(labels, C.c_int32), _p(area),
                                   _p(cen))
        return dict(status=st, counts=counts, verts=verts, labels=labels, area=area, centroid=cen)

    def faces(self):
        L = lib()
        rowptr = np.zeros(self.n + 1, np.int64)
        nf = L.lvref_get_faces(self.h, _p(rowptr, C.c_int64), None, None, None, None, None, 0)
        nbr = np.zeros(nf, np.int32)
        lrr = np.zeros(nf)
        mid = np.zeros((nf, 2))
        y = np.zeros((nf, 2))
        ln = np.zeros(nf)
        L.lvref_get_faces(self.h, _p(rowptr, C.c_int64), _p(nbr, C.c_int32), _p(lrr), _p(mid), _p(y), _p(ln), nf)
        return dict(rowptr=rowptr, nbr=nbr, lrr=lrr, mid=mid, y=y, len=ln)

    # physics (same names as the reference, without '!')
    def ideal_eos(self, gamma=1.4, Pmin=0.0):
        return lib().lvref_ideal_eos(self.h, gamma, Pmin)

    def stiffened_eos(self, gamma=1.4, P0=0.0):
        return lib().lvref_stiffened_eos(self.h, gamma, P0)

    def find_rho(self):
        return lib().lvref_find_rho(self.h)

    def gravity_step(self, g, dt):
        return lib().lvref_gravity_step(self.h, float(g[0]), float(g[1]), dt)

    def pressure_step(self, dt):
        return lib().lvref_pressure_step(self.h, dt)

    def find_D(self):
        return lib().lvref_find_D(self.h)

    def viscous_step(self, dt, artificial_viscosity=True):
        return lib().lvref_viscous_step(self.h, dt, int(artificial_viscosity))

    def bdary_friction(self, vwall, dt):
        w = np.ascontiguousarray(np.asarray(vwall, np.float64).reshape(8))
        return lib().lvref_bdary_friction(self.h, _p(w), dt)

    def ideal_temperature(self):
        lib().lvref_ideal_temperature(self.h)

    def fourier_step(self, dt):
        lib().lvref_fourier_step(self.h, dt)

    def heat_from_bdary(self, dt, Tb):
        """Tb: the wall temperature of every boundary edge (NaN: adiabatic)."""
        t = np.ascontiguousarray(np.asarray(Tb, np.float64))
        return lib().lvref_heat_from_bdary(self.h, dt, _p(t))

    def viscous_solve(self, dt, tol=1e-6, itmax=2000):
        """ViscousSolver + viscous_step!(solver, dt): returns (iterations, converged, rel_residual)."""
        st = SolveStats()
        lib().lvref_viscous_solve(self.h, dt, tol, itmax, C.byref(st))
        return st.iterations, st.converged, st.rel_residual

    def boundary_edges(self):
        """Midpoints [nb][2] and labels [nb] of the boundary edges, in the
        order of boundaries(p) over the polygons."""
        nb = lib().lvref_boundary_edges(self.h, None, None, 0)
        mid = np.zeros((nb, 2))
        lab = np.zeros(nb, np.int32)
        lib().lvref_boundary_edges(self.h, _p(mid), _p(lab, C.c_int32), nb)
        return mid, lab

    def set_edge_values(self, vb=None, act=None):
        """Per-edge boundary velocities (and charfun flags) for the next
        right-hand sides and frictions; vb None returns to the label table."""
        if vb is None:
            lib().lvref_set_edge_values(self.h, 0, None, None)
            return
        vb = np.ascontiguousarray(np.asarray(vb, np.float64).reshape(-1, 2))
        a = None if act is None else np.ascontiguousarray(np.asarray(act, np.uint8))
        lib().lvref_set_edge_values(self.h, len(vb), _p(vb), None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint8)))

    def find_dv(self, dt, alpha=1.0):
        return lib().lvref_find_dv(self.h, dt, alpha)

    def relaxation_step(self, dt, rusanov=True, remesh=True):
        if remesh:
            return lib().lvref_relaxation_step(self.h, dt, int(rusanov))
        return lib().lvref_relax_no_remesh(self.h, dt, int(rusanov))

    def move(self, dt, remesh=True):
        if remesh:
            return lib().lvref_move(self.h, dt)
        return lib().lvref_move_no_remesh(self.h, dt)

    def pressure_operator(self, dt):
        L = lib()
        rowptr = np.zeros(self.n + 1, np.int64)
        diag = np.zeros(self.n)
        nnz = L.lvref_pressure_operator(self.h, dt, _p(diag), _p(rowptr, C.c_int64), None, None, 0)
        col = np.zeros(nnz, np.int32)
        w = np.zeros(nnz)
        L.lvref_pressure_operator(self.h, dt, _p(diag), _p(rowptr, C.c_int64), _p(col, C.c_int32), _p(w), nnz)
        return dict(diag=diag, rowptr=rowptr, col=col, w=w)

    def pressure_rhs(self, dt, gp_step, vbc=None):
        b = np.zeros(self.n)
        gp = np.zeros((self.n, 2))
        v = None if vbc is None else np.ascontiguousarray(np.asarray(vbc, np.float64).reshape(8))
        lib().lvref_pressure_rhs(self.h, dt, int(gp_step), _p(v), _p(b), _p(gp))
        return b, gp

    def operator_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n)
        lib().lvref_operator_apply(self.h, _p(x), _p(y))
        return y

    def find_pressure(self, dt, niter=10, vbc=None, method="pcg", tol=1e-8, itmax=10000, guess=False):
        """guess: with method "pcg", start each sweep from the GPU solver's
        Galerkin guess (the span of the last sweep's change and the previous
        call's change of the same sweep) instead of the previous sweep's P."""
        stats = (SolveStats * niter)()
        v = None if vbc is None else np.ascontiguousarray(np.asarray(vbc, np.float64).reshape(8))
        m = 0 if method == "minres" else (2 if guess else 1)
        lib().lvref_find_pressure(self.h, dt, niter, _p(v), m, tol, itmax, stats)
        return [(s.iterations, s.converged, s.rel_residual) for s in stats]

    def solve(self, b, x0, method="pcg", tol=1e-8, itmax=10000):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.ascontiguousarray(np.array(x0, dtype=np.float64))
        st = SolveStats()
        lib().lvref_solve(self.h, _p(b), _p(x), 0 if method == "minres" else 1, tol, itmax, C.byref(st))
        return x, (st.iterations, st.converged, st.rel_residual)

    def multiphase_projection(self, quality_threshold=0.25, tol=1e-4, itmax=200):
        st = SolveStats()
        lib().lvref_multiphase_projection(self.h, quality_threshold, tol, itmax, C.byref(st))
        return st.iterations, st.converged


    # post-processing (voronoigrid.jl:154-178, movingls.jl:52-146)
    def nearest_polygon(self, pts):
        pts = np.ascontiguousarray(np.asarray(pts, np.float64).reshape(-1, 2))
        out = np.zeros(len(pts), np.int32)
        lib().lvref_nearest_polygon(self.h, len(pts), _p(pts), _p(out, C.c_int32))
        return out

    def movingls(self, order, values, h, polys=None):
        nc = {1: 2, 2: 5, 3: 9}[order]
        f = np.ascontiguousarray(values, dtype=np.float64)
        m = self.n if polys is None else len(polys)
        pl = None if polys is None else np.ascontiguousarray(polys, dtype=np.int32)
        out = np.zeros((m, nc))
        lib().lvref_movingls(self.h, order, m, _p(pl, C.c_int32), _p(f), float(h), _p(out))
        return out

    def point_value(self, pts, values):
        pts = np.ascontiguousarray(np.asarray(pts, np.float64).reshape(-1, 2))
        f = np.ascontiguousarray(values, dtype=np.float64)
        out = np.zeros(len(pts))
        lib().lvref_point_value(self.h, len(pts), _p(pts), _p(f), _p(out))
        return out


def clip_polygon(px, y, label, edges, labels, cap=64):
    """Half-plane clip of one polygon (polygon.jl:51-97) — for known-answer tests."""
    L = lib()
    k = len(edges)
    verts = np.zeros((cap, 4))
    verts[:k] = np.asarray(edges, np.float64).reshape(k, 4)
    lab = np.zeros(cap, np.int32)
    lab[:k] = labels
    cut = C.c_int()
    px = np.ascontiguousarray(px, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    n = L.lvref_clip_polygon(_p(px), _p(y), int(label), k, _p(verts), _p(lab, C.c_int32), cap, C.byref(cut))
    return verts[:n].copy(), lab[:n].copy(), bool(cut.value)


def set_threads(nt):
    return lib().lvref_num_threads(int(nt))
