"""GB300 implementation of the Lagrangian Voronoi per-timestep path.

Host-side mirror of the LagrangianVoronoi.jl API (src/LagrangianVoronoi.jl
exports) over the C ABI of liblvgpu.so (include/lvgpu.h).  The Julia names
are kept without the trailing '!':

    grid = VoronoiGrid(Rectangle((0, 1), (0, 1)), dr, xperiodic=True, yperiodic=True)
    populate_jittered(grid, 256, 256)            # push seeds, remesh on the GPU
    grid["v"] = v0; grid["mass"] = rho * grid["area"]
    solver = PressureSolver(grid)
    move(grid, dt); stiffened_eos(grid, 1.4, P0); find_pressure(solver, dt)
    pressure_step(grid, dt); find_D(grid); viscous_step(grid, dt)
    find_dv(grid, dt); relaxation_step(grid, dt)

All state lives on the GPU; fields are copied to or from the host only when
indexed.  Every compute call goes to liblvgpu.so; there is no CPU path.
"""
import ctypes as C

import numpy as np

from . import _lib
from . import populate as _pop
from ._lib import LV_MAX_EDGES, LvError, LvParams, LvSolveStats

BDARY_UP, BDARY_RIGHT, BDARY_DOWN, BDARY_LEFT = -1, -2, -3, -4

__all__ = [
    "Rectangle", "UnitRectangle", "VoronoiGrid", "PressureSolver", "MultiphaseSolver", "remesh", "move",
    "ideal_eos", "stiffened_eos", "find_rho", "gravity_step", "find_pressure", "pressure_step", "find_D",
    "viscous_step", "bdary_friction", "find_dv", "relaxation_step", "multiphase_projection", "populate_jittered",
    "populate_rect", "populate_hex", "populate_circ", "populate_rand", "populate_vogel", "populate_lloyd", "run",
    "export_grid", "export_points", "LinearExpansion", "QuadraticExpansion", "CubicExpansion", "gaussian_kernel",
    "power_vector", "poly_eval", "nearest_polygon", "movingls", "point_value", "integral",
    "LvError", "BDARY_UP", "BDARY_RIGHT", "BDARY_DOWN", "BDARY_LEFT", "LV_MAX_EDGES", "wall_velocity_table",
    "zero_vbc", "ViscousSolver", "ideal_temperature", "fourier_step", "heat_from_bdary",
]


class Rectangle:
    """Rectangle(xlims, ylims) (src/geometry.jl:94-111)."""

    def __init__(self, xlims, ylims):
        self.xmin = (float(xlims[0]), float(ylims[0]))
        self.xmax = (float(xlims[1]), float(ylims[1]))

    @property
    def xlims(self):
        return (self.xmin[0], self.xmax[0])

    @property
    def ylims(self):
        return (self.xmin[1], self.xmax[1])


def UnitRectangle():
    return Rectangle((0.0, 1.0), (0.0, 1.0))


def _check(grid, rc):
    if rc != 0:
        msg = _lib.load().lv_last_error(grid._ctx)
        raise LvError(rc, msg.decode() if msg else "")


class VoronoiGrid:
    """VoronoiGrid{T}(rect, dr; h = 2dr, r_max = 10dr, xperiodic, yperiodic)
    (src/voronoigrid.jl:14-50).  `capacity` bounds the number of particles the
    device buffers hold; it defaults to the first particle count pushed."""

    def __init__(self, rect, dr, h=None, r_max=None, xperiodic=False, yperiodic=False, capacity=None, device=0):
        self.rect = rect
        self.dr = float(dr)
        self.h = float(2.0 * dr if h is None else h)
        self.r_max = float(10.0 * dr if r_max is None else r_max)
        self.xperiodic = bool(xperiodic)
        self.yperiodic = bool(yperiodic)
        self.capacity = capacity
        self.device = int(device)
        self._ctx = None
        self._pending = []
        self.n = 0

    # -- particle set
    def push(self, x):
        """push!(grid.polygons, T(x = x)) for every row of x ([k][2])."""
        self._pending.append(np.asarray(x, dtype=np.float64).reshape(-1, 2))

    def _ensure_ctx(self, n):
        if self._ctx is None:
            cap = int(self.capacity or n)
            p = LvParams()
            p.xmin[0], p.xmin[1] = self.rect.xmin
            p.xmax[0], p.xmax[1] = self.rect.xmax
            p.dr, p.h, p.r_max = self.dr, self.h, self.r_max
            p.xperiodic, p.yperiodic = int(self.xperiodic), int(self.yperiodic)
            p.capacity, p.device = cap, self.device
            ctx = _lib.load().lv_create(C.byref(p))
            if not ctx:
                raise LvError(7, "lv_create failed (no CUDA device or out of memory)")
            self._ctx = ctx
            self.capacity = cap

    def _flush(self):
        if not self._pending:
            return
        old = self.get("x") if (self._ctx is not None and self.n > 0) else np.zeros((0, 2))
        x = np.ascontiguousarray(np.concatenate([old] + self._pending, axis=0))
        self._pending = []
        self._ensure_ctx(len(x))
        _check(self, _lib.load().lv_set_positions(self._ctx, len(x), _lib.ptr(x)))
        self.n = len(x)

    def close(self):
        if self._ctx is not None:
            _lib.load().lv_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- fields
    def get(self, name):
        fid, k = _lib.FIELDS[name]
        a = np.empty(self.n * k, dtype=np.float64)
        _check(self, _lib.load().lv_get_field(self._ctx, fid, _lib.ptr(a)))
        return a.reshape(self.n, k) if k > 1 else a

    def get_many(self, names, out=None):
        """Several fields in one call (one synchronisation); `out` may hold
        preallocated float64 arrays of the right shapes."""
        L = _lib.load()
        arrays = []
        for k, name in enumerate(names):
            fid, w = _lib.FIELDS[name]
            a = out[k] if out is not None else np.empty((self.n, w) if w > 1 else self.n, dtype=np.float64)
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.n * w
            arrays.append(a)
        ids = np.array([_lib.FIELDS[nm][0] for nm in names], np.int32)
        ptrs = (C.c_void_p * len(names))(*[a.ctypes.data for a in arrays])
        _check(self, L.lv_get_fields(self._ctx, len(names), _lib.ptr(ids, C.c_int32), ptrs))
        return arrays

    def set_many(self, fields):
        """Several fields {name: array} in one call (one synchronisation)."""
        self._flush()
        L = _lib.load()
        names = list(fields)
        arrays = []
        for name in names:
            fid, w = _lib.FIELDS[name]
            a = np.ascontiguousarray(fields[name], dtype=np.float64)
            if a.size != self.n * w:
                raise ValueError(f"{name}: expected {self.n * w} values, got {a.size}")
            arrays.append(a)
        ids = np.array([_lib.FIELDS[nm][0] for nm in names], np.int32)
        ptrs = (C.c_void_p * len(names))(*[a.ctypes.data for a in arrays])
        _check(self, L.lv_set_fields(self._ctx, len(names), _lib.ptr(ids, C.c_int32), ptrs))

    def set(self, name, values):
        fid, k = _lib.FIELDS[name]
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(values, dtype=np.float64),
                                                 (self.n, k) if k > 1 else (self.n,)).reshape(-1))
        _check(self, _lib.load().lv_set_field(self._ctx, fid, _lib.ptr(a)))

    __getitem__ = get
    __setitem__ = set

    # -- geometry mirror (lazy downloads)
    def geometry(self):
        """Edges of every polygon in stored order: counts[n], verts[n][E][4], labels[n][E]."""
        L = _lib.load()
        counts = np.zeros(self.n, np.int32)
        verts = np.zeros((self.n, LV_MAX_EDGES, 4))
        labels = np.zeros((self.n, LV_MAX_EDGES), np.int32)
        _check(self, L.lv_get_geometry(self._ctx, _lib.ptr(counts, C.c_int32), _lib.ptr(verts),
                                       _lib.ptr(labels, C.c_int32)))
        return counts, verts, labels

    def faces(self):
        """Interior faces in `neighbors` order: rowptr, nbr, lrr, mid, y, len."""
        L = _lib.load()
        nf = C.c_int64()
        _check(self, L.lv_get_faces(self._ctx, C.byref(nf), None, None, None, None, None, None))
        F = nf.value
        rowptr = np.zeros(self.n + 1, np.int64)
        nbr = np.zeros(F, np.int32)
        lrr = np.zeros(F)
        mid = np.zeros((F, 2))
        y = np.zeros((F, 2))
        ln = np.zeros(F)
        _check(self, L.lv_get_faces(self._ctx, None, _lib.ptr(rowptr, C.c_int64), _lib.ptr(nbr, C.c_int32),
                                    _lib.ptr(lrr), _lib.ptr(mid), _lib.ptr(y), _lib.ptr(ln)))
        return dict(rowptr=rowptr, nbr=nbr, lrr=lrr, mid=mid, y=y, len=ln)

    def neighbors(self, i, faces=None):
        """neighbors(p, grid) (src/iterators.jl:19-33) for polygon i: (j, mid, y) triples."""
        F = faces or self.faces()
        a, b = F["rowptr"][i], F["rowptr"][i + 1]
        return [(int(F["nbr"][k]), F["mid"][k], F["y"][k]) for k in range(a, b)]

    def boundary_edges(self):
        """boundaries(p) (src/iterators.jl:46-57) over all polygons: the
        midpoints [nb][2] and labels [nb] of the boundary edges, in the order
        the per-edge entry points take their values."""
        L = _lib.load()
        nb = C.c_int64()
        _check(self, L.lv_get_boundary_edges(self._ctx, C.byref(nb), None, None))
        mid = np.zeros((nb.value, 2))
        lab = np.zeros(nb.value, np.int32)
        if nb.value:
            _check(self, L.lv_get_boundary_edges(self._ctx, None, _lib.ptr(mid), _lib.ptr(lab, C.c_int32)))
        return mid, lab

    def cell_list(self):
        L = _lib.load()
        nc, ni = C.c_int64(), C.c_int64()
        _check(self, L.lv_get_cell_list(self._ctx, C.byref(nc), C.byref(ni), None, None))
        starts = np.zeros(nc.value + 1, np.int32)
        items = np.zeros(max(ni.value, 1), np.int32)
        _check(self, L.lv_get_cell_list(self._ctx, None, None, _lib.ptr(starts, C.c_int32),
                                        _lib.ptr(items, C.c_int32)))
        return starts, items[:ni.value]

    def clip_captures(self):
        """Polygons of the last remesh finished by the second clipping pass."""
        n = C.c_int32()
        _check(self, _lib.load().lv_mesh_captures(self._ctx, C.byref(n)))
        return int(n.value)

    def synchronize(self):
        _check(self, _lib.load().lv_synchronize(self._ctx))

    def launch_count(self):
        return int(_lib.load().lv_launch_count(self._ctx)) if self._ctx is not None else 0


def zero_vbc(x, label):
    """The default boundary velocity of find_pressure! (src/pressure.jl:205-207)."""
    return (0.0, 0.0)


def _per_edge(f):
    """Whether a boundary closure is the reference's per-point form: f(x,
    label) for find_pressure!, f(x) for bdary_friction! (a one-argument
    closure of find_pressure! takes the label only, the label-table form)."""
    import inspect
    try:
        return len(inspect.signature(f).parameters)
    except (TypeError, ValueError):
        return 2


def wall_velocity_table(boundary_velocity):
    """Constant wall velocity per boundary label as the [4][2] table the C ABI
    takes (index -label-1: UP, RIGHT, DOWN, LEFT).  Accepts None (zero), a
    dict {label: (vx, vy)} or a callable f(label) -> (vx, vy)."""
    t = np.zeros((4, 2))
    if boundary_velocity is None:
        return None
    for lab in (BDARY_UP, BDARY_RIGHT, BDARY_DOWN, BDARY_LEFT):
        if callable(boundary_velocity):
            v = boundary_velocity(lab)
        else:
            v = boundary_velocity.get(lab, (0.0, 0.0))
        t[-lab - 1] = v
    return np.ascontiguousarray(t.reshape(8))


# ------------------------------------------------------------ operations

def remesh(grid, sync=True):
    """remesh!(grid) (src/voronoigrid.jl:89-108)."""
    grid._flush()
    L = _lib.load()
    _check(grid, L.lv_remesh(grid._ctx) if sync else L.lv_remesh_async(grid._ctx))


def move(grid, dt):
    """move!(grid, dt) (src/move.jl:9-21); remeshes."""
    _check(grid, _lib.load().lv_move(grid._ctx, float(dt)))


def ideal_eos(grid, gamma=1.4, Pmin=0.0):
    _check(grid, _lib.load().lv_ideal_eos(grid._ctx, float(gamma), float(Pmin)))


def stiffened_eos(grid, gamma=1.4, P0=0.0):
    _check(grid, _lib.load().lv_stiffened_eos(grid._ctx, float(gamma), float(P0)))


def find_rho(grid):
    _check(grid, _lib.load().lv_find_rho(grid._ctx))


def gravity_step(grid, g, dt):
    _check(grid, _lib.load().lv_gravity_step(grid._ctx, float(g[0]), float(g[1]), float(dt)))


def pressure_step(grid, dt):
    _check(grid, _lib.load().lv_pressure_step(grid._ctx, float(dt)))


def find_D(grid):
    _check(grid, _lib.load().lv_find_D(grid._ctx))


class ViscousSolver:
    """ViscousSolver(grid) (src/viscous_solver.jl:43-66): the implicit viscous
    step, solved by MINRES (atol = rtol = 1e-6, itmax = 2000)."""

    def __init__(self, grid, verbose=0):
        self.grid = grid
        self.verbose = verbose
        self.last_stats = None


def viscous_step(target, dt, artificial_viscosity=True):
    """viscous_step!(grid, dt; artificial_viscosity) (src/diffusion.jl:39-53),
    explicit; or viscous_step!(solver::ViscousSolver, dt)
    (src/viscous_solver.jl:109-129), implicit: returns (iterations,
    converged)."""
    if isinstance(target, ViscousSolver):
        g = target.grid
        st = LvSolveStats()
        _check(g, _lib.load().lv_viscous_solve(g._ctx, float(dt), C.byref(st)))
        target.last_stats = (st.iterations, bool(st.converged), st.rel_residual)
        return st.iterations, bool(st.converged)
    _check(target, _lib.load().lv_viscous_step(target._ctx, float(dt), int(bool(artificial_viscosity))))


def ideal_temperature(grid):
    """ideal_temperature!(grid) (src/fourier.jl:1-12): T = (e - |v|^2/2) / cV."""
    _check(grid, _lib.load().lv_ideal_temperature(grid._ctx))


def fourier_step(grid, dt):
    """fourier_step!(grid, dt) (src/fourier.jl:14-28): heat conduction with the
    fields T and k."""
    _check(grid, _lib.load().lv_fourier_step(grid._ctx, float(dt)))


def heat_from_bdary(grid, dt, T_bc, gamma=1.4):
    """heat_from_bdary!(grid, dt, T_bc, gamma) (src/fourier.jl:30-62):
    T_bc(x, label) -> wall temperature (NaN: adiabatic), evaluated here at
    every boundary edge's midpoint."""
    mid, lab = grid.boundary_edges()
    Tb = np.ascontiguousarray(np.array([T_bc(m, int(l)) for m, l in zip(mid, lab)], dtype=np.float64))
    _check(grid, _lib.load().lv_heat_from_bdary_edges(grid._ctx, len(mid), _lib.ptr(Tb), float(gamma), float(dt)))


def bdary_friction(grid, vDirichlet, dt, charfun=None):
    """bdary_friction!(grid, vDirichlet, dt; charfun) (src/diffusion.jl:64-79).
    vDirichlet is the reference's closure of the boundary point, vDirichlet(x)
    -> (vx, vy), evaluated here at every boundary edge's midpoint, with
    charfun(x) -> bool selecting the edges; or a constant wall velocity per
    label (a dict {label: (vx, vy)}, None for zero)."""
    L = _lib.load()
    if callable(vDirichlet) or charfun is not None:
        mid, lab = grid.boundary_edges()
        if callable(vDirichlet):
            vb = np.array([vDirichlet(m) for m in mid], dtype=np.float64).reshape(-1, 2)
        else:
            t = wall_velocity_table(vDirichlet)
            t = np.zeros(8) if t is None else t
            vb = t.reshape(4, 2)[-lab - 1] if len(lab) else np.zeros((0, 2))
        vb = np.ascontiguousarray(vb)
        act = None
        if charfun is not None:
            act = np.ascontiguousarray(np.array([bool(charfun(m)) for m in mid], dtype=np.uint8))
        _check(grid, L.lv_bdary_friction_edges(grid._ctx, len(mid), _lib.ptr(vb),
                                               None if act is None else _lib.ptr(act, C.c_uint8), float(dt)))
        return
    t = wall_velocity_table(vDirichlet)
    if t is None:
        t = np.zeros(8)
    _check(grid, L.lv_bdary_friction(grid._ctx, _lib.ptr(t), float(dt)))


def find_dv(grid, dt, alpha=1.0):
    _check(grid, _lib.load().lv_find_dv(grid._ctx, float(dt), float(alpha)))


def relaxation_step(grid, dt, rusanov=True):
    """relaxation_step!(grid, dt; rusanov) (src/relaxation.jl:36-73); remeshes."""
    _check(grid, _lib.load().lv_relaxation_step(grid._ctx, float(dt), int(bool(rusanov))))


class PressureSolver:
    """PressureSolver(grid) (src/pressure.jl:142-159) with the solver choice.
    The default is the reference's own solve: method 'minres' (FP64 MINRES
    without a preconditioner, stopping at ||r|| <= tol + tol ||r0||, warm
    started from P), tol 1e-6, itmax 1000 (pressure.jl:219).  The CG methods
    'jacobi_pcg' (FP64), 'mixed_ir' and 'learned_pcg' (FP32 inner CG in FP64
    refinement) stop at the relative residual ||b - A x|| / ||b|| <= tol."""

    def __init__(self, grid, method="minres", tol=None, itmax=None, verbose=False):
        self.grid = grid
        self.method = method
        ref = method == "minres"
        self.tol = float(tol if tol is not None else (1e-6 if ref else 1e-8))
        self.itmax = int(itmax if itmax is not None else (1000 if ref else 10000))
        self.verbose = verbose
        self.last_stats = []

    def configure(self):
        g = self.grid
        _check(g, _lib.load().lv_set_solver(g._ctx, _lib.METHODS[self.method], self.tol, self.itmax))


def find_pressure(solver, dt, niter=10, boundary_velocity=None, stats=True):
    """find_pressure!(solver, dt, niter; boundary_velocity) (src/pressure.jl:215-224).
    boundary_velocity is the reference's closure boundary_velocity(x, label)
    -> (vx, vy), evaluated here at every boundary edge's midpoint
    (pressure.jl:182); or a constant velocity per label (a dict {label:
    (vx, vy)} or a closure of the label alone); None or zero_vbc for zero.
    Returns per-sweep (iterations, converged, rel_residual, method used,
    refinement steps) when stats=True (which synchronises); stats=False
    queues the work and returns None."""
    g = solver.grid
    solver.configure()
    L = _lib.load()
    st = (LvSolveStats * niter)() if stats else None
    if boundary_velocity is zero_vbc:
        boundary_velocity = None
    if callable(boundary_velocity) and _per_edge(boundary_velocity) >= 2:
        mid, lab = g.boundary_edges()
        vb = np.ascontiguousarray(np.array([boundary_velocity(m, int(l)) for m, l in zip(mid, lab)],
                                           dtype=np.float64).reshape(-1, 2))
        _check(g, L.lv_find_pressure_edges(g._ctx, float(dt), int(niter), len(mid), _lib.ptr(vb), st))
    else:
        vbc = wall_velocity_table(boundary_velocity)
        _check(g, L.lv_find_pressure(g._ctx, float(dt), int(niter), _lib.ptr(vbc), st))
    if stats:
        solver.last_stats = [(s.iterations, bool(s.converged), s.rel_residual, s.method, s.outer) for s in st]
        if solver.verbose:
            print(solver.last_stats)
        return solver.last_stats
    return None


class MultiphaseSolver:
    """MultiphaseSolver(grid; quality_threshold = 0.25) (src/relaxation.jl:137-153)."""

    def __init__(self, grid, quality_threshold=0.25):
        self.grid = grid
        self.quality_threshold = float(quality_threshold)


def multiphase_projection(solver):
    g = solver.grid
    st = LvSolveStats()
    _check(g, _lib.load().lv_multiphase_projection(g._ctx, solver.quality_threshold, C.byref(st)))
    return st.iterations, bool(st.converged)


# ------------------------------------------------------------- populate

def _populate(grid, pts):
    grid.push(pts)
    remesh(grid)


def populate_jittered(grid, nx, ny, jitter=0.1, seed=12345):
    """Seeded jittered lattice (nx*ny seeds, U(-jitter*h, jitter*h)), then remesh."""
    _populate(grid, _pop.jittered_lattice(grid.rect.xlims, grid.rect.ylims, nx, ny, jitter, seed))


def populate_rect(grid, charfun=None):
    _populate(grid, _pop.rect_seeds(grid.rect.xlims, grid.rect.ylims, grid.dr, charfun))


def populate_hex(grid, charfun=None):
    _populate(grid, _pop.hex_seeds(grid.rect.xlims, grid.rect.ylims, grid.dr, charfun))


def populate_circ(grid, center=(0.0, 0.0), charfun=None):
    _populate(grid, _pop.circ_seeds(grid.rect.xlims, grid.rect.ylims, grid.dr, center, charfun))


def populate_rand(grid, seed=1, charfun=None):
    _populate(grid, _pop.rand_seeds(grid.rect.xlims, grid.rect.ylims, grid.dr, seed, charfun))


def populate_vogel(grid, center=(0.0, 0.0), charfun=None):
    _populate(grid, _pop.vogel_seeds(grid.rect.xlims, grid.rect.ylims, grid.dr, center, charfun))


def populate_lloyd(grid, niterations=100, seed=1, charfun=None):
    """populate_lloyd! (src/populate.jl:118-139): random seeds moved to their
    cell centroids niterations times, each time remeshed on the GPU."""
    populate_rand(grid, seed, charfun)
    for _ in range(niterations):
        grid["x"] = grid["centroid"]
        remesh(grid)


from .vtkio import export_grid, export_points, run  # noqa: E402  (src/IO.jl, src/simulation.jl)
from .movingls import (LinearExpansion, QuadraticExpansion, CubicExpansion, gaussian_kernel,  # noqa: E402
                       power_vector, poly_eval, nearest_polygon, movingls, point_value, integral)
