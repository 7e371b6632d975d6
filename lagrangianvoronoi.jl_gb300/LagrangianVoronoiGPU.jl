"""
    LagrangianVoronoiGPU

Julia front end of liblvgpu.so, the GB300 implementation of the per-timestep
path of LagrangianVoronoi.jl.  It keeps the reference's names, arguments and
keyword arguments (src/LagrangianVoronoi.jl:14-69) for what a `step!` and its
set-up call:

    grid = GridNS(UnitRectangle(), dr; xperiodic = true, yperiodic = true)
    populate_hex!(grid; ic! = ic!)
    solver = PressureSolver(grid)
    function step!(sim, t)
        move!(grid, dt); stiffened_eos!(grid, gamma, P0); find_pressure!(solver, dt)
        pressure_step!(grid, dt); find_D!(grid); viscous_step!(grid, dt)
        find_dv!(grid, dt); relaxation_step!(grid, dt)
    end
    run!(sim, dt, t_end, step!; path = "results", vtp_vars = (:v, :P))

The particle state lives on the GPU.  The closures the reference calls inside
its loops run here on the host: `ic!(p)` once on a host mirror of the
polygons; `boundary_velocity(x, label)`, `vDirichlet(x)` and `charfun(x)` at
the midpoint of every boundary edge (lv_get_boundary_edges), whose values are
then passed per edge.  `polygons(grid)` downloads a host mirror for
`postproc!` code that reads `p.v`, `area(p)`, `centroid(p)` or iterates
`neighbors(p, mirror)` / `boundaries(p)`.

Errors map to the reference's throws: a NaN velocity raises
"Velocity field invalidated." (move.jl:25) and a mesh whose candidate search
passes r_max raises "The Voronoi Mesh has been destroyed." (voronoigrid.jl:64).

Julia is not installed on the build or test machines of this repository, so
this file is not exercised by its test suite; the same C ABI is exercised
through Python ctypes in tests/ (lagrangianvoronoi.jl_gb300/__init__.py is
the same front end in Python).
"""
module LagrangianVoronoiGPU

using LinearAlgebra: norm

const libpath = joinpath(@__DIR__, "liblvgpu.so")

export Rectangle, UnitRectangle, VoronoiPolygon, PolygonNS, VoronoiGrid, GridNS, Edge,
    BDARY_UP, BDARY_RIGHT, BDARY_DOWN, BDARY_LEFT,
    remesh!, move!, ideal_eos!, stiffened_eos!, find_rho!, gravity_step!, PressureSolver, find_pressure!, zero_vbc,
    pressure_step!, find_D!, viscous_step!, bdary_friction!, find_dv!, relaxation_step!, MultiphaseSolver,
    multiphase_projection!, populate_rect!, populate_hex!, populate_circ!, populate_rand!, populate_vogel!,
    populate_lloyd!, polygons, upload!, neighbors, boundaries, area, centroid, SimulationWorkspace, run!, field, field!

const BDARY_UP = -1
const BDARY_RIGHT = -2
const BDARY_DOWN = -3
const BDARY_LEFT = -4

# ---------------------------------------------------------------- C types

struct LvParams  # lv_params, include/lvgpu.h
    xmin::NTuple{2,Float64}
    xmax::NTuple{2,Float64}
    dr::Float64
    h::Float64
    r_max::Float64
    xperiodic::Int32
    yperiodic::Int32
    capacity::Int32
    device::Int32
end

struct LvSolveStats  # lv_solve_stats
    iterations::Int32
    converged::Int32
    outer::Int32
    method::Int32
    rel_residual::Float64
end

const MESSAGES = Dict(1 => "Velocity field invalidated.", 2 => "The Voronoi Mesh has been destroyed.")
const FIELDS = Dict(:x => (0, 2), :v => (1, 2), :e => (2, 1), :P => (3, 1), :rho => (4, 1), :c2 => (5, 1),
    :dv => (6, 2), :mass => (7, 1), :momentum => (8, 2), :energy => (9, 1), :phase => (10, 1),
    :quality => (11, 1), :D => (12, 4), :mu => (13, 1), :area => (20, 1), :centroid => (21, 2))
const METHODS = Dict(:jacobi_pcg => 0, :mixed_ir => 1, :learned_pcg => 2, :minres => 3)
const LV_MAX_EDGES = 20

# ---------------------------------------------------------------- domain

"""
    Rectangle(xlims, ylims)

The boundary rectangle (geometry.jl:94-111).
"""
struct Rectangle
    xmin::NTuple{2,Float64}
    xmax::NTuple{2,Float64}
end
Rectangle(xlims::Tuple{<:Real,<:Real}, ylims::Tuple{<:Real,<:Real}) =
    Rectangle((Float64(xlims[1]), Float64(ylims[1])), (Float64(xlims[2]), Float64(ylims[2])))
UnitRectangle() = Rectangle((0.0, 1.0), (0.0, 1.0))
isinside(r::Rectangle, x) = r.xmin[1] <= x[1] <= r.xmax[1] && r.xmin[2] <= x[2] <= r.xmax[2]

abstract type VoronoiPolygon end
"The Navier-Stokes polygon (celldefs.jl:7-41); on the GPU its fields are the device state."
struct PolygonNS <: VoronoiPolygon end

"""
    VoronoiGrid{T}(rect, dr; h = 2dr, r_max = 10dr, xperiodic = false, yperiodic = false)

The grid of the reference (voronoigrid.jl:14-50), its state on the GPU.
`capacity` bounds the particle count (default: the count of the first
remesh!); `push!(grid, x)` adds a seed as `push!(grid.polygons, T(x = x))`
does.
"""
mutable struct VoronoiGrid{T<:VoronoiPolygon}
    ctx::Ptr{Cvoid}
    n::Int
    boundary_rect::Rectangle
    dr::Float64
    h::Float64
    r_max::Float64
    xperiodic::Bool
    yperiodic::Bool
    capacity::Int
    device::Int
    pending::Vector{NTuple{2,Float64}}
end

function VoronoiGrid{T}(rect::Rectangle, dr::Float64; h::Float64 = 2dr, r_max::Float64 = 10dr,
                        xperiodic::Bool = false, yperiodic::Bool = false, capacity::Integer = 0,
                        device::Integer = 0) where {T<:VoronoiPolygon}
    grid = VoronoiGrid{T}(C_NULL, 0, rect, dr, h, r_max, xperiodic, yperiodic, capacity, device,
                          NTuple{2,Float64}[])
    finalizer(grid) do g
        g.ctx != C_NULL && ccall((:lv_destroy, libpath), Cint, (Ptr{Cvoid},), g.ctx)
    end
    return grid
end

const GridNS = VoronoiGrid{PolygonNS}

function check(grid::VoronoiGrid, rc::Integer)
    rc == 0 && return
    msg = get(MESSAGES, Int(rc)) do
        unsafe_string(ccall((:lv_last_error, libpath), Cstring, (Ptr{Cvoid},), grid.ctx))
    end
    throw(ErrorException(msg))
end

Base.push!(grid::VoronoiGrid, x) = (push!(grid.pending, (Float64(x[1]), Float64(x[2]))); grid)

# the seeds pushed since the last remesh! join the particle set
function flush!(grid::VoronoiGrid)
    isempty(grid.pending) && return
    old = grid.n > 0 ? field(grid, :x) : zeros(2, 0)
    x = hcat(old, reduce(hcat, [[p[1], p[2]] for p in grid.pending]))
    empty!(grid.pending)
    n = size(x, 2)
    if grid.ctx == C_NULL
        cap = max(grid.capacity, n)
        p = Ref(LvParams(grid.boundary_rect.xmin, grid.boundary_rect.xmax, grid.dr, grid.h, grid.r_max,
                         grid.xperiodic, grid.yperiodic, cap, grid.device))
        grid.ctx = ccall((:lv_create, libpath), Ptr{Cvoid}, (Ref{LvParams},), p)
        grid.ctx == C_NULL && error("lv_create failed (no CUDA device or out of memory)")
        grid.capacity = cap
    end
    check(grid, ccall((:lv_set_positions, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), grid.ctx, n, x))
    grid.n = n
end

"""
    field(grid, name) / field!(grid, name, values)

One field of every particle (names of celldefs.jl: :x, :v, :e, :P, :rho, :c2,
:dv, :mass, :momentum, :energy, :phase, :quality, :D, :mu; read-only :area,
:centroid); vector fields are 2×n matrices, D a 4×n matrix.
"""
function field(grid::VoronoiGrid, name::Symbol)
    id, k = FIELDS[name]
    a = Vector{Float64}(undef, k * grid.n)
    check(grid, ccall((:lv_get_field, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), grid.ctx, id, a))
    return k == 1 ? a : reshape(a, k, grid.n)
end

function field!(grid::VoronoiGrid, name::Symbol, values::AbstractArray{<:Real})
    id, _ = FIELDS[name]
    a = Vector{Float64}(vec(values))
    check(grid, ccall((:lv_set_field, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), grid.ctx, id, a))
end

# ---------------------------------------------------------------- steps

remesh!(g::VoronoiGrid) = (flush!(g); check(g, ccall((:lv_remesh, libpath), Cint, (Ptr{Cvoid},), g.ctx)))
move!(g::VoronoiGrid, dt::Float64) = check(g, ccall((:lv_move, libpath), Cint, (Ptr{Cvoid}, Float64), g.ctx, dt))
ideal_eos!(g::VoronoiGrid, gamma::Float64 = 1.4; Pmin::Float64 = 0.0) =
    check(g, ccall((:lv_ideal_eos, libpath), Cint, (Ptr{Cvoid}, Float64, Float64), g.ctx, gamma, Pmin))
stiffened_eos!(g::VoronoiGrid, gamma::Float64 = 1.4, P0::Float64 = 0.0) =
    check(g, ccall((:lv_stiffened_eos, libpath), Cint, (Ptr{Cvoid}, Float64, Float64), g.ctx, gamma, P0))
find_rho!(g::VoronoiGrid) = check(g, ccall((:lv_find_rho, libpath), Cint, (Ptr{Cvoid},), g.ctx))
gravity_step!(g::VoronoiGrid, gv, dt::Float64) =
    check(g, ccall((:lv_gravity_step, libpath), Cint, (Ptr{Cvoid}, Float64, Float64, Float64), g.ctx, gv[1], gv[2], dt))
pressure_step!(g::VoronoiGrid, dt::Float64) =
    check(g, ccall((:lv_pressure_step, libpath), Cint, (Ptr{Cvoid}, Float64), g.ctx, dt))
find_D!(g::VoronoiGrid) = check(g, ccall((:lv_find_D, libpath), Cint, (Ptr{Cvoid},), g.ctx))
viscous_step!(g::VoronoiGrid, dt::Float64; artificial_viscosity::Bool = true) =
    check(g, ccall((:lv_viscous_step, libpath), Cint, (Ptr{Cvoid}, Float64, Int32), g.ctx, dt, artificial_viscosity))
find_dv!(g::VoronoiGrid, dt::Float64, alpha::Float64 = 1.0) =
    check(g, ccall((:lv_find_dv, libpath), Cint, (Ptr{Cvoid}, Float64, Float64), g.ctx, dt, alpha))
relaxation_step!(g::VoronoiGrid, dt::Float64; rusanov::Bool = true) =
    check(g, ccall((:lv_relaxation_step, libpath), Cint, (Ptr{Cvoid}, Float64, Int32), g.ctx, dt, rusanov))

# midpoints (2×nb) and labels of the boundary edges, in the per-edge order
function boundary_edges(g::VoronoiGrid)
    nb = Ref{Int64}(0)
    check(g, ccall((:lv_get_boundary_edges, libpath), Cint, (Ptr{Cvoid}, Ref{Int64}, Ptr{Float64}, Ptr{Int32}),
                   g.ctx, nb, C_NULL, C_NULL))
    mid = zeros(2, nb[])
    lab = zeros(Int32, nb[])
    nb[] > 0 && check(g, ccall((:lv_get_boundary_edges, libpath), Cint,
                               (Ptr{Cvoid}, Ptr{Int64}, Ptr{Float64}, Ptr{Int32}), g.ctx, C_NULL, mid, lab))
    return mid, lab
end

_everywhere(x) = true

"""
    bdary_friction!(grid, vDirichlet, dt; charfun = x -> true)

diffusion.jl:64-79: `vDirichlet(m)` and `charfun(m)` are evaluated at the
midpoint m of every boundary edge.
"""
function bdary_friction!(g::VoronoiGrid, vDirichlet::Function, dt::Float64; charfun::Function = _everywhere)
    mid, _ = boundary_edges(g)
    nb = size(mid, 2)
    vb = zeros(2, nb)
    act = ones(UInt8, nb)
    for q in 1:nb
        m = (mid[1, q], mid[2, q])
        v = vDirichlet(m)
        vb[1, q] = v[1]
        vb[2, q] = v[2]
        act[q] = charfun(m) ? 0x01 : 0x00
    end
    check(g, ccall((:lv_bdary_friction_edges, libpath), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{UInt8}, Float64),
                   g.ctx, nb, vb, act, dt))
end

"""
    PressureSolver(grid; method = :minres, tol, itmax)

pressure.jl:142-159.  The default is the reference's own solve (:minres,
atol = rtol = 1e-6, itmax = 1000, warm-started from P); :jacobi_pcg (FP64),
:mixed_ir and :learned_pcg (FP32 inner CG in FP64 refinement) stop at
||b - A x|| <= tol ||b|| (default 1e-8).
"""
struct PressureSolver{T}
    grid::VoronoiGrid{T}
    method::Int32
    tol::Float64
    itmax::Int32
end

function PressureSolver(grid::VoronoiGrid{T}; method::Symbol = :minres, tol::Union{Nothing,Float64} = nothing,
                        itmax::Union{Nothing,Integer} = nothing) where {T}
    ref = method == :minres
    return PressureSolver{T}(grid, METHODS[method], something(tol, ref ? 1e-6 : 1e-8),
                             something(itmax, ref ? 1000 : 10000))
end

"The default boundary velocity of find_pressure! (pressure.jl:205-207)."
zero_vbc(x, label::Integer) = (0.0, 0.0)

"""
    find_pressure!(solver, dt, niter = 10; boundary_velocity = zero_vbc)

pressure.jl:215-224; `boundary_velocity(midpoint(e), e.label)` is evaluated
per boundary edge.  Returns the per-sweep statistics.
"""
function find_pressure!(s::PressureSolver, dt::Float64, niter::Integer = 10; boundary_velocity::Function = zero_vbc)
    g = s.grid
    check(g, ccall((:lv_set_solver, libpath), Cint, (Ptr{Cvoid}, Int32, Float64, Int32), g.ctx, s.method, s.tol,
                   s.itmax))
    stats = Vector{LvSolveStats}(undef, niter)
    if boundary_velocity === zero_vbc
        check(g, ccall((:lv_find_pressure, libpath), Cint,
                       (Ptr{Cvoid}, Float64, Int32, Ptr{Float64}, Ptr{LvSolveStats}), g.ctx, dt, niter, C_NULL, stats))
    else
        mid, lab = boundary_edges(g)
        nb = size(mid, 2)
        vb = zeros(2, nb)
        for q in 1:nb
            v = boundary_velocity((mid[1, q], mid[2, q]), Int(lab[q]))
            vb[1, q] = v[1]
            vb[2, q] = v[2]
        end
        check(g, ccall((:lv_find_pressure_edges, libpath), Cint,
                       (Ptr{Cvoid}, Float64, Int32, Int64, Ptr{Float64}, Ptr{LvSolveStats}),
                       g.ctx, dt, niter, nb, vb, stats))
    end
    return stats
end

"MultiphaseSolver(grid; quality_threshold = 0.25) (relaxation.jl:137-153)."
struct MultiphaseSolver{T}
    grid::VoronoiGrid{T}
    quality_threshold::Float64
end
MultiphaseSolver(grid::VoronoiGrid{T}; quality_threshold::Float64 = 0.25) where {T} =
    MultiphaseSolver{T}(grid, quality_threshold)

function multiphase_projection!(s::MultiphaseSolver)
    st = Ref{LvSolveStats}()
    check(s.grid, ccall((:lv_multiphase_projection, libpath), Cint, (Ptr{Cvoid}, Float64, Ref{LvSolveStats}),
                        s.grid.ctx, s.quality_threshold, st))
    return st[]
end

# ---------------------------------------------------------------- host mirror

"An edge of a polygon (geometry.jl): end points and the label (neighbour index, or a BDARY_* value)."
struct Edge
    v1::NTuple{2,Float64}
    v2::NTuple{2,Float64}
    label::Int
end

"""
One polygon of a host mirror: the PolygonNS fields (celldefs.jl:7-41), its
edges and its geometry.  `ic!(p)` and `postproc!` code read and write these.
"""
mutable struct HostPolygon
    index::Int
    x::NTuple{2,Float64}
    v::NTuple{2,Float64}
    dv::NTuple{2,Float64}
    momentum::NTuple{2,Float64}
    e::Float64
    P::Float64
    rho::Float64
    c2::Float64
    mass::Float64
    energy::Float64
    quality::Float64
    mu::Float64
    phase::Int
    D::NTuple{4,Float64}
    area::Float64
    centroid::NTuple{2,Float64}
    edges::Vector{Edge}
end

area(p::HostPolygon) = p.area
centroid(p::HostPolygon) = p.centroid
boundaries(p::HostPolygon) = (e for e in p.edges if e.label < 0)

struct HostMirror
    polygons::Vector{HostPolygon}
    xperiodic::Bool
    yperiodic::Bool
    period::NTuple{2,Float64}
end

"""
    polygons(grid) -> mirror

Downloads every polygon (fields, edges, area, centroid) into a host mirror;
`mirror.polygons[i]`, `neighbors(p, mirror)`.  `upload!(grid, mirror)` sends
the fields back.
"""
function polygons(g::VoronoiGrid)
    n = g.n
    f = Dict(k => field(g, k) for k in (:x, :v, :dv, :momentum, :e, :P, :rho, :c2, :mass, :energy, :quality, :mu,
                                          :phase, :D, :area, :centroid))
    cnt = zeros(Int32, n)
    verts = zeros(4, LV_MAX_EDGES, n)
    labels = zeros(Int32, LV_MAX_EDGES, n)
    check(g, ccall((:lv_get_geometry, libpath), Cint, (Ptr{Cvoid}, Ptr{Int32}, Ptr{Float64}, Ptr{Int32}),
                   g.ctx, cnt, verts, labels))
    v2(a, i) = (a[1, i], a[2, i])
    ps = Vector{HostPolygon}(undef, n)
    for i in 1:n
        edges = [Edge((verts[1, k, i], verts[2, k, i]), (verts[3, k, i], verts[4, k, i]),
                      labels[k, i] >= 0 ? Int(labels[k, i]) + 1 : Int(labels[k, i])) for k in 1:cnt[i]]
        D = f[:D]
        ps[i] = HostPolygon(i, v2(f[:x], i), v2(f[:v], i), v2(f[:dv], i), v2(f[:momentum], i), f[:e][i], f[:P][i],
                            f[:rho][i], f[:c2][i], f[:mass][i], f[:energy][i], f[:quality][i], f[:mu][i],
                            round(Int, f[:phase][i]), (D[1, i], D[2, i], D[3, i], D[4, i]), f[:area][i],
                            v2(f[:centroid], i), edges)
    end
    rect = g.boundary_rect
    return HostMirror(ps, g.xperiodic, g.yperiodic, (rect.xmax[1] - rect.xmin[1], rect.xmax[2] - rect.xmin[2]))
end

function upload!(g::VoronoiGrid, m::HostMirror)
    ps = m.polygons
    vec2(getter) = reduce(hcat, [[getter(p)[1], getter(p)[2]] for p in ps])
    field!(g, :v, vec2(p -> p.v))
    field!(g, :dv, vec2(p -> p.dv))
    field!(g, :momentum, vec2(p -> p.momentum))
    for k in (:e, :P, :rho, :c2, :mass, :energy, :quality, :mu)
        field!(g, k, [getfield(p, k) for p in ps])
    end
    field!(g, :phase, Float64[p.phase for p in ps])
    field!(g, :D, reduce(hcat, [collect(p.D) for p in ps]))
end

# get_arrow (voronoigrid.jl:116-125): the minimum-image vector from b to a
function arrow(m::HostMirror, a, b)
    v = [a[1] - b[1], a[2] - b[2]]
    if m.xperiodic && abs(v[1]) > 0.5 * m.period[1]
        v[1] -= sign(v[1]) * m.period[1]
    end
    if m.yperiodic && abs(v[2]) > 0.5 * m.period[2]
        v[2] -= sign(v[2]) * m.period[2]
    end
    return (v[1], v[2])
end

"""
    neighbors(p, mirror)

iterators.jl:19-33: `(q, e, y)` for every edge of `p` with a neighbour: the
neighbour polygon, the edge and the neighbour's position seen from `p`.
"""
function neighbors(p::HostPolygon, m::HostMirror)
    out = Tuple{HostPolygon,Edge,NTuple{2,Float64}}[]
    for e in p.edges
        e.label > 0 || continue
        q = m.polygons[e.label]
        a = arrow(m, q.x, p.x)
        push!(out, (q, e, (p.x[1] + a[1], p.x[2] + a[2])))
    end
    return out
end

# ---------------------------------------------------------------- populate (populate.jl)

_noop(p) = nothing

function finish_populate!(grid::VoronoiGrid, ic!::Function)
    remesh!(grid)
    if ic! !== _noop
        m = polygons(grid)
        foreach(ic!, m.polygons)
        upload!(grid, m)
    end
end

function add_seeds!(grid::VoronoiGrid, pts, charfun::Function)
    for x in pts
        if charfun(x) && isinside(grid.boundary_rect, x)
            push!(grid, x)
        end
    end
end

"populate_rect!(grid; charfun, ic!) (populate.jl:45-62)."
function populate_rect!(grid::VoronoiGrid; charfun::Function = _everywhere, ic!::Function = _noop)
    r = grid.boundary_rect
    N = round(Int, (r.xmax[1] - r.xmin[1]) / grid.dr)
    M = round(Int, (r.xmax[2] - r.xmin[2]) / grid.dr)
    pts = [(x1 + 0.5grid.dr, x2 + 0.5grid.dr) for x1 in range(r.xmin[1], r.xmax[1], length = N)
           for x2 in range(r.xmin[2], r.xmax[2], length = M)]
    add_seeds!(grid, pts, charfun)
    finish_populate!(grid, ic!)
end

"populate_hex!(grid; charfun, ic!) (populate.jl:155-179)."
function populate_hex!(grid::VoronoiGrid; charfun::Function = _everywhere, ic!::Function = _noop)
    r = grid.boundary_rect
    a = (4.0 / 3.0)^0.25 * grid.dr
    b = (3.0 / 4.0)^0.25 * grid.dr
    pts = NTuple{2,Float64}[]
    for i in (floor(Int, r.xmin[1] / a) - 1):ceil(Int, r.xmax[1] / a), j in floor(Int, r.xmin[2] / b):ceil(Int, r.xmax[2] / b)
        push!(pts, ((i + (j % 2) / 2) * a, j * b))
    end
    add_seeds!(grid, pts, charfun)
    finish_populate!(grid, ic!)
end

_corner_radius(r::Rectangle, c) = maximum(norm([x[1] - c[1], x[2] - c[2]]) for x in
    (r.xmin, (r.xmin[1], r.xmax[2]), r.xmax, (r.xmax[1], r.xmin[2])))

"populate_circ!(grid; charfun, center, ic!) (populate.jl:18-35)."
function populate_circ!(grid::VoronoiGrid; charfun::Function = _everywhere, center = (0.0, 0.0),
                        ic!::Function = _noop)
    rmax = _corner_radius(grid.boundary_rect, center)
    pts = NTuple{2,Float64}[]
    for r in (0.5grid.dr):grid.dr:rmax
        kmax = round(Int, 2pi * r / grid.dr)
        for k in 1:kmax
            th = 2pi * k / kmax
            push!(pts, (center[1] + r * cos(th), center[2] + r * sin(th)))
        end
    end
    add_seeds!(grid, pts, charfun)
    finish_populate!(grid, ic!)
end

"populate_rand!(grid; charfun, ic!) (populate.jl:75-91)."
function populate_rand!(grid::VoronoiGrid; charfun::Function = _everywhere, ic!::Function = _noop)
    r = grid.boundary_rect
    N = round(Int, abs(r.xmax[1] - r.xmin[1]) * abs(r.xmax[2] - r.xmin[2]) / grid.dr^2)
    pts = NTuple{2,Float64}[]
    for _ in 1:N
        u, w = rand(), rand()
        push!(pts, (u * r.xmax[1] + (1 - u) * r.xmin[1], w * r.xmax[2] + (1 - w) * r.xmin[2]))
    end
    add_seeds!(grid, pts, charfun)
    finish_populate!(grid, ic!)
end

"populate_vogel!(grid; charfun, center, ic!) (populate.jl:105-121)."
function populate_vogel!(grid::VoronoiGrid; charfun::Function = _everywhere, center = (0.0, 0.0),
                         ic!::Function = _noop)
    rmax = _corner_radius(grid.boundary_rect, center)
    N = round(Int, pi * rmax^2 / grid.dr^2)
    golden = pi * (3 - sqrt(5))
    pts = [(center[1] + rmax * sqrt(i / N) * cos(golden * i), center[2] + rmax * sqrt(i / N) * sin(golden * i))
           for i in 1:N]
    add_seeds!(grid, pts, charfun)
    finish_populate!(grid, ic!)
end

"populate_lloyd!(grid; charfun, niterations, ic!) (populate.jl:132-150): random seeds moved to their centroids."
function populate_lloyd!(grid::VoronoiGrid; charfun::Function = _everywhere, niterations::Int = 100,
                         ic!::Function = _noop)
    populate_rand!(grid; charfun = charfun)
    for _ in 1:niterations
        field!(grid, :x, field(grid, :centroid))
        remesh!(grid)
    end
    if ic! !== _noop
        m = polygons(grid)
        foreach(ic!, m.polygons)
        upload!(grid, m)
    end
end

# ---------------------------------------------------------------- run! (simulation.jl:35-94)

abstract type SimulationWorkspace end
donothing(sim, t) = nothing

# one frame of the cells as VTK XML PolyData (ASCII), the per-polygon fields as cell data
function export_grid(grid::VoronoiGrid, filename::String, vars::Symbol...)
    m = polygons(grid)
    pts = Float64[]
    conn = Int[]
    offs = Int[]
    for p in m.polygons
        for e in p.edges
            append!(pts, (e.v1[1], e.v1[2], 0.0))
            push!(conn, length(conn))
        end
        push!(offs, length(conn))
    end
    open(filename, "w") do io
        println(io, "<?xml version=\"1.0\"?>\n<VTKFile type=\"PolyData\" version=\"1.0\" byte_order=\"LittleEndian\">")
        println(io, "<PolyData><Piece NumberOfPoints=\"$(length(pts) ÷ 3)\" NumberOfPolys=\"$(length(offs))\">")
        println(io, "<Points><DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">",
                join(pts, ' '), "</DataArray></Points>")
        println(io, "<Polys><DataArray type=\"Int64\" Name=\"connectivity\" format=\"ascii\">", join(conn, ' '),
                "</DataArray><DataArray type=\"Int64\" Name=\"offsets\" format=\"ascii\">", join(offs, ' '),
                "</DataArray></Polys>")
        println(io, "<CellData>")
        for v in vars
            a = field(grid, v)
            if ndims(a) == 1
                println(io, "<DataArray type=\"Float64\" Name=\"$v\" format=\"ascii\">", join(a, ' '), "</DataArray>")
            else
                b = vcat(a[1:2, :], zeros(1, size(a, 2)))
                println(io, "<DataArray type=\"Float64\" Name=\"$v\" NumberOfComponents=\"3\" format=\"ascii\">",
                        join(b, ' '), "</DataArray>")
            end
        end
        println(io, "</CellData></Piece></PolyData></VTKFile>")
    end
    return filename
end

"""
    run!(sim, dt, t_end, step!; nframes = 100, path = "results", save_grid = true, save_csv = true,
         vtp_vars = Symbol[], csv_vars = Symbol[], postproc! = donothing)

The time-marching loop of simulation.jl:35-94: `step!(sim, t)` every step;
every `t_end / (nframes dt)` steps `postproc!(sim, t)`, a frame of `sim.grid`
(`path/cframe<k>.vtp`, listed in `path/cells.pvd`) and a row of `csv_vars` in
`path/simdata.csv`.
"""
function run!(sim::SimulationWorkspace, dt::Float64, t_end::Float64, step!::Function; nframes::Int = 100,
              path::String = "results", save_points::Bool = false, save_grid::Bool = true, save_csv::Bool = true,
              vtp_vars = Symbol[], csv_vars = Symbol[], postproc!::Function = donothing)
    ispath(path) || mkpath(path)
    k_frame = nframes > 0 ? max(round(Int, t_end / (nframes * dt)), 1) : typemax(Int)
    rows = Vector{Vector{Float64}}()
    frames = Tuple{Float64,String}[]
    k = 0
    nframe = 0
    t = 0.0
    while t < t_end
        k += 1
        step!(sim, t)
        if k % k_frame == 0
            postproc!(sim, t)
            push!(rows, vcat(t, Float64[getproperty(sim, v) for v in csv_vars]))
            if save_grid
                push!(frames, (t, export_grid(sim.grid, joinpath(path, "cframe$(nframe).vtp"), vtp_vars...)))
            end
            nframe += 1
        end
        t += dt
    end
    if save_grid
        open(joinpath(path, "cells.pvd"), "w") do io
            println(io, "<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"1.0\"><Collection>")
            for (tt, f) in frames
                println(io, "<DataSet timestep=\"$tt\" file=\"$(basename(f))\"/>")
            end
            println(io, "</Collection></VTKFile>")
        end
    end
    if save_csv
        open(joinpath(path, "simdata.csv"), "w") do io
            println(io, join(vcat("time", string.(csv_vars)), ','))
            foreach(r -> println(io, join(r, ',')), rows)
        end
    end
    return
end

end # module
