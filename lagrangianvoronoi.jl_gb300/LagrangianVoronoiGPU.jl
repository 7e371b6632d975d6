"""
    LagrangianVoronoiGPU

Julia front end of liblvgpu.so: the per-timestep functions of
LagrangianVoronoi.jl (`remesh!`, `move!`, `*_eos!`, `find_pressure!`,
`pressure_step!`, `find_D!`, `viscous_step!`, `bdary_friction!`, `find_dv!`,
`relaxation_step!`) with the reference's names and arguments, forwarded to the
GB300 library through `ccall`.  The particle state lives on the GPU; `getfield`
style access goes through `field(grid, :v)` / `setfield!(grid, :v, values)`.

Errors map to the reference's throws: a NaN velocity raises
"Velocity field invalidated." (move.jl:25) and a mesh whose candidate search
passes r_max raises "The Voronoi Mesh has been destroyed." (voronoigrid.jl:64).

Julia is not installed on the build or test machines of this repository, so
this file is not exercised by its test suite; the same C ABI is exercised
through Python ctypes in tests/.
"""
module LagrangianVoronoiGPU

const libpath = joinpath(@__DIR__, "liblvgpu.so")

export VoronoiGridGPU, remesh!, move!, ideal_eos!, stiffened_eos!, find_rho!, gravity_step!, PressureSolverGPU,
    find_pressure!, pressure_step!, find_D!, viscous_step!, bdary_friction!, find_dv!, relaxation_step!,
    field, setfield!, populate_positions!

struct LvParams
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

struct LvSolveStats
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

mutable struct VoronoiGridGPU
    ctx::Ptr{Cvoid}
    n::Int
    dr::Float64
end

function check(grid::VoronoiGridGPU, rc::Integer)
    rc == 0 && return
    msg = get(MESSAGES, Int(rc), unsafe_string(ccall((:lv_last_error, libpath), Cstring, (Ptr{Cvoid},), grid.ctx)))
    throw(msg)
end

"""
    VoronoiGridGPU(xlims, ylims, dr; h = 2dr, r_max = 10dr, xperiodic = false, yperiodic = false, capacity)

Counterpart of `VoronoiGrid{T}(rect, dr; h, r_max, xperiodic, yperiodic)` (voronoigrid.jl:14-50).
"""
function VoronoiGridGPU(xlims, ylims, dr::Float64; h = 2dr, r_max = 10dr, xperiodic::Bool = false,
                        yperiodic::Bool = false, capacity::Integer, device::Integer = 0)
    p = Ref(LvParams((xlims[1], ylims[1]), (xlims[2], ylims[2]), dr, h, r_max, xperiodic, yperiodic, capacity,
                     device))
    ctx = ccall((:lv_create, libpath), Ptr{Cvoid}, (Ref{LvParams},), p)
    ctx == C_NULL && error("lv_create failed")
    grid = VoronoiGridGPU(ctx, 0, dr)
    finalizer(g -> ccall((:lv_destroy, libpath), Cint, (Ptr{Cvoid},), g.ctx), grid)
    return grid
end

"""
    populate_positions!(grid, x::Matrix{Float64})

`push!(grid.polygons, T(x = x[:, i]))` for every column of the 2×n matrix `x`, then `remesh!`.
"""
function populate_positions!(grid::VoronoiGridGPU, x::Matrix{Float64})
    n = size(x, 2)
    check(grid, ccall((:lv_set_positions, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), grid.ctx, n, x))
    grid.n = n
    remesh!(grid)
end

function field(grid::VoronoiGridGPU, name::Symbol)
    id, k = FIELDS[name]
    a = Vector{Float64}(undef, k * grid.n)
    check(grid, ccall((:lv_get_field, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), grid.ctx, id, a))
    return k == 1 ? a : reshape(a, k, grid.n)
end

function setfield!(grid::VoronoiGridGPU, name::Symbol, values::AbstractArray{Float64})
    id, _ = FIELDS[name]
    a = collect(values)
    check(grid, ccall((:lv_set_field, libpath), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), grid.ctx, id, a))
end

remesh!(g::VoronoiGridGPU) = check(g, ccall((:lv_remesh, libpath), Cint, (Ptr{Cvoid},), g.ctx))
move!(g::VoronoiGridGPU, dt::Float64) = check(g, ccall((:lv_move, libpath), Cint, (Ptr{Cvoid}, Float64), g.ctx, dt))
ideal_eos!(g::VoronoiGridGPU, gamma::Float64 = 1.4; Pmin::Float64 = 0.0) =
    check(g, ccall((:lv_ideal_eos, libpath), Cint, (Ptr{Cvoid}, Float64, Float64), g.ctx, gamma, Pmin))
stiffened_eos!(g::VoronoiGridGPU, gamma::Float64 = 1.4, P0::Float64 = 0.0) =
    check(g, ccall((:lv_stiffened_eos, libpath), Cint, (Ptr{Cvoid}, Float64, Float64), g.ctx, gamma, P0))
find_rho!(g::VoronoiGridGPU) = check(g, ccall((:lv_find_rho, libpath), Cint, (Ptr{Cvoid},), g.ctx))
gravity_step!(g::VoronoiGridGPU, gv, dt::Float64) =
    check(g, ccall((:lv_gravity_step, libpath), Cint, (Ptr{Cvoid}, Float64, Float64, Float64), g.ctx, gv[1], gv[2], dt))
pressure_step!(g::VoronoiGridGPU, dt::Float64) =
    check(g, ccall((:lv_pressure_step, libpath), Cint, (Ptr{Cvoid}, Float64), g.ctx, dt))
find_D!(g::VoronoiGridGPU) = check(g, ccall((:lv_find_D, libpath), Cint, (Ptr{Cvoid},), g.ctx))
viscous_step!(g::VoronoiGridGPU, dt::Float64; artificial_viscosity::Bool = true) =
    check(g, ccall((:lv_viscous_step, libpath), Cint, (Ptr{Cvoid}, Float64, Int32), g.ctx, dt, artificial_viscosity))
find_dv!(g::VoronoiGridGPU, dt::Float64, alpha::Float64 = 1.0) =
    check(g, ccall((:lv_find_dv, libpath), Cint, (Ptr{Cvoid}, Float64, Float64), g.ctx, dt, alpha))
relaxation_step!(g::VoronoiGridGPU, dt::Float64; rusanov::Bool = true) =
    check(g, ccall((:lv_relaxation_step, libpath), Cint, (Ptr{Cvoid}, Float64, Int32), g.ctx, dt, rusanov))

# constant wall velocity per boundary label, [4][2] indexed by -label-1
function wall_table(f)
    t = zeros(Float64, 8)
    for lab in (-1, -2, -3, -4)
        v = f(lab)
        t[2(-lab - 1) + 1] = v[1]
        t[2(-lab - 1) + 2] = v[2]
    end
    return t
end

"""
    bdary_friction!(grid, vDirichlet, dt)

`vDirichlet(label)` gives the wall velocity of each side (BDARY_UP = -1, RIGHT = -2, DOWN = -3, LEFT = -4).
"""
bdary_friction!(g::VoronoiGridGPU, vDirichlet::Function, dt::Float64) =
    check(g, ccall((:lv_bdary_friction, libpath), Cint, (Ptr{Cvoid}, Ptr{Float64}, Float64), g.ctx,
                   wall_table(vDirichlet), dt))

struct PressureSolverGPU
    grid::VoronoiGridGPU
    method::Int32
    tol::Float64
    itmax::Int32
end

"""
    PressureSolverGPU(grid; method = :jacobi_pcg, tol = 1e-8, itmax = 10000)

Counterpart of `PressureSolver(grid)` (pressure.jl:142-159); `method` is one of
`:jacobi_pcg`, `:mixed_ir`, `:learned_pcg`.
"""
function PressureSolverGPU(grid::VoronoiGridGPU; method::Symbol = :jacobi_pcg, tol::Float64 = 1e-8,
                           itmax::Integer = 10000)
    m = Dict(:jacobi_pcg => 0, :mixed_ir => 1, :learned_pcg => 2)[method]
    return PressureSolverGPU(grid, m, tol, itmax)
end

zero_vbc(label::Int) = (0.0, 0.0)

function find_pressure!(s::PressureSolverGPU, dt::Float64, niter::Int64 = 10; boundary_velocity::Function = zero_vbc)
    g = s.grid
    check(g, ccall((:lv_set_solver, libpath), Cint, (Ptr{Cvoid}, Int32, Float64, Int32), g.ctx, s.method, s.tol,
                   s.itmax))
    stats = Vector{LvSolveStats}(undef, niter)
    check(g, ccall((:lv_find_pressure, libpath), Cint, (Ptr{Cvoid}, Float64, Int32, Ptr{Float64}, Ptr{LvSolveStats}),
                   g.ctx, dt, niter, wall_table(boundary_velocity), stats))
    return stats
end

end # module
