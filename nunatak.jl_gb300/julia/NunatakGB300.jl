"""
    NunatakGB300

The Julia side of `libnunatak_gb300.so`: the velocity solve of Nunatak.jl's `update_velocities!` (Picard iteration
around preconditioned conjugate gradients for the SSA and DIVA stress balances) on one GB300 GPU, through the C ABI
of `include/nunatak_gb300.h`.  A maintainer loads this module next to Nunatak.jl and passes a
`GB300StressBalanceSolver` as the `linear_solver` of a `StressBalanceSolver`; the methods below then take over
`picard_solve!`, `solve!`, `adjoint_solve!` and `precondition!` for it, and the Enzyme rules take over their
reverse passes.  Every other solver keeps the reference's generic methods.

This file is the binding as source.  It has not been run: the environment this library is built and tested in has
no Julia, Oceananigans, KernelAbstractions or Enzyme, so its `ccall` signatures are checked only against the header
(the Python ctypes mirror, `nunatak_gb300/abi.py`, is tested against the same layout).

Fields cross the boundary as their Oceananigans parent arrays (`parent(field)`: x fastest, halos included, host
`Array` or a `CuArray` on the problem's device); the library reads and writes the interior points only.
"""
module NunatakGB300

using Nunatak
using Nunatak: VelocityVector, PicardIteration, Convergence, FixedIterations
using Nunatak: GlenFlowLaw, ArrheniusRateFactor, WeertmanFriction, RegularizedCoulombFriction
using Nunatak: FreeSlipWalls, NoSlipWalls, SubgridGroundedFraction, SmoothIceMask, DIVAShear
using Nunatak: StressBalanceMultigridPreconditioner, StressBalanceDiagonalPreconditioner, PointJacobi, LineJacobi
using Nunatak.Oceananigans: Oceananigans, interior, Field
using Nunatak.Oceananigans.Grids: topology, Bounded, Periodic, halo_size, xnodes, ynodes, Face
using Nunatak.Oceananigans.BoundaryConditions: fill_halo_regions!
using Enzyme
using Enzyme.EnzymeRules

import Nunatak: picard_solve!, solve!, adjoint_solve!, precondition!, update_preconditioner!

export GB300StressBalanceSolver, GB300MultigridPreconditioner, checkpointed_gradient!

const libnk = get(ENV, "NUNATAK_GB300_LIB", joinpath(@__DIR__, "..", "_build", "libnunatak_gb300.so"))

#####
##### Mirrors of the C descriptors (field order and types as in include/nunatak_gb300.h)
#####

const NK_OK, NK_NOT_CONVERGED, NK_NONFINITE, NK_BAD_ARGUMENT = Int32(0), Int32(1), Int32(2), Int32(5)
const NK_BOUNDED, NK_PERIODIC = Int32(0), Int32(1)
const NK_SSA, NK_DIVA = Int32(0), Int32(1)
const NK_FRICTION_NONE, NK_WEERTMAN, NK_REGULARIZED_COULOMB = Int32(0), Int32(1), Int32(2)
const NK_RATE_FACTOR_2D, NK_RATE_FACTOR_SIGMA = Int32(0), Int32(1)
const NK_PRECONDITIONER_NONE, NK_PRECONDITIONER_DIAGONAL, NK_PRECONDITIONER_MULTIGRID = Int32(0), Int32(1), Int32(2)
const NK_PRECISION_FP64, NK_PRECISION_MIXED = Int32(0), Int32(1)
const NK_CONVERGENCE, NK_FIXED_ITERATIONS = Int32(0), Int32(1)

const FIELD = (u = 0, v = 1, H = 2, bed = 3, s = 4, ice_mask = 5, φ = 6, φᵘ = 7, φᵛ = 8, N = 9, τᵘ = 10, τᵛ = 11,
               A = 12, C = 13, η̄H = 14, η̄Hᶠᶠ = 15, βᵘ = 16, βᵛ = 17, ησ = 18, F₂ = 19, βᵇᵘ = 20, βᵇᵛ = 21,
               uᵇ = 22, vᵇ = 23, uσ = 24, vσ = 25, T = 26, a = 31, m = 32)

struct IterationControl
    kind::Int32; iterations::Int32; maxiter::Int32; reserved::Int32; reltol::Float64; abstol::Float64
end
IterationControl(c::Convergence) = IterationControl(NK_CONVERGENCE, 0, c.maxiter, 0, c.reltol, c.abstol)
IterationControl(c::FixedIterations) = IterationControl(NK_FIXED_ITERATIONS, c.iterations, c.iterations, 0, 0.0, 0.0)

struct GridDesc
    Nx::Int32; Ny::Int32; topology_x::Int32; topology_y::Int32; halo_x::Int32; halo_y::Int32
    Nsigma::Int32; reserved::Int32; x_faces::Ptr{Float64}; y_faces::Ptr{Float64}
    x0::Float64; Lx::Float64; y0::Float64; Ly::Float64; sigma_faces::Ptr{Float64}; bed_refinement::Float64
end

struct PhysicsDesc
    stress_balance::Int32; side_walls::Int32; rate_factor_layout::Int32; friction::Int32
    glen_exponent::Float64; strain_rate_regularization::Float64; friction_exponent::Float64
    coulomb_coefficient::Float64; velocity_regularization::Float64; ice_density::Float64
    ocean_density::Float64; gravitational_acceleration::Float64
    use_ice_mask::Int32; grounding::Int32; grounding_line_driving_stress::Int32; use_effective_pressure::Int32
    mask_minimum_thickness::Float64; mask_transition_thickness::Float64
end

struct SolverDesc
    precision::Int32; preconditioner::Int32; smoother::Int32; smoothing_sweeps::Int32
    coarsest_sweeps::Int32; minimum_coarse_size::Int32; linear::IterationControl; picard::IterationControl
    flags::Int32; reserved::Int32
end

mutable struct SolveStats
    status::Int32; picard_iterations::Int32; linear_iterations_last::Int32; linear_iterations_total::Int32
    residual_norm::Float64; initial_residual_norm::Float64; picard_change::Float64; picard_norm::Float64
    device_ms::Float64; device_start_ms::Float64; device_end_ms::Float64
    SolveStats() = new(0, 0, 0, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
end

#####
##### Context and errors
#####

mutable struct Context
    ptr::Ptr{Cvoid}
end

function Context(device::Integer = 0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:nk_context_create, libnk), Int32, (Int32, Ref{Ptr{Cvoid}}), device, r)
    st == NK_OK || error("nk_context_create(device = $device) failed with status $st")
    ctx = Context(r[])
    finalizer(c -> ccall((:nk_context_destroy, libnk), Int32, (Ptr{Cvoid},), c.ptr), ctx)
    return ctx
end

last_error(ctx::Context) = unsafe_string(ccall((:nk_last_error, libnk), Cstring, (Ptr{Cvoid},), ctx.ptr))

# The reference's behaviour for each status: a bad argument throws ArgumentError (as ssa_operator! does for
# missing walls), a solve that stops at maxiter returns its count silently (conjugate_gradient!, picard_solve!),
# a non-finite result throws.
function check(st, ctx::Context, what)
    st == NK_OK && return nothing
    st == NK_NOT_CONVERGED && return nothing
    st == NK_BAD_ARGUMENT && throw(ArgumentError("$what: $(last_error(ctx))"))
    st == NK_NONFINITE && throw(DomainError(what, last_error(ctx)))
    error("$what: status $st, $(last_error(ctx))")
end

#####
##### The problem of one grid: descriptors from the reference's configuration objects
#####

topology_code(::Type{Periodic}) = NK_PERIODIC
topology_code(::Type) = NK_BOUNDED

wall_code(::FreeSlipWalls) = Int32(0)
wall_code(::NoSlipWalls) = Int32(1)

friction_code(::Nothing) = NK_FRICTION_NONE
friction_code(::WeertmanFriction) = NK_WEERTMAN
friction_code(::RegularizedCoulombFriction) = NK_REGULARIZED_COULOMB

friction_parameters(::Nothing) = (1 / 3, 0.0, 1e-8)
friction_parameters(f::WeertmanFriction) = (f.exponent, 0.0, f.velocity_regularization)
friction_parameters(f::RegularizedCoulombFriction) = (f.exponent, f.coulomb_coefficient, f.velocity_regularization)

rate_factor_field(r::GlenFlowLaw) = rate_factor_field(r.rate_factor)
rate_factor_field(a::ArrheniusRateFactor) = a.field
rate_factor_field(a::Field) = a
rate_layout(a::Field) = size(a, 3) > 1 ? NK_RATE_FACTOR_SIGMA : NK_RATE_FACTOR_2D

preconditioner_code(::Nothing) = NK_PRECONDITIONER_NONE
preconditioner_code(::StressBalanceDiagonalPreconditioner) = NK_PRECONDITIONER_DIAGONAL
preconditioner_code(::StressBalanceMultigridPreconditioner) = NK_PRECONDITIONER_MULTIGRID

"""
    GB300StressBalanceSolver(model; precision = :mixed, preconditioner = :multigrid, smoothing_sweeps = 2,
                             coarsest_sweeps = 20, minimum_coarse_size = 2,
                             linear_iteration_control = Convergence(reltol = 1e-8, maxiter = 10_000),
                             device = 0)

The linear solver a `StressBalanceSolver` takes in place of `VelocityConjugateGradientSolver` to run the whole
Picard + PCG loop on the GPU.  It creates one `nk_problem` for the model's grid, σ grid, stress balance, rheology,
friction, grounding and masking.  `precision = :mixed` runs the multigrid preconditioner in FP32 under FP64
flexible conjugate gradients; `:fp64` reproduces the reference's arithmetic.
"""
mutable struct GB300StressBalanceSolver{L}
    ctx::Context
    problem::Ptr{Cvoid}
    hx::Int32
    hy::Int32
    Nsigma::Int32
    linear_iteration_control::L
    stats::SolveStats
end

function GB300StressBalanceSolver(model; precision = :mixed, preconditioner = :multigrid, smoothing_sweeps = 2,
                                  coarsest_sweeps = 20, minimum_coarse_size = 2, smoother = PointJacobi(),
                                  linear_iteration_control = Convergence(; reltol = 1e-8, maxiter = 10_000),
                                  picard_iteration_control = Convergence(; reltol = 1e-6, maxiter = 100),
                                  device = 0, context = Context(device))
    grid, σgrid = model.grid, model.σgrid
    TX, TY, _ = topology(grid)
    Hx, Hy, _ = halo_size(grid)
    Nx, Ny, _ = size(grid)
    Nσ = size(σgrid, 3)
    xf = collect(Float64, xnodes(grid, Face()))
    yf = collect(Float64, ynodes(grid, Face()))
    TX === Bounded && length(xf) == Nx && push!(xf, xf[end] + (xf[end] - xf[end-1]))
    TY === Bounded && length(yf) == Ny && push!(yf, yf[end] + (yf[end] - yf[end-1]))
    TX === Periodic && push!(xf, xf[1] + grid.Lx)
    TY === Periodic && push!(yf, yf[1] + grid.Ly)
    ζ = collect(Float64, σgrid.ζᶠ)                       # the σ faces 0 … 1 of SigmaGrid
    A = rate_factor_field(model.rheology)
    fr = model.friction
    m, α², u₀ = friction_parameters(fr)
    c = model.constants
    masked = model.masking isa SmoothIceMask
    GC.@preserve xf yf ζ begin
        g = GridDesc(Nx, Ny, topology_code(TX), topology_code(TY), Hx, Hy, Nσ, 0, pointer(xf), pointer(yf),
                     xf[1], xf[end] - xf[1], yf[1], yf[end] - yf[1], pointer(ζ), 2.0)
        p = PhysicsDesc(model.stress_balance.shear isa DIVAShear ? NK_DIVA : NK_SSA, wall_code(model.stress_balance.side_walls),
                        rate_layout(A), friction_code(fr), model.rheology.exponent, model.rheology.strain_rate_regularization,
                        m, α², u₀, c.ice_density, c.ocean_density, c.gravitational_acceleration,
                        Int32(masked), Int32(model.grounding isa SubgridGroundedFraction),
                        Int32(model.grounding isa SubgridGroundedFraction && model.grounding.driving_stress),
                        Int32(true), masked ? model.masking.minimum_thickness : 1.0,
                        masked ? model.masking.transition_thickness : 1.0)
        code = preconditioner === :multigrid ? NK_PRECONDITIONER_MULTIGRID :
               preconditioner === :diagonal ? NK_PRECONDITIONER_DIAGONAL : NK_PRECONDITIONER_NONE
        s = SolverDesc(precision === :mixed ? NK_PRECISION_MIXED : NK_PRECISION_FP64, code, Int32(smoother isa LineJacobi),
                       smoothing_sweeps, coarsest_sweeps, minimum_coarse_size, IterationControl(linear_iteration_control),
                       IterationControl(picard_iteration_control), 0, 0)
        r = Ref{Ptr{Cvoid}}(C_NULL)
        st = ccall((:nk_problem_create, libnk), Int32, (Ptr{Cvoid}, Ref{GridDesc}, Ref{PhysicsDesc}, Ref{SolverDesc}, Ref{Ptr{Cvoid}}),
                   context.ptr, g, p, s, r)
        check(st, context, "nk_problem_create")
    end
    solver = GB300StressBalanceSolver(context, r[], Int32(Hx), Int32(Hy), Int32(Nσ), linear_iteration_control, SolveStats())
    finalizer(s -> ccall((:nk_problem_destroy, libnk), Int32, (Ptr{Cvoid},), s.problem), solver)
    return solver
end

# σ fields carry the σ grid's one-level z halo (src/Grids/sigma_grid.jl:57); 2-D fields none.
z_halo(f) = size(parent(f), 3) > 1 ? Int32((size(parent(f), 3) - size(f, 3)) ÷ 2) : Int32(0)

function set_field!(s::GB300StressBalanceSolver, id, f)
    a = parent(f)
    st = ccall((:nk_problem_set_field_parent, libnk), Int32, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Int32, Int32, Int64),
               s.problem, id, a, s.hx, s.hy, z_halo(f), length(a))
    return check(st, s.ctx, "set field $id")
end

function get_field!(f, s::GB300StressBalanceSolver, id)
    a = parent(f)
    st = ccall((:nk_problem_get_field_parent, libnk), Int32, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Int32, Int32, Int64),
               s.problem, id, a, s.hx, s.hy, z_halo(f), length(a))
    check(st, s.ctx, "get field $id")
    fill_halo_regions!(f)
    return f
end

set_vector!(s, x::VelocityVector) = (set_field!(s, FIELD.u, x.u); set_field!(s, FIELD.v, x.v))
get_vector!(x::VelocityVector, s) = (get_field!(x.u, s, FIELD.u); get_field!(x.v, s, FIELD.v); x)

# The coefficient tuple of update_velocities! (src/Models/ice_sheet_model_methods.jl:119-147):
#   SSA  (η̄H, η̄Hᶠᶠ, βᵘ, βᵛ, ησ, F₂, H, rheology, friction, φᵘ, φᵛ, N, ice_mask, walls)
#   DIVA (η̄H, η̄Hᶠᶠ, βᵘ, βᵛ, ησ, F₂, H, rheology, friction, φᵘ, φᵛ, N, ice_mask, βᵇᵘ, βᵇᵛ, uᵇ, vᵇ, walls)
coefficients(args) = (η̄H = args[1], η̄Hᶠᶠ = args[2], βᵘ = args[3], βᵛ = args[4], ησ = args[5], F₂ = args[6], H = args[7],
                      rheology = args[8], friction = args[9], φᵘ = args[10], φᵛ = args[11], N = args[12], μ = args[13],
                      diva = length(args) == 18, βᵇᵘ = get(args, 14, nothing), βᵇᵛ = get(args, 15, nothing),
                      uᵇ = get(args, 16, nothing), vᵇ = get(args, 17, nothing))

friction_field(::Nothing) = nothing
friction_field(f) = f.coefficient

# The inputs of the Picard loop: thickness, geometry the host computed, rate factor, friction coefficient and, for
# the DIVA, the lagged coefficients its first update reads (diva.jl:77-80).
function push_inputs!(s, b, args)
    c = coefficients(args)
    set_field!(s, FIELD.H, c.H)
    set_field!(s, FIELD.φᵘ, c.φᵘ); set_field!(s, FIELD.φᵛ, c.φᵛ)
    set_field!(s, FIELD.N, c.N); set_field!(s, FIELD.ice_mask, c.μ)
    set_field!(s, FIELD.A, rate_factor_field(c.rheology))
    C = friction_field(c.friction)
    C === nothing || set_field!(s, FIELD.C, C)
    set_field!(s, FIELD.τᵘ, b.u); set_field!(s, FIELD.τᵛ, b.v)
    if c.diva
        set_field!(s, FIELD.βᵇᵘ, c.βᵇᵘ); set_field!(s, FIELD.βᵇᵛ, c.βᵇᵛ)
        set_field!(s, FIELD.F₂, c.F₂); set_field!(s, FIELD.ησ, c.ησ)
    end
    return nothing
end

# The coefficients the loop leaves, as update_stress_balance_coefficients! / update_diva_coefficients! would.
function pull_coefficients!(args, s)
    c = coefficients(args)
    get_field!(c.η̄H, s, FIELD.η̄H); get_field!(c.η̄Hᶠᶠ, s, FIELD.η̄Hᶠᶠ)
    get_field!(c.βᵘ, s, FIELD.βᵘ); get_field!(c.βᵛ, s, FIELD.βᵛ)
    get_field!(c.ησ, s, FIELD.ησ); get_field!(c.F₂, s, FIELD.F₂)
    if c.diva
        get_field!(c.βᵇᵘ, s, FIELD.βᵇᵘ); get_field!(c.βᵇᵛ, s, FIELD.βᵇᵛ)
        get_field!(c.uᵇ, s, FIELD.uᵇ); get_field!(c.vᵇ, s, FIELD.vᵇ)
    end
    return nothing
end

function push_coefficients!(s, args)
    c = coefficients(args)
    set_field!(s, FIELD.η̄H, c.η̄H); set_field!(s, FIELD.η̄Hᶠᶠ, c.η̄Hᶠᶠ)
    set_field!(s, FIELD.βᵘ, c.βᵘ); set_field!(s, FIELD.βᵛ, c.βᵛ)
    return nothing
end

#####
##### The drop-in methods
#####

"""
    picard_solve!(x, picard, s::GB300StressBalanceSolver, update_coefficients!, b, args...)

The whole loop of `picard_solve!` (src/Solvers/picard.jl:63-90) as one library call: `x` is the warm start and the
result, `b` the driving stress, `args` the coefficient tuple of `update_velocities!`.  The library runs
`update_coefficients!`'s equivalent (SSA or DIVA, chosen when the solver was built) on the device.  Returns the
Picard iteration count.  The Picard control is `picard.iteration_control`.
"""
function picard_solve!(x, picard::PicardIteration, s::GB300StressBalanceSolver, update_coefficients!, b, args...)
    push_inputs!(s, b, args)
    set_vector!(s, x)
    stats = s.stats
    st = ccall((:nk_picard_solve, libnk), Int32, (Ptr{Cvoid}, Ref{SolveStats}), s.problem, stats)
    check(st, s.ctx, "nk_picard_solve")
    get_vector!(x, s)
    pull_coefficients!(args, s)
    return Int(stats.picard_iterations)
end

# b crosses as the dense interior of each component (interior layout).
interior_copy(f) = Array{Float64}(collect(interior(f)))

"""
    solve!(x, s::GB300StressBalanceSolver, b, args...)

`solve!` of `VelocityConjugateGradientSolver` (src/Solvers/conjugate_gradient.jl:128-129) with the coefficients of
`args` (η̄H, η̄Hᶠᶠ, βᵘ, βᵛ, …) and the warm start in `x`.
"""
function solve!(x, s::GB300StressBalanceSolver, b, args...)
    push_coefficients!(s, args)
    set_vector!(s, x)
    st = ccall((:nk_linear_solve, libnk), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{SolveStats}),
               s.problem, interior_copy(b.u), interior_copy(b.v), s.stats)
    check(st, s.ctx, "nk_linear_solve")
    return get_vector!(x, s)
end

"""
    adjoint_solve!(λ, s::GB300StressBalanceSolver, b, args...)

`adjoint_solve!` (src/Solvers/conjugate_gradient.jl:155-156): the SSA operator is self-adjoint, so the same solve.
"""
function adjoint_solve!(λ, s::GB300StressBalanceSolver, b, args...)
    push_coefficients!(s, args)
    set_vector!(s, λ)
    st = ccall((:nk_adjoint_solve, libnk), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{SolveStats}),
               s.problem, interior_copy(b.u), interior_copy(b.v), s.stats)
    check(st, s.ctx, "nk_adjoint_solve")
    return get_vector!(λ, s)
end

"""
    GB300MultigridPreconditioner(solver::GB300StressBalanceSolver)

The library's configured preconditioner (multigrid, in FP32 for a mixed-precision solver) for a reference
`VelocityConjugateGradientSolver` that keeps its own loop: `precondition!(z, P, r, args...)` is one application.
"""
struct GB300MultigridPreconditioner{S}
    solver::S
end

update_preconditioner!(P::GB300MultigridPreconditioner, args...) = push_coefficients!(P.solver, args)

function precondition!(z, P::GB300MultigridPreconditioner, r, args...)
    s = P.solver
    zu, zv = interior_copy(z.u), interior_copy(z.v)
    st = ccall((:nk_precondition, libnk), Int32, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
               s.problem, interior_copy(r.u), interior_copy(r.v), zu, zv)
    check(st, s.ctx, "nk_precondition")
    interior(z.u) .= zu
    interior(z.v) .= zv
    fill_halo_regions!(z.u); fill_halo_regions!(z.v)
    return z
end

#####
##### Enzyme: the fixed-point adjoint of a converged picard_solve! (ext/NunatakEnzymeExt.jl:159-240) and the implicit
##### adjoint of solve! (:66-111), each one library call in `reverse`
#####

const Shadowed = Union{Duplicated, MixedDuplicated}
shadow(a::Duplicated) = a.dval
shadow(a::MixedDuplicated) = a.dval[]
const GB300Solver = Union{Const{<:GB300StressBalanceSolver}, Duplicated{<:GB300StressBalanceSolver}}
const ConvergedPicard = Enzyme.EnzymeCore.Annotation{<:PicardIteration{<:Convergence}}

function EnzymeRules.augmented_primal(config, func::Const{typeof(picard_solve!)}, ::Type{RT}, x::Shadowed,
                                      picard::ConvergedPicard, linear_solver::GB300Solver, update!::Const,
                                      b, args...) where RT
    iterations = picard_solve!(x.val, picard.val, linear_solver.val, update!.val, b.val, map(a -> a.val, args)...)
    # The library keeps x* and its coefficients resident: the reverse pass reads them there, so the tape is empty.
    primal = EnzymeRules.needs_primal(config) ? iterations : nothing
    return EnzymeRules.AugmentedReturn(primal, nothing, nothing)
end

accumulate!(::Const, g) = nothing
accumulate!(a::Shadowed, g) = (interior(shadow(a)) .+= g; nothing)

function EnzymeRules.reverse(config, func::Const{typeof(picard_solve!)}, ::Type{RT}, tape, x::Shadowed,
                             picard::ConvergedPicard, linear_solver::GB300Solver, update!::Const,
                             b, args...) where RT
    s = linear_solver.val
    c = coefficients(args)
    x̄ = shadow(x)
    λu, λv = zeros(size(interior(x̄.u))), zeros(size(interior(x̄.v)))
    C = friction_field(c.friction)
    A = rate_factor_field(c.rheology)
    glogC = zeros(size(interior(c.H)))
    glogA = zeros(size(interior(A)))
    ctl = Ref(IterationControl(picard.val.adjoint_iteration_control))
    st = ccall((:nk_picard_adjoint, libnk), Int32,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{IterationControl}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                Ptr{Float64}, Ref{SolveStats}),
               s.problem, interior_copy(x̄.u), interior_copy(x̄.v), ctl, λu, λv, glogC, glogA, s.stats)
    check(st, s.ctx, "nk_picard_adjoint")
    st == NK_NOT_CONVERGED && @warn "Picard adjoint did not converge: ‖Δλ‖ = $(s.stats.picard_change), ‖λ‖ = $(s.stats.picard_norm)"
    # b̄ += λ on the solved cells (accumulate_right_hand_side_adjoint!)
    if b isa Shadowed
        view(interior(shadow(b).u), axes(λu)...) .+= λu
        view(interior(shadow(b).v), axes(λv)...) .+= λv
    end
    # C̄ and Ā from the log-space gradients: ∂J/∂p = (∂J/∂log p) / p
    C === nothing || !(args[9] isa Shadowed) || (interior(shadow(args[9]).coefficient) .+= glogC ./ interior(C))
    args[8] isa Shadowed && (interior(rate_factor_field(shadow(args[8]))) .+= glogA ./ interior(A))
    # The thickness enters the viscosity, the driving stress and the geometry; the library returns no ∂J/∂H.
    args[7] isa Shadowed && @warn "NunatakGB300: the Picard adjoint returns no thickness gradient; H's shadow is left as it was"
    # A converged fixed point depends on neither the initial guess nor the lagged DIVA coefficients.
    c.diva && foreach(i -> args[i] isa Shadowed && (parent(shadow(args[i])) .= 0), (5, 6, 14, 15))
    parent(x̄.u) .= 0
    parent(x̄.v) .= 0
    return (nothing, nothing, nothing, nothing, nothing, map(a -> nothing, args)...)
end

function EnzymeRules.augmented_primal(config, func::Const{typeof(solve!)}, ::Type{RT}, x::Shadowed,
                                      solver::GB300Solver, b, args...) where RT
    solve!(x.val, solver.val, b.val, map(a -> a.val, args)...)
    primal = EnzymeRules.needs_primal(config) ? x.val : nothing
    x̄ = EnzymeRules.needs_shadow(config) ? shadow(x) : nothing
    return EnzymeRules.AugmentedReturn(primal, x̄, nothing)
end

# λ = A⁻ᵀ x̄ by nk_adjoint_solve, accumulated into b̄.  The coefficient shadows (η̄H, η̄Hᶠᶠ, β) would take
# -(∂(A x)/∂c)ᵀ λ, which the library computes inside nk_picard_adjoint but does not export alone: differentiate the
# Picard loop instead, or keep the coefficients Const here.
function EnzymeRules.reverse(config, func::Const{typeof(solve!)}, ::Type{RT}, tape, x::Shadowed,
                             solver::GB300Solver, b, args...) where RT
    any(a -> a isa Shadowed, args[1:4]) &&
        throw(ArgumentError("NunatakGB300: differentiate picard_solve! for coefficient gradients; solve! returns b̄ only"))
    s = solver.val
    x̄ = shadow(x)
    λ = similar(x̄)
    fill!(parent(λ.u), 0); fill!(parent(λ.v), 0)
    adjoint_solve!(λ, s, x̄, map(a -> a.val, args)...)
    if b isa Shadowed
        interior(shadow(b).u) .+= interior(λ.u)
        interior(shadow(b).v) .+= interior(λ.v)
    end
    parent(x̄.u) .= 0
    parent(x̄.v) .= 0
    return (nothing, nothing, nothing, map(a -> nothing, args)...)
end

#####
##### The gradient through time steps (checkpointed_gradient!, ext/NunatakEnzymeExt.jl:245-263)
#####

struct AdvectionDesc
    scheme::Int32; order::Int32; bounded::Int32; reserved::Int32; lower::Float64; upper::Float64
end

struct CostState
    step::Int32; steps::Int32; H::Ptr{Float64}; u::Ptr{Float64}; v::Ptr{Float64}; ice_mask::Ptr{Float64}
end

struct TimeGradientDesc
    dt::Float64; steps::Int32; checkpoint_interval::Int32; velocity_solves::Int32; reserved::Int32
    melt_weights::Ptr{Float64}; adjoint_control::Ptr{IterationControl}
end

struct TimeGradient
    grad_H::Ptr{Float64}; grad_u::Ptr{Float64}; grad_v::Ptr{Float64}; grad_smb::Ptr{Float64}; grad_melt::Ptr{Float64}
    grad_log_C::Ptr{Float64}; grad_log_A::Ptr{Float64}
end

mutable struct TimeGradientStats
    J::Float64; segments::Int32; picard_solves::Int32; picard_adjoints::Int32; adjoint_iterations::Int32
    worst_solve_status::Int32; reserved::Int32; elapsed_ms::Float64
    TimeGradientStats() = new(0.0, 0, 0, 0, 0, 0, 0, 0.0)
end

# The model's thickness advection (IceSheetModel's `advection`) as the library's descriptor: UpwindBiased{N} and
# WENO{N} carry their order as 2N - 1; a bounds-preserving WENO its bounds.
scheme_order(::Oceananigans.Advection.UpwindBiased{N}) where N = Int32(2N - 1)
scheme_order(::Oceananigans.Advection.WENO{N}) where N = Int32(2N - 1)
advection_desc(a::Oceananigans.Advection.UpwindBiased) = AdvectionDesc(0, scheme_order(a), 0, 0, 0.0, 0.0)
function advection_desc(a::Oceananigans.Advection.WENO)
    b = a.bounds
    return b === nothing ? AdvectionDesc(1, scheme_order(a), 0, 0, 0.0, 0.0) : AdvectionDesc(1, scheme_order(a), 1, 0, b[1], b[2])
end

# The host's cost of the final model, differentiated by Enzyme on the host: the model's H, u, v and ice mask are set
# to the state the library hands over, and ∂J/∂(H, u, v) are the shadows of a zeroed model.  The library calls this
# after every step; the reference's cost is a function of the final model only.
mutable struct CostCallback{F, M}
    cost::F
    model::M
    err::Any
end

function set_interior!(f, p::Ptr{Float64})
    a = interior(f, :, :, 1)
    a .= unsafe_wrap(Array, p, size(a))
    fill_halo_regions!(f)
    return f
end
get_interior!(p::Ptr{Float64}, f) = (unsafe_wrap(Array, p, size(interior(f, :, :, 1))) .= interior(f, :, :, 1); nothing)

function cost_callback(user::Ptr{Cvoid}, state::Ptr{CostState}, J::Ptr{Float64}, dH::Ptr{Float64}, du::Ptr{Float64},
                       dv::Ptr{Float64})::Int32
    cb = unsafe_pointer_to_objref(user)::CostCallback
    s = unsafe_load(state)
    unsafe_store!(J, 0.0)
    s.step == s.steps || return Int32(0)
    try
        model = cb.model
        set_interior!(model.geometry.H, s.H)
        set_interior!(model.velocities.u, s.u)
        set_interior!(model.velocities.v, s.v)
        set_interior!(model.geometry.ice_mask, s.ice_mask)
        dmodel = Enzyme.make_zero(model)
        _, Jv = autodiff(set_runtime_activity(ReverseWithPrimal), cb.cost, Active, Duplicated(model, dmodel))
        unsafe_store!(J, Jv)
        get_interior!(dH, dmodel.geometry.H)
        get_interior!(du, dmodel.velocities.u)
        get_interior!(dv, dmodel.velocities.v)
        return Int32(0)
    catch e
        cb.err = e
        return Int32(1)
    end
end

"""
    checkpointed_gradient!(dmodel, cost, model, Δt, Nt; checkpoint_interval = ceil(Int, sqrt(Nt)),
                           solver = model.velocity_solver.linear_solver, melt_weights = nothing)

`checkpointed_gradient!` for a model whose stress-balance solver is a `GB300StressBalanceSolver`: `Nt` time steps of
`Δt` (three split Runge-Kutta thickness stages with the model's advection, a Picard solve after each) and the
gradient of `cost(model)` after them, on the GPU, by nk_checkpointed_gradient.  The gradient with respect to the
initial thickness and velocities, the surface mass balance, the basal melt rate, the friction coefficient and the
rate factor accumulates into `dmodel`; `model` is left at the final state; returns the cost.  The cost itself is
differentiated by Enzyme on the host.  Not covered by the library: the energy step.
"""
function checkpointed_gradient!(dmodel, cost, model, Δt, Nt; checkpoint_interval = ceil(Int, sqrt(Nt)),
                                solver::GB300StressBalanceSolver = model.velocity_solver.linear_solver, melt_weights = nothing)
    s = solver
    set_field!(s, FIELD.H, model.geometry.H)
    set_field!(s, FIELD.bed, model.bed)
    set_field!(s, FIELD.u, model.velocities.u); set_field!(s, FIELD.v, model.velocities.v)
    A = rate_factor_field(model.rheology)
    set_field!(s, FIELD.A, A)
    C = friction_field(model.friction)
    C === nothing || set_field!(s, FIELD.C, C)
    set_field!(s, FIELD.a, model.surface_mass_balance)
    set_field!(s, FIELD.m, model.basal_melt_rate)
    adv = Ref(advection_desc(model.advection))
    check(ccall((:nk_set_thickness_advection, libnk), Int32, (Ptr{Cvoid}, Ref{AdvectionDesc}), s.problem, adv), s.ctx,
          "nk_set_thickness_advection")
    check(ccall((:nk_compute_geometry, libnk), Int32, (Ptr{Cvoid},), s.problem), s.ctx, "nk_compute_geometry")

    Nx, Ny = size(model.grid)[1:2]
    gH, gsmb, gmelt, glogC = (zeros(Nx, Ny) for _ in 1:4)
    gu, gv = zeros(size(interior(model.velocities.u, :, :, 1))), zeros(size(interior(model.velocities.v, :, :, 1)))
    glogA = zeros(size(interior(A)))
    w = melt_weights === nothing ? nothing : collect(Float64, melt_weights)
    ctl = Ref(IterationControl(model.velocity_solver.picard.adjoint_iteration_control))
    cb = CostCallback(cost, model, nothing)
    fn = @cfunction(cost_callback, Int32, (Ptr{Cvoid}, Ptr{CostState}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}))
    stats = TimeGradientStats()
    st = GC.@preserve cb gH gu gv gsmb gmelt glogC glogA w ctl begin
        d = Ref(TimeGradientDesc(Δt, Nt, checkpoint_interval, 1, 0, w === nothing ? C_NULL : pointer(w),
                                 Base.unsafe_convert(Ptr{IterationControl}, ctl)))
        out = Ref(TimeGradient(pointer(gH), pointer(gu), pointer(gv), pointer(gsmb), pointer(gmelt), pointer(glogC),
                               pointer(glogA)))
        ccall((:nk_checkpointed_gradient, libnk), Int32,
              (Ptr{Cvoid}, Ref{TimeGradientDesc}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{TimeGradient}, Ref{TimeGradientStats}),
              s.problem, d, fn, pointer_from_objref(cb), out, stats)
    end
    cb.err === nothing || throw(cb.err)
    check(st, s.ctx, "nk_checkpointed_gradient")

    interior(dmodel.geometry.H, :, :, 1) .+= gH
    interior(dmodel.velocities.u, :, :, 1) .+= gu
    interior(dmodel.velocities.v, :, :, 1) .+= gv
    interior(dmodel.surface_mass_balance, :, :, 1) .+= gsmb
    interior(dmodel.basal_melt_rate, :, :, 1) .+= gmelt
    C === nothing || (interior(friction_field(dmodel.friction)) .+= glogC ./ interior(C))
    interior(rate_factor_field(dmodel.rheology)) .+= glogA ./ interior(A)

    # the final state, as checkpointed_gradient! leaves the model
    get_field!(model.geometry.H, s, FIELD.H)
    get_field!(model.velocities.u, s, FIELD.u); get_field!(model.velocities.v, s, FIELD.v)
    Nunatak.update_geometry_state!(model)
    return stats.J
end

end # module
