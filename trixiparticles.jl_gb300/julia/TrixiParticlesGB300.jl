# TrixiParticlesGB300.jl — `ccall` shim that routes the WCSPH right-hand side of
# TrixiParticles.jl to libtp_wcsph.so (sm_103a).  Load after TrixiParticles and CUDA:
#
#     using TrixiParticles, CUDA
#     include("TrixiParticlesGB300.jl"); using .TrixiParticlesGB300
#     semi = Semidiscretization(fluid_system, boundary_system;
#                               neighborhood_search=GridNeighborhoodSearch{3}(; cell_list),
#                               parallelization_backend=GB300Backend())
#     ode = semidiscretize(semi, tspan)      # allocates CuArrays (GB300Backend <: GPU)
#     sol = solve(ode, CarpenterKennedy2N54(williamson_condition=false), dt=5e-5, ...)
#
# How it plugs in (paths relative to the TrixiParticles.jl source tree):
#   * `Semidiscretization{BACKEND, S, RU, RV, NSH, IM, UCU, IT}` carries the backend in its
#     FIRST type parameter (src/general/semidiscretization.jl:78-86), so
#     `Semidiscretization{<:GB300Backend}` selects the simulations that run on this library.
#   * `semidiscretize` stores `p = (; semi, split_integration_data)` in the ODE problem
#     (semidiscretization.jl:386-395); kick!/drift! are specialised on that NamedTuple type.
#   * The fluid's grid search is `get_neighborhood_search(fluid, fluid, semi)`, which reads it
#     from `semi.neighborhood_search_handler` (src/general/neighborhood_search.jl:397-416); its
#     `cell_list` is the FullGridCellList whose corners define the library's grid.
#   * Everything `semidiscretize` and `initialize!` do on a GPU backend outside kick!/drift!
#     (allocation, `Adapt.adapt(backend, systems)`, `@threaded semi` loops) is forwarded to
#     CUDA.jl's CUDABackend (src/general/gpu.jl:41-43, semidiscretization.jl:354-379).
#
# kick!/drift! of such a Semidiscretization call tp_kick/tp_drift with the raw device pointers
# of v_ode/u_ode/dv_ode/du_ode at the fluid system's ranges.  Supported system pair:
# WeaklyCompressibleSPHSystem(ContinuityDensity, WendlandC2Kernel, StateEquationCole,
# ArtificialViscosityMonaghan|nothing, DensityDiffusionMolteniColagrossi|nothing) with a
# WallBoundarySystem(BoundaryModelDummyParticles(AdamiPressureExtrapolation)), Float64 arrays.
# Anything else throws ArgumentError (docs/src/development.md:96).  This file is written
# against the reference sources; Julia is not installed where it was written, so it has not
# been executed (tests/test_julia_shim.py checks its C declarations against the header).
module TrixiParticlesGB300

using Adapt: Adapt
using CUDA: CUDA, CuArray, CuMatrix, CuPtr
using KernelAbstractions: KernelAbstractions
using ChainRulesCore: ChainRulesCore
using TrixiParticles: TrixiParticles, Semidiscretization, WeaklyCompressibleSPHSystem,
                      WallBoundarySystem, BoundaryModelDummyParticles,
                      AdamiPressureExtrapolation, ContinuityDensity, WendlandC2Kernel,
                      StateEquationCole, ArtificialViscosityMonaghan,
                      DensityDiffusionMolteniColagrossi, FullGridCellList
using TrixiParticles.PointNeighbors: PointNeighbors

export GB300Backend

const libtp = get(ENV, "TP_WCSPH_LIB", joinpath(@__DIR__, "..", "libtp_wcsph.so"))

# A KernelAbstractions GPU backend, so that `semidiscretize` takes its GPU branch.
struct GB300Backend <: KernelAbstractions.GPU
    precision::Int32   # 0 = Float64 drop-in, 1 = FP32 precision form
end
GB300Backend() = GB300Backend(Int32(0))

# Generic GPU work outside the right-hand side runs on CUDA.jl's own backend.
const CUDA_BACKEND = CUDA.CUDABackend()
KernelAbstractions.allocate(::GB300Backend, ::Type{T}, dims::Tuple) where {T} =
    CuArray{T}(undef, dims)
KernelAbstractions.synchronize(::GB300Backend) = KernelAbstractions.synchronize(CUDA_BACKEND)
Adapt.adapt_storage(::GB300Backend, x::AbstractArray) = Adapt.adapt(CuArray, x)
PointNeighbors.parallel_foreach(f, iterator, ::GB300Backend) =
    PointNeighbors.parallel_foreach(f, iterator, CUDA_BACKEND)

# tp_config of include/tp_wcsph.h: same field order and C types.
struct TpConfig
    ndims::Int32
    precision::Int32
    n_fluid::Int64
    n_wall::Int64
    smoothing_length::Float64
    reference_density::Float64
    sound_speed::Float64
    exponent::Float64
    background_pressure::Float64
    fluid_clip_negative_pressure::Int32
    wall_clip_negative_pressure::Int32
    viscosity_model::Int32
    density_diffusion_model::Int32
    viscosity_alpha::Float64
    viscosity_beta::Float64
    viscosity_epsilon::Float64
    density_diffusion_delta::Float64
    acceleration::NTuple{3, Float64}
    pressure_offset::Float64
    min_corner::NTuple{3, Float64}
    max_corner::NTuple{3, Float64}
end

pad3(x) = ntuple(i -> i <= length(x) ? Float64(x[i]) : 0.0, 3)

function check(h, status)
    status == 0 && return nothing
    msg = unsafe_string(ccall((:tp_last_error, libtp), Cstring, (Ptr{Cvoid},), h))
    status in (1, 5) && throw(ArgumentError(msg))
    throw(ErrorException("libtp_wcsph status $status: $msg"))
end

const GB300Semi = Semidiscretization{<:GB300Backend}
const GB300Params = NamedTuple{(:semi, :split_integration_data), <:Tuple{GB300Semi, Any}}

# The fluid and the wall system of the semidiscretization, with their positions in `systems`.
function system_pair(semi)
    fi = findall(s -> s isa WeaklyCompressibleSPHSystem, semi.systems)
    wi = findall(s -> s isa WallBoundarySystem, semi.systems)
    (length(fi) == 1 && length(wi) == 1 && length(semi.systems) == 2) ||
        throw(ArgumentError("GB300Backend supports one WeaklyCompressibleSPHSystem and one " *
                            "WallBoundarySystem"))
    return semi.systems[fi[1]], fi[1], semi.systems[wi[1]]
end

function tp_config(fluid, wall, nhs, backend)
    fluid.density_calculator isa ContinuityDensity ||
        throw(ArgumentError("GB300Backend supports ContinuityDensity only"))
    fluid.smoothing_kernel isa WendlandC2Kernel ||
        throw(ArgumentError("GB300Backend supports WendlandC2Kernel only"))
    (isnothing(fluid.correction) && isnothing(fluid.surface_tension) &&
     isnothing(fluid.shifting_technique)) ||
        throw(ArgumentError("corrections, surface tension and shifting are not supported"))
    eltype(fluid.mass) == Float64 || throw(ArgumentError("GB300Backend needs Float64 arrays"))
    bm = wall.boundary_model
    (bm isa BoundaryModelDummyParticles &&
     bm.density_calculator isa AdamiPressureExtrapolation &&
     isnothing(bm.viscosity) && isnothing(bm.correction)) ||
        throw(ArgumentError("wall must be BoundaryModelDummyParticles(AdamiPressureExtrapolation)"))
    nhs isa PointNeighbors.GridNeighborhoodSearch ||
        throw(ArgumentError("GPU execution needs a GridNeighborhoodSearch"))
    cl = nhs.cell_list
    cl isa FullGridCellList || throw(ArgumentError("GPU execution needs a FullGridCellList"))
    se = fluid.state_equation
    se isa StateEquationCole || throw(ArgumentError("StateEquationCole is required"))
    visc = fluid.viscosity
    dd = fluid.density_diffusion
    (isnothing(visc) || visc isa ArtificialViscosityMonaghan) ||
        throw(ArgumentError("only ArtificialViscosityMonaghan is supported"))
    (isnothing(dd) || dd isa DensityDiffusionMolteniColagrossi) ||
        throw(ArgumentError("only DensityDiffusionMolteniColagrossi is supported"))
    monaghan = visc isa ArtificialViscosityMonaghan
    mc = dd isa DensityDiffusionMolteniColagrossi
    return TpConfig(ndims(fluid), backend.precision, TrixiParticles.nparticles(fluid),
                    TrixiParticles.nparticles(wall),
                    TrixiParticles.initial_smoothing_length(fluid),
                    se.reference_density, se.sound_speed, se.exponent,
                    se.background_pressure, TrixiParticles.clip_negative_pressure(se),
                    bm.clip_negative_pressure,
                    monaghan ? 1 : 0, mc ? 1 : 0,
                    monaghan ? visc.alpha : 0.0, monaghan ? visc.beta : 0.0,
                    monaghan ? visc.epsilon : 0.01, mc ? dd.delta : 0.0,
                    pad3(fluid.acceleration),
                    bm.density_calculator.pressure_offset,
                    pad3(cl.min_corner), pad3(cl.max_corner))
end

# One library handle per simulation.  `Semidiscretization` is immutable (no finalizer), so the
# handle is keyed on the fluid's device mass array, which `semidiscretize` creates once per
# simulation; the handle is destroyed when that array is collected.
mutable struct Handle
    ptr::Ptr{Cvoid}
    fluid_index::Int
end
const HANDLES = WeakKeyDict{Any, Handle}()

function handle(semi)
    fluid, fi, wall = system_pair(semi)
    return get!(HANDLES, fluid.mass) do
        nhs = TrixiParticles.get_neighborhood_search(fluid, fluid, semi)
        cfg = tp_config(fluid, wall, nhs, semi.parallelization_backend)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(C_NULL, ccall((:tp_create, libtp), Cint, (Ref{TpConfig}, Ref{Ptr{Cvoid}}), cfg, h))
        hd = Handle(h[], fi)
        finalizer(x -> ccall((:tp_destroy, libtp), Cint, (Ptr{Cvoid},), x.ptr), hd)
        check(h[], ccall((:tp_set_stream, libtp), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h[],
                         CUDA.stream().handle))
        check(h[], ccall((:tp_set_wall, libtp), Cint, (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}),
                         h[], wall.coordinates, wall.boundary_model.hydrodynamic_mass))
        check(h[], ccall((:tp_set_fluid_mass, libtp), Cint, (Ptr{Cvoid}, CuPtr{Float64}),
                         h[], fluid.mass))
        hd
    end
end

# Device pointers of the fluid's block of an ODE vector (its `ranges_u` / `ranges_v` entry).
u_ptr(a, semi, hd) = pointer(a, first(semi.ranges_u[hd.fluid_index]))
v_ptr(a, semi, hd) = pointer(a, first(semi.ranges_v[hd.fluid_index]))

function no_split(p)
    isnothing(p.split_integration_data) ||
        throw(ArgumentError("GB300Backend does not support split integration"))
end

# kick! (src/general/semidiscretization.jl:589-612)
function TrixiParticles.kick!(dv_ode, v_ode, u_ode, p::GB300Params, t)
    no_split(p)
    semi = p.semi
    hd = handle(semi)
    check(hd.ptr, ccall((:tp_kick, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Float64),
                        hd.ptr, v_ptr(dv_ode, semi, hd), v_ptr(v_ode, semi, hd),
                        u_ptr(u_ode, semi, hd), t))
    return dv_ode
end

# drift! (src/general/semidiscretization.jl:522-536)
function TrixiParticles.drift!(du_ode, v_ode, u_ode, p::GB300Params, t)
    semi = p.semi
    hd = handle(semi)
    check(hd.ptr, ccall((:tp_drift, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Float64),
                        hd.ptr, u_ptr(du_ode, semi, hd), v_ptr(v_ode, semi, hd),
                        u_ptr(u_ode, semi, hd), t))
    return du_ode
end

# Host reads of results (callbacks) must wait for the handle's stream; also reports particles
# that left the FullGridCellList box.
sync!(semi) = (hd = handle(semi); check(hd.ptr, ccall((:tp_sync, libtp), Cint,
                                                      (Ptr{Cvoid},), hd.ptr)))

# Whole CarpenterKennedy2N54 steps in one call (device arrays are advanced in place).
function integrate_ck2n54!(semi, v_ode, u_ode, t0, dt, nsteps)
    hd = handle(semi)
    check(hd.ptr, ccall((:tp_integrate_ck2n54, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Float64, Int64),
                        hd.ptr, v_ptr(v_ode, semi, hd), u_ptr(u_ode, semi, hd), t0, dt, nsteps))
    sync!(semi)
    return v_ode, u_ode
end

# ---- SymplecticPositionVerlet, SortingCallback's sort, interpolation ----------------------
function integrate_spv!(semi, v_ode, u_ode, t0, dt, nsteps)
    hd = handle(semi)
    check(hd.ptr, ccall((:tp_integrate_spv, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Float64, Int64),
                        hd.ptr, v_ptr(v_ode, semi, hd), u_ptr(u_ode, semi, hd), t0, dt, nsteps))
    return v_ode, u_ode
end

# sort_particles! of SortingCallback (the reference leaves masses in place: sort_masses=false)
function sort_particles!(semi, v_ode, u_ode; sort_masses=false)
    hd = handle(semi)
    fluid, _, _ = system_pair(semi)
    perm = CUDA.zeros(Int32, TrixiParticles.nparticles(fluid))
    check(hd.ptr, ccall((:tp_sort_particles, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Int32, CuPtr{Int32}),
                        hd.ptr, v_ptr(v_ode, semi, hd), u_ptr(u_ode, semi, hd),
                        Int32(sort_masses), perm))
    return perm .+ Int32(1)
end

function interpolate_points(points::CuMatrix{Float64}, semi, v_ode, u_ode; smoothing_length,
                            cut_off_bnd=true, clip_negative_pressure=false,
                            include_wall_velocity=false)
    hd = handle(semi)
    n = size(points, 2)
    cd, p, rho = CUDA.zeros(n), CUDA.zeros(n), CUDA.zeros(n)
    vel = CUDA.zeros(size(points, 1), n)
    count = CUDA.zeros(Int32, n)
    check(hd.ptr, ccall((:tp_interpolate_points, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Int64,
                         Float64, Int32, Int32, Int32, CuPtr{Float64}, CuPtr{Float64},
                         CuPtr{Float64}, CuPtr{Float64}, CuPtr{Int32}),
                        hd.ptr, v_ptr(v_ode, semi, hd), u_ptr(u_ode, semi, hd), points, n,
                        smoothing_length, Int32(cut_off_bnd), Int32(clip_negative_pressure),
                        Int32(include_wall_velocity), cd, vel, p, rho, count))
    return (; computed_density=cd, point_coords=points, neighbor_count=count, velocity=vel,
            pressure=p, density=rho)
end

# ---- Differentiation form: rrule of a fixed-step CarpenterKennedy2N54 solve -------------
# `params = (alpha, delta, gravity magnitude)` must be the values the semidiscretization was
# built with: they are differentiated, not changed.  Forward: tp_adjoint_forward advances
# (v, u) in place and checkpoints every `every` steps.  Pullback: tp_adjoint_backward maps the
# cotangents of the final (v, u) to those of (v0, u0) and returns the parameter gradient.
function model_params(semi)
    fluid, _, _ = system_pair(semi)
    visc, dd = fluid.viscosity, fluid.density_diffusion
    return (visc isa ArtificialViscosityMonaghan ? Float64(visc.alpha) : 0.0,
            dd isa DensityDiffusionMolteniColagrossi ? Float64(dd.delta) : 0.0,
            sqrt(sum(abs2, fluid.acceleration)))
end

function solve_ck2n54(params::NTuple{3, Float64}, semi, v0::CuArray{Float64},
                      u0::CuArray{Float64}, dt, nsteps; every=25)
    params == model_params(semi) ||
        throw(ArgumentError("params must equal (alpha, delta, |g|) of the semidiscretization"))
    hd = handle(semi)
    v, u = copy(v0), copy(u0)
    check(hd.ptr, ccall((:tp_adjoint_forward, libtp), Cint,
                        (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Int64, Int64),
                        hd.ptr, v_ptr(v, semi, hd), u_ptr(u, semi, hd), dt, nsteps, every))
    return v, u
end

function ChainRulesCore.rrule(::typeof(solve_ck2n54), params::NTuple{3, Float64}, semi, v0,
                              u0, dt, nsteps; every=25)
    v, u = solve_ck2n54(params, semi, v0, u0, dt, nsteps; every)
    function solve_ck2n54_pullback(ȳ)
        v̄, ū = ChainRulesCore.unthunk.(ChainRulesCore.unthunk(ȳ))
        vb = v̄ isa ChainRulesCore.AbstractZero ? CUDA.zeros(Float64, size(v)) : copy(v̄)
        ub = ū isa ChainRulesCore.AbstractZero ? CUDA.zeros(Float64, size(u)) : copy(ū)
        pbar = zeros(Float64, 3)
        hd = handle(semi)
        check(hd.ptr, ccall((:tp_adjoint_backward, libtp), Cint,
                            (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Ptr{Float64}),
                            hd.ptr, v_ptr(vb, semi, hd), u_ptr(ub, semi, hd), pbar))
        p̄ = ChainRulesCore.Tangent{NTuple{3, Float64}}(pbar[1], pbar[2], pbar[3])
        return (ChainRulesCore.NoTangent(), p̄, ChainRulesCore.NoTangent(), vb, ub,
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return (v, u), solve_ck2n54_pullback
end

# ---- Batching form: several Semidiscretizations per CUDA-graph launch ----------------------
# members: Vector of (semi, v::CuArray, u::CuArray, dt).  Returns the batch pointer.
# persistent=true: one work-queue pair launch per stage for all members (FP32 members on
# neighbour lists); the default records the members as parallel graph branches.
function batch_create(members; steps=5, autotune=true, growth=1.5, persistent=false)
    hds = [handle(m[1]) for m in members]
    hs = [hd.ptr for hd in hds]
    b = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:tp_batch_create, libtp), Cint, (Ptr{Ptr{Cvoid}}, Int32, Ref{Ptr{Cvoid}}),
               hs, Int32(length(hs)), b)
    st == 0 || error("tp_batch_create failed ($st)")
    bcheck(st) = st == 0 || error(unsafe_string(ccall((:tp_batch_last_error, libtp), Cstring,
                                                      (Ptr{Cvoid},), b[])))
    for (k, (semi, v, u, dt)) in enumerate(members)
        bcheck(ccall((:tp_batch_set_state, libtp), Cint,
                     (Ptr{Cvoid}, Int32, CuPtr{Float64}, CuPtr{Float64}, Float64),
                     b[], Int32(k - 1), v_ptr(v, semi, hds[k]), u_ptr(u, semi, hds[k]), dt))
    end
    autotune && bcheck(ccall((:tp_batch_autotune, libtp), Cint,
                             (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}, Ptr{Int32},
                              Ptr{Float64}),
                             b[], Int32(6), C_NULL, C_NULL, C_NULL, C_NULL))
    persistent && bcheck(ccall((:tp_batch_set_mode, libtp), Cint, (Ptr{Cvoid}, Int32),
                               b[], Int32(1)))
    bcheck(ccall((:tp_batch_capture, libtp), Cint, (Ptr{Cvoid}, Int64, Float64),
                 b[], steps, growth))
    return b[]
end

batch_launch!(b) = ccall((:tp_batch_launch, libtp), Cint, (Ptr{Cvoid}, Ptr{Cvoid}),
                         b, CUDA.stream().handle)
batch_sync!(b) = ccall((:tp_batch_sync, libtp), Cint, (Ptr{Cvoid},), b)
batch_destroy!(b) = ccall((:tp_batch_destroy, libtp), Cint, (Ptr{Cvoid},), b)

end # module
