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
# kick!/drift! of a Semidiscretization whose backend is GB300Backend call tp_kick/tp_drift
# with the raw device pointers of v_ode/u_ode/dv_ode/du_ode.  Supported system pair:
# WeaklyCompressibleSPHSystem(ContinuityDensity, WendlandC2Kernel, StateEquationCole,
# ArtificialViscosityMonaghan|nothing, DensityDiffusionMolteniColagrossi|nothing) with a
# WallBoundarySystem(BoundaryModelDummyParticles(AdamiPressureExtrapolation)).  Anything else
# throws ArgumentError.  This file is written against the reference sources; Julia is not
# installed where it was written, so it has not been executed.
module TrixiParticlesGB300

using CUDA: CUDA, CuArray, CuMatrix, CuPtr
using KernelAbstractions: KernelAbstractions
using ChainRulesCore: ChainRulesCore
using TrixiParticles: TrixiParticles, WeaklyCompressibleSPHSystem, WallBoundarySystem,
                      BoundaryModelDummyParticles, AdamiPressureExtrapolation,
                      ContinuityDensity, WendlandC2Kernel, StateEquationCole,
                      ArtificialViscosityMonaghan, DensityDiffusionMolteniColagrossi,
                      FullGridCellList

export GB300Backend

const libtp = get(ENV, "TP_WCSPH_LIB",
                  joinpath(@__DIR__, "..", "libtp_wcsph.so"))

# Dispatches like any KernelAbstractions GPU backend, so `semidiscretize` allocates CuArrays.
struct GB300Backend <: KernelAbstractions.GPU
    precision::Int32   # 0 = Float64 drop-in, 1 = FP32 precision form
end
GB300Backend() = GB300Backend(Int32(0))
KernelAbstractions.allocate(::GB300Backend, T, dims) = CuArray{T}(undef, dims)

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

const HANDLES = IdDict{Any, Ptr{Cvoid}}()

function tp_config(fluid, wall, nhs, backend)
    fluid isa WeaklyCompressibleSPHSystem ||
        throw(ArgumentError("GB300Backend supports WeaklyCompressibleSPHSystem only"))
    fluid.density_calculator isa ContinuityDensity ||
        throw(ArgumentError("GB300Backend supports ContinuityDensity only"))
    fluid.smoothing_kernel isa WendlandC2Kernel ||
        throw(ArgumentError("GB300Backend supports WendlandC2Kernel only"))
    isnothing(fluid.correction) || throw(ArgumentError("corrections are not supported"))
    bm = wall.boundary_model
    (bm isa BoundaryModelDummyParticles &&
     bm.density_calculator isa AdamiPressureExtrapolation &&
     isnothing(bm.viscosity)) ||
        throw(ArgumentError("wall must be BoundaryModelDummyParticles(AdamiPressureExtrapolation)"))
    cl = nhs.cell_list
    cl isa FullGridCellList || throw(ArgumentError("GPU execution needs a FullGridCellList"))
    se = fluid.state_equation
    se isa StateEquationCole || throw(ArgumentError("StateEquationCole is required"))
    visc = fluid.viscosity
    dd = fluid.density_diffusion
    nd = ndims(fluid)
    return TpConfig(nd, backend.precision, TrixiParticles.nparticles(fluid),
                    TrixiParticles.nparticles(wall),
                    TrixiParticles.initial_smoothing_length(fluid),
                    se.reference_density, se.sound_speed, se.exponent,
                    se.background_pressure, TrixiParticles.clip_negative_pressure(se),
                    bm.clip_negative_pressure,
                    visc isa ArtificialViscosityMonaghan ? 1 : 0,
                    dd isa DensityDiffusionMolteniColagrossi ? 1 : 0,
                    visc isa ArtificialViscosityMonaghan ? visc.alpha : 0.0,
                    visc isa ArtificialViscosityMonaghan ? visc.beta : 0.0,
                    visc isa ArtificialViscosityMonaghan ? visc.epsilon : 0.01,
                    dd isa DensityDiffusionMolteniColagrossi ? dd.delta : 0.0,
                    pad3(fluid.acceleration),
                    bm.density_calculator.pressure_offset,
                    pad3(cl.min_corner), pad3(cl.max_corner))
end

function handle(semi)
    get!(HANDLES, semi) do
        fluid, wall = semi.systems
        cfg = tp_config(fluid, wall, semi.neighborhood_searches[1][1],
                        semi.parallelization_backend)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(C_NULL, ccall((:tp_create, libtp), Cint, (Ref{TpConfig}, Ref{Ptr{Cvoid}}), cfg, h))
        check(h[], ccall((:tp_set_stream, libtp), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h[],
                         CUDA.stream().handle))
        check(h[], ccall((:tp_set_wall, libtp), Cint, (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}),
                         h[], wall.coordinates, wall.boundary_model.hydrodynamic_mass))
        check(h[], ccall((:tp_set_fluid_mass, libtp), Cint, (Ptr{Cvoid}, CuPtr{Float64}),
                         h[], fluid.mass))
        finalizer(_ -> ccall((:tp_destroy, libtp), Cint, (Ptr{Cvoid},), h[]), semi)
        h[]
    end
end

const GB300Semi = TrixiParticles.Semidiscretization{<:Any, <:Any, <:Any, <:Any, <:GB300Backend}

# kick! (src/general/semidiscretization.jl:589-612)
function TrixiParticles.kick!(dv_ode, v_ode, u_ode, p::NamedTuple{(:semi, :split_integration_data), <:Tuple{GB300Semi, Any}}, t)
    h = handle(p.semi)
    check(h, ccall((:tp_kick, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Float64),
                   h, dv_ode, v_ode, u_ode, t))
    return dv_ode
end

# drift! (src/general/semidiscretization.jl:522-536)
function TrixiParticles.drift!(du_ode, v_ode, u_ode, p::NamedTuple{(:semi, :split_integration_data), <:Tuple{GB300Semi, Any}}, t)
    h = handle(p.semi)
    check(h, ccall((:tp_drift, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Float64),
                   h, du_ode, v_ode, u_ode, t))
    return du_ode
end

# Whole CarpenterKennedy2N54 steps in one call (device arrays are advanced in place).
function integrate_ck2n54!(semi, v_ode, u_ode, t0, dt, nsteps)
    h = handle(semi)
    check(h, ccall((:tp_integrate_ck2n54, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Float64, Int64),
                   h, v_ode, u_ode, t0, dt, nsteps))
    check(h, ccall((:tp_sync, libtp), Cint, (Ptr{Cvoid},), h))
    return v_ode, u_ode
end

# ---- SymplecticPositionVerlet, SortingCallback's sort, interpolation ----------------------
function integrate_spv!(semi, v_ode, u_ode, t0, dt, nsteps)
    h = handle(semi)
    check(h, ccall((:tp_integrate_spv, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Float64, Int64),
                   h, v_ode, u_ode, t0, dt, nsteps))
    return v_ode, u_ode
end

# sort_particles! of SortingCallback (the reference leaves masses in place: sort_masses=false)
function sort_particles!(semi, v_ode, u_ode; sort_masses=false)
    h = handle(semi)
    perm = CUDA.zeros(Int32, length(u_ode) ÷ ndims(semi.systems[1]))
    check(h, ccall((:tp_sort_particles, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Int32, CuPtr{Int32}),
                   h, v_ode, u_ode, sort_masses, perm))
    return perm .+ Int32(1)
end

function interpolate_points(points::CuMatrix{Float64}, semi, v_ode, u_ode; smoothing_length,
                            cut_off_bnd=true, clip_negative_pressure=false,
                            include_wall_velocity=false)
    h = handle(semi)
    n = size(points, 2)
    cd, p, rho = CUDA.zeros(n), CUDA.zeros(n), CUDA.zeros(n)
    vel = CUDA.zeros(size(points, 1), n)
    count = CUDA.zeros(Int32, n)
    check(h, ccall((:tp_interpolate_points, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64}, Int64, Float64,
                    Int32, Int32, Int32, CuPtr{Float64}, CuPtr{Float64}, CuPtr{Float64},
                    CuPtr{Float64}, CuPtr{Int32}),
                   h, v_ode, u_ode, points, n, smoothing_length, cut_off_bnd,
                   clip_negative_pressure, include_wall_velocity, cd, vel, p, rho, count))
    return (; computed_density=cd, point_coords=points, neighbor_count=count, velocity=vel,
            pressure=p, density=rho)
end

# ---- Differentiation form: rrule of a fixed-step CarpenterKennedy2N54 solve -------------
# Forward: tp_adjoint_forward advances (v, u) in place and checkpoints every `every` steps.
# Pullback: tp_adjoint_backward maps the cotangents of the final (v, u) to those of the initial
# (v0, u0) and returns the gradient with respect to (alpha, delta, |g|) of the handle's config.
function solve_ck2n54(semi, v0::CuArray{Float64}, u0::CuArray{Float64}, dt, nsteps; every=25)
    h = handle(semi)
    v, u = copy(v0), copy(u0)
    check(h, ccall((:tp_adjoint_forward, libtp), Cint,
                   (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Float64, Int64, Int64),
                   h, v, u, dt, nsteps, every))
    return v, u
end

function ChainRulesCore.rrule(::typeof(solve_ck2n54), semi, v0, u0, dt, nsteps; every=25)
    v, u = solve_ck2n54(semi, v0, u0, dt, nsteps; every)
    function solve_ck2n54_pullback(ȳ)
        v̄, ū = ChainRulesCore.unthunk.(ȳ)
        vb = v̄ isa ChainRulesCore.AbstractZero ? CUDA.zeros(Float64, size(v)) : copy(v̄)
        ub = ū isa ChainRulesCore.AbstractZero ? CUDA.zeros(Float64, size(u)) : copy(ū)
        params = zeros(Float64, 3)   # (alpha, delta, gravity magnitude)
        h = handle(semi)
        check(h, ccall((:tp_adjoint_backward, libtp), Cint,
                       (Ptr{Cvoid}, CuPtr{Float64}, CuPtr{Float64}, Ptr{Float64}),
                       h, vb, ub, params))
        semī = ChainRulesCore.Tangent{typeof(semi)}(; parameters=params)
        return (ChainRulesCore.NoTangent(), semī, vb, ub,
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return (v, u), solve_ck2n54_pullback
end

# ---- Batching form: several Semidiscretizations per CUDA-graph launch ----------------------
# members: Vector of (semi, v::CuArray, u::CuArray, dt).  Returns the batch pointer.
function batch_create(members; steps=5, autotune=true, growth=1.5)
    hs = [handle(m[1]) for m in members]
    b = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:tp_batch_create, libtp), Cint, (Ptr{Ptr{Cvoid}}, Int32, Ref{Ptr{Cvoid}}),
               hs, length(hs), b)
    st == 0 || error("tp_batch_create failed ($st)")
    bcheck(st) = st == 0 || error(unsafe_string(ccall((:tp_batch_last_error, libtp), Cstring,
                                                      (Ptr{Cvoid},), b[])))
    for (k, (semi, v, u, dt)) in enumerate(members)
        bcheck(ccall((:tp_batch_set_state, libtp), Cint,
                     (Ptr{Cvoid}, Int32, CuPtr{Float64}, CuPtr{Float64}, Float64),
                     b[], k - 1, v, u, dt))
    end
    autotune && bcheck(ccall((:tp_batch_autotune, libtp), Cint,
                             (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}),
                             b[], 3, C_NULL, C_NULL, C_NULL))
    bcheck(ccall((:tp_batch_capture, libtp), Cint, (Ptr{Cvoid}, Int64, Float64),
                 b[], steps, growth))
    return b[]
end

batch_launch!(b) = ccall((:tp_batch_launch, libtp), Cint, (Ptr{Cvoid}, Ptr{Cvoid}),
                         b, CUDA.stream().handle)
batch_sync!(b) = ccall((:tp_batch_sync, libtp), Cint, (Ptr{Cvoid},), b)
batch_destroy!(b) = ccall((:tp_batch_destroy, libtp), Cint, (Ptr{Cvoid},), b)

end # module
