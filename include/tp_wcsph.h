/*
 * tp_wcsph.h — C ABI of the GB300 (sm_103a) weakly-compressible SPH right-hand side.
 *
 * This library is a drop-in backend for the WCSPH hot path of TrixiParticles.jl:
 * the fluid/wall system pair
 *   WeaklyCompressibleSPHSystem(ContinuityDensity, WendlandC2Kernel, StateEquationCole,
 *                               ArtificialViscosityMonaghan, DensityDiffusionMolteniColagrossi)
 *   WallBoundarySystem(BoundaryModelDummyParticles(AdamiPressureExtrapolation))
 * under Semidiscretization(...; neighborhood_search=GridNeighborhoodSearch{d}(;
 * cell_list=FullGridCellList(...)), parallelization_backend=<GPU>).
 *
 * Each entry point names the reference function it replaces (paths are relative to the
 * TrixiParticles.jl source tree).  All array arguments of the compute entry points are
 * DEVICE pointers (CUDA global memory) in the reference's column-major SoA layout:
 *   u_ode : (ndims,   n_fluid)  -> particle i, component k at u_ode[i*ndims + k]
 *   v_ode : (ndims+1, n_fluid)  -> velocity in rows 0..ndims-1, density in row ndims
 *   dv_ode: same layout as v_ode;  du_ode: same layout as u_ode.
 * (src/general/semidiscretization.jl:457-508 wrap_u/wrap_v;
 *  src/schemes/fluid/weakly_compressible_sph/system.jl:232-242 v_nvariables.)
 *
 * Calls on one handle are serialised on the handle's CUDA stream and are asynchronous
 * with respect to the host: call tp_sync() (or synchronise the stream) before reading
 * results on the host.  Errors found on the device (a particle outside the cell grid,
 * a non-finite coordinate) are latched in a device word and returned by the next
 * tp_sync() as TP_ERR_OUT_OF_GRID / TP_ERR_NONFINITE.  No entry point aborts the process.
 */
#ifndef TP_WCSPH_H
#define TP_WCSPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TP_ABI_VERSION 1

typedef enum tp_status {
    TP_OK = 0,
    TP_ERR_ARGUMENT = 1,        /* invalid argument (null pointer, bad size, bad config)  */
    TP_ERR_CUDA = 2,            /* a CUDA runtime call failed                             */
    TP_ERR_OUT_OF_GRID = 3,     /* a particle left the FullGridCellList bounding box      */
    TP_ERR_NOT_READY = 4,       /* wall geometry / masses not set yet                     */
    TP_ERR_UNSUPPORTED = 5,     /* configuration outside the implemented hot path         */
    TP_ERR_NONFINITE = 6,       /* NaN or Inf coordinate seen by the neighbour search     */
    TP_ERR_CAPACITY = 7         /* request larger than a fixed capacity                   */
} tp_status;

/* Arithmetic form of the pair kernels. */
enum {
    TP_PRECISION_FP64 = 0, /* plain drop-in: every quantity in Float64, like the reference  */
    TP_PRECISION_FP32 = 1  /* precision form: FP32 pair arithmetic on cell-relative offsets,
                              Kahan-compensated FP32 sums, FP64 positions and reductions  */
};

enum { TP_VISCOSITY_NONE = 0, TP_VISCOSITY_MONAGHAN = 1 };
enum { TP_DIFFUSION_NONE = 0, TP_DIFFUSION_MOLTENI_COLAGROSSI = 1 };

/*
 * Plain-old-data configuration.  Field meanings follow the reference constructors:
 *   smoothing_length      WeaklyCompressibleSPHSystem(...; smoothing_length) and the wall
 *                         BoundaryModelDummyParticles smoothing length (must be equal here);
 *                         the kernel is WendlandC2Kernel{ndims} (compact support 2h).
 *   reference_density,sound_speed,exponent,background_pressure
 *                         StateEquationCole (state_equations.jl:100-139); the same EOS is used
 *                         by the fluid and by the Adami wall model.
 *   fluid_clip_negative_pressure   StateEquationCole(...; clip_negative_pressure)
 *   wall_clip_negative_pressure    BoundaryModelDummyParticles(...; clip_negative_pressure)
 *   viscosity_*           ArtificialViscosityMonaghan(alpha, beta, epsilon) (viscosity.jl:68-132)
 *   density_diffusion_delta  DensityDiffusionMolteniColagrossi(delta) (density_diffusion.jl:41-55)
 *   acceleration          fluid system gravity (semidiscretization.jl:701-731)
 *   pressure_offset       AdamiPressureExtrapolation(pressure_offset) (dummy_particles.jl:142-149)
 *   min_corner/max_corner FullGridCellList(; min_corner, max_corner); every particle must stay
 *                         inside this box (the grid adds one padding layer of cells per side).
 */
typedef struct tp_config {
    int32_t ndims;                       /* 2 or 3                                          */
    int32_t precision;                   /* TP_PRECISION_*                                  */
    int64_t n_fluid;                     /* integrated fluid particles (>= 0)               */
    int64_t n_wall;                      /* dummy wall particles (>= 0)                     */
    double smoothing_length;
    double reference_density;
    double sound_speed;
    double exponent;
    double background_pressure;
    int32_t fluid_clip_negative_pressure;
    int32_t wall_clip_negative_pressure;
    int32_t viscosity_model;             /* TP_VISCOSITY_*                                  */
    int32_t density_diffusion_model;     /* TP_DIFFUSION_*                                  */
    double viscosity_alpha;
    double viscosity_beta;
    double viscosity_epsilon;
    double density_diffusion_delta;
    double acceleration[3];
    double pressure_offset;
    double min_corner[3];
    double max_corner[3];
} tp_config;

typedef struct tp_handle tp_handle;

/* Version of this ABI (TP_ABI_VERSION). */
int32_t tp_abi_version(void);

/* Fill *cfg with the reference defaults (Monaghan alpha=0.02 beta=0 epsilon=0.01,
 * Molteni-Colagrossi delta=0.1, no clipping, zero offsets).  Sizes and bounds stay zero. */
void tp_config_default(tp_config* cfg);

/*
 * Create a handle: validates the configuration, lays out the cell grid and allocates the
 * device buffers.  Replaces the device-side part of
 * semidiscretize (src/general/semidiscretization.jl:293-396: allocate, initialize NHS,
 * Adapt systems to the device) for the supported system pair.
 */
tp_status tp_create(const tp_config* cfg, tp_handle** out);
tp_status tp_destroy(tp_handle* h);

/* Use `stream` (a cudaStream_t, may be NULL = legacy default stream) for every launch. */
tp_status tp_set_stream(tp_handle* h, void* stream);

/*
 * Static wall: coordinates (ndims, n_wall) and hydrodynamic masses (n_wall), device pointers.
 * Builds the wall cell list once (walls do not move: WallBoundarySystem.ismoving = false,
 * neighborhood_search.jl:509-519, 671-686).
 */
tp_status tp_set_wall(tp_handle* h, const double* x_wall, const double* m_wall);

/* Fluid masses (n_fluid), device pointer (WeaklyCompressibleSPHSystem.mass). */
tp_status tp_set_fluid_mass(tp_handle* h, const double* m_fluid);

/*
 * One right-hand-side evaluation dv = kick!(v, u) (semidiscretization.jl:589-612):
 * zero dv -> neighbour search update -> fluid EOS -> Adami wall pressure -> fluid-fluid and
 * fluid-wall interactions (weakly_compressible_sph/rhs.jl:5-127) -> gravity.
 * `dv_ode` must not alias `v_ode`/`u_ode`.  `t` is accepted for interface parity (unused:
 * the supported RHS is autonomous).
 */
tp_status tp_kick(tp_handle* h, double* dv_ode, const double* v_ode, const double* u_ode,
                  double t);

/* du = drift!(v, u) (semidiscretization.jl:522-536, 561-571): du[:, i] = v[1:ndims, i]. */
tp_status tp_drift(tp_handle* h, double* du_ode, const double* v_ode, const double* u_ode,
                   double t);

/*
 * `n_steps` steps of the five-stage fourth-order low-storage Runge-Kutta method
 * CarpenterKennedy2N54(williamson_condition=false) at fixed `dt`, advancing v_ode and u_ode
 * in place (device pointers).  Every stage evaluates kick!/drift! exactly as tp_kick/tp_drift,
 * fused with the 2N register update.  Replaces the OrdinaryDiffEq stage loop that calls
 * kick!/drift! five times per step.  Particles are kept physically ordered by cell inside the
 * library (the SortingCallback idea, src/callbacks/sorting.jl:116-158); v_ode/u_ode are
 * written back in the caller's particle order.
 */
tp_status tp_integrate_ck2n54(tp_handle* h, double* v_ode, double* u_ode, double t0,
                              double dt, int64_t n_steps);

/* Fluid pressure (n_fluid) of the last right-hand side evaluation, in caller order
 * (system.jl:426-438): the last tp_kick, or the last stage of the last step of
 * tp_integrate_ck2n54 / tp_integrate_spv, as the reference's pressure cache holds after solve.
 * TP_ERR_NOT_READY when an unconditional reordering (tp_sort_particles, tp_interpolate_points
 * without walls, tp_nhs_debug, the adjoint) came after it. */
tp_status tp_fluid_pressure(tp_handle* h, double* p_fluid);

/* Wall pressure, density and kernel volume sum (n_wall each, caller order) from the last
 * Adami update (dummy_particles.jl:489-569).  Any pointer may be NULL. */
tp_status tp_wall_state(tp_handle* h, double* p_wall, double* rho_wall, double* volume_wall);

/*
 * Neighbour-search diagnostics for coordinates u_ode (device pointers, all int32, any may be
 * NULL):  cell[i]      linear cell index of fluid particle i (x fastest) in the padded grid,
 *         order[k]     fluid particle index at position k of the cell-sorted order
 *                      (stable: ties broken by ascending particle index),
 *         nnb_ff[i]    fluid neighbours b of fluid particle i with |x_i - x_b|^2 <= (2h)^2
 *                      (i itself included, as the reference's foreach_neighbor visits it),
 *         nnb_fw[i]    wall neighbours of fluid particle i, same criterion,
 *         nnb_wf[w]    fluid neighbours of wall particle w, same criterion.
 */
tp_status tp_nhs_debug(tp_handle* h, const double* u_ode, int32_t* cell, int32_t* order,
                       int32_t* nnb_ff, int32_t* nnb_fw, int32_t* nnb_wf);

/* Diagnostic (parity checks): the divisions the pair kernels use where the reference writes
 * `div_fast` (src/util.jl:3-5, its CUDA definitions ext/TrixiParticlesCUDAExt.jl:12-32), run on
 * the device over n device elements:  out64[i] = x64 / y64[i] as the FP64 drop-in divides (the
 * approximate reciprocal rcp.approx.ftz.f64 refined by one cubic step, then multiplied),
 * out32[i] = x32 / y32[i] as the FP32 form divides (__fdividef).  Either pair of arrays may be
 * NULL.  Asynchronous on the handle's stream. */
tp_status tp_div_fast(tp_handle* h, double x64, const double* y64, double* out64, float x32,
                      const float* y32, float* out32, int64_t n);

/* Diagnostic (parity checks): the pair distance of the FP64 kernels, r[i] = |x_ab| from
 * d2[i] = |x_ab|^2 (> 0, normal) as the pair and Adami kernels form it (the approximate
 * reciprocal square root rsqrt.approx.ftz.f64 refined by one third-order step, times d2; the
 * reference takes sqrt, src/schemes/fluid/weakly_compressible_sph/rhs.jl:27), over n device
 * elements.  Asynchronous on the handle's stream. */
tp_status tp_pair_distance(tp_handle* h, const double* d2, double* r, int64_t n);

/* Grid layout: dims[0..2] cells per dimension (padding included), *cell_size = 2h. */
tp_status tp_grid_info(tp_handle* h, int32_t dims[3], double* cell_size, double lo[3]);

/*
 * Conservation reductions over the fluid in FP64 (the quantities of
 * src/general/custom_quantities.jl:6-57): out[0] = total mass, out[1..3] = linear momentum
 * (out[3] = 0 in 2D), out[4] = kinetic energy.  v_ode is a device pointer, `out` is HOST
 * memory; the call synchronises the handle's stream.  Partial sums are combined in a fixed
 * order, so the result is deterministic.
 */
tp_status tp_conservation(tp_handle* h, const double* v_ode, double out[5]);

/* Block until all work on the handle's stream is done; returns latched device errors. */
tp_status tp_sync(tp_handle* h);

/* Per-phase device time (ms), summed over the RHS evaluations of the last tp_kick /
 * tp_integrate_ck2n54 call, when timing is enabled.  Phases carry the reference's TimerOutputs
 * labels (semidiscretization.jl:596-609): 0 "update nhs" (neighbour search incl. the fluid EOS
 * pack), 1 "compute boundary pressure" (Adami), 2 "system interaction" (pair kernel with the
 * fused Runge-Kutta update).  Events are read back once at the end of the call, so timing adds
 * no synchronisation inside the stage loop.  Returns the number of phases. */
int32_t tp_phase_times(tp_handle* h, double* ms, int32_t n);
tp_status tp_enable_timing(tp_handle* h, int32_t enable);

/*
 * Neighbour-list skin of tp_integrate_ck2n54 (default 0.05): candidate lists are built at radius
 * 2h (1 + skin) and reused across Runge-Kutta stages until some particle has moved more than
 * skin * h since the last rebuild (checked on the device every stage); pairs are still decided
 * exactly with |x_a - x_b|^2 <= (2h)^2 at each stage, so the skin changes speed, not results.
 * 0 rebuilds the cell list and the lists at every stage, as the reference's update_nhs! does.
 */
tp_status tp_set_skin(tp_handle* h, double skin);

/*
 * Sizes the neighbour lists once for coordinates u_ode (device pointer) with room for `growth`
 * times the densest cell seen now (>= 1), allocates the integrator state, and fixes both: later
 * tp_kick / tp_integrate_ck2n54 calls then issue no host synchronisation and no allocation, so
 * they can be recorded into a CUDA graph (a list that still overflows is reported as
 * TP_ERR_CAPACITY by tp_sync).  Without this call the lists are re-sized at every call; a later
 * tp_set_skin with a different skin also returns to that mode.  While a stream capture is
 * active on the handle's stream, tp_integrate_ck2n54 requires this call first (and timing off)
 * and fails with TP_ERR_ARGUMENT otherwise.  A captured graph refers to the handle's device
 * buffers: a later call that grows them (a larger growth or skin) requires a new capture.
 */
tp_status tp_prepare_lists(tp_handle* h, const double* u_ode, double growth);

/*
 * Pair-pass mode.  FP64 drop-in: TP_PAIR_GATHER (default): every fluid particle sums its own pair
 * terms in the reference's neighbour order (bitwise reproducible run to run).
 * TP_PAIR_SYMMETRIC: every fluid-fluid pair is evaluated once and its two halves go to both
 * particles (the second by an FP64 atomic add), which cuts the FP64 arithmetic per pair by about
 * 40 %; the terms are the same, their summation order is not, so results differ from the gather
 * mode in the last bits and are not bitwise reproducible.  On GB300 the symmetric pass is not
 * faster (lane imbalance of the half lists and atomic traffic eat the saving); it is kept for
 * GPUs with a different FP64 / atomic balance.
 * FP32 form: TP_PAIR_GATHER (default) walks per-particle neighbour lists built at a rebuild;
 * TP_PAIR_TILED builds no fluid lists: each warp stages the candidate cell rows of its particles
 * in shared memory and evaluates the pairs from there (the same neighbour set and pair terms; the
 * summation order differs).  Other combinations return TP_ERR_ARGUMENT.
 */
enum { TP_PAIR_GATHER = 0, TP_PAIR_SYMMETRIC = 1, TP_PAIR_TILED = 2 };
tp_status tp_set_pair_mode(tp_handle* h, int32_t mode);

/*
 * interpolate_points (src/general/interpolation.jl:480-697) at n_points points (device array,
 * (ndims, n_points) reference layout) from the fluid state (v_ode, u_ode): the SPH interpolation
 * with the WendlandC2 kernel of smoothing length `smoothing_length` (support 2 h), after the
 * system update the reference performs first (fluid pressure from the current density; the
 * Adami wall state when walls take part).  Outputs (device arrays): computed_density
 * (sum m_b W), velocity (ndims, n_points), pressure, density (Shepard-normalised), and
 * neighbor_count; points where computed_density < eps() -- or, with cut_off_bnd, where the wall
 * particles add more kernel-weighted mass than the fluid -- get NaN and a zero count.
 * clip_negative_pressure clips the interpolated pressure contributions at 0;
 * include_wall_velocity renormalises the velocity with the wall particles' volume (fixed walls:
 * zero velocity).  Points must lie inside the FullGridCellList box.  FP64 in both precision
 * forms.  Asynchronous on the handle's stream.
 */
tp_status tp_interpolate_points(tp_handle* h, const double* v_ode, const double* u_ode,
                                const double* points, int64_t n_points, double smoothing_length,
                                int32_t cut_off_bnd, int32_t clip_negative_pressure,
                                int32_t include_wall_velocity, double* computed_density,
                                double* velocity, double* pressure, double* density,
                                int32_t* neighbor_count);

/* Copy of the configuration the handle was created with. */
tp_status tp_get_config(const tp_handle* h, tp_config* out);

/* Threads per block of the pair and Adami kernels: 64, 128 (default) or 256 (autotuning). */
tp_status tp_set_launch(tp_handle* h, int32_t pair_block);

/*
 * SymplecticPositionVerlet (ext/TrixiParticlesOrdinaryDiffEqSymplecticRKExt.jl:89-171): n_steps
 * steps of size dt on (v_ode, u_ode) in place, two kick! evaluations per step -- half drift,
 * half kick, kick at the midpoint, velocity update, the scheme's density update
 * rho = rho_prev (2 - eps) / (2 + eps) with eps = -(drho/dt) dt / rho_half, second half drift.
 * Each kick rebuilds the neighbour search from the caller-ordered state (as tp_kick).
 */
tp_status tp_integrate_spv(tp_handle* h, double* v_ode, double* u_ode, double t0, double dt,
                           int64_t n_steps);

/*
 * SortingCallback's sort_particles! (src/callbacks/sorting.jl:116-158): reorders the fluid
 * particles of (v_ode, u_ode) in place by their neighbour-search cell -- the stable order of the
 * lexicographic cell coordinates (cx, cy, cz), as Julia's sortperm over SVector cell coordinates
 * -- and writes the permutation (new position j holds old particle perm_out[j], 0-based) when
 * perm_out is non-null (device).  The reference moves coordinates, velocity, density and
 * pressure but not the masses (a TODO there); sort_masses = 0 keeps that behaviour, 1 also
 * moves the handle's fluid masses with their particles.  Asynchronous.
 */
tp_status tp_sort_particles(tp_handle* h, double* v_ode, double* u_ode, int32_t sort_masses,
                            int32_t* perm_out);

/* Number of CUDA kernels this handle has launched so far (diagnostics; memcpys not counted). */
int64_t tp_kernel_launches(const tp_handle* h);

/* Number of neighbour-search rebuilds (cell list + neighbour lists) the displacement gate of
 * tp_kick / tp_integrate_ck2n54 has let through since tp_create (diagnostics, the counterpart of
 * how often the reference's update_nhs! would have had to move a particle between cells).  HOST
 * `count`; synchronises the handle's stream. */
tp_status tp_rebuild_count(tp_handle* h, int64_t* count);

/*
 * Cell sort without any device allocation.  This entry point has no counterpart in the
 * reference: it serves callers that must not allocate device memory -- a host that owns all
 * device memory through its own pool (a Julia process running CUDA.jl) or a fixed-budget
 * real-time loop -- and gives them the neighbour-search counting sort of this library:
 * cell[i] and order[k] exactly as tp_nhs_debug returns them, for `n` particles with
 * coordinates u (ndims, n) on the grid that `cfg` describes (ndims, smoothing_length,
 * min_corner, max_corner; the other fields are ignored).  u, cell and order are device
 * pointers; `stream` is a cudaStream_t (NULL = legacy default stream).
 * All scratch lives in one fixed device array owned by the library (about 10 MB, held by every
 * GPU that loads the library until the process exits): at most TP_NOALLOC_MAX_PARTICLES
 * particles and TP_NOALLOC_MAX_CELLS grid cells (padding included), larger requests return
 * TP_ERR_CAPACITY before any GPU work.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) in the context current at the call, so switching contexts or devices
 * between calls is safe.  Calls share the scratch: the call clears what must start at zero, and
 * calls that overlap on the GPU race, so serialise them.  The call is synchronous: it returns
 * after the sort has finished (it synchronises `stream`) and reports TP_ERR_OUT_OF_GRID /
 * TP_ERR_NONFINITE directly, so it must not be called while `stream` is being captured into a
 * CUDA graph.  It calls no cudaMalloc, cudaFree or allocating library routine.
 */
#define TP_NOALLOC_MAX_PARTICLES 262144
#define TP_NOALLOC_MAX_CELLS 524288
tp_status tp_cell_sort_noalloc(const tp_config* cfg, const double* u, int64_t n, int32_t* cell,
                               int32_t* order, void* stream);

/*
 * Differentiation form: reverse-mode gradients of a CarpenterKennedy2N54 trajectory.  Stands
 * where the reference would take gradients through `solve` with ChainRulesCore rules (the
 * Julia shim defines an rrule over these two calls); the reference itself ships no adjoint.
 *
 * tp_adjoint_forward advances (v_ode, u_ode) in place by n_steps steps of size dt, exactly
 * like tp_integrate_ck2n54 but in caller order with neighbour lists rebuilt at the start of
 * every step and held fixed for its five stages, and records a checkpoint of the state every
 * `checkpoint_every` steps on the device.  Arithmetic follows the handle's precision (FP32
 * form: FP32 pair arithmetic and adjoint; FP64: everything in FP64).  Synchronises once at the
 * end (error check).
 *
 * tp_adjoint_backward takes the cotangents of the final state -- v_bar (ndims+1, n_fluid:
 * velocity rows, then the density row) and u_bar (ndims, n_fluid), device arrays in the
 * reference layout -- and overwrites them with the cotangents of the initial state (the
 * gradient with respect to v0 / rho0 and u0).  params_bar (host, 3 doubles) receives the
 * gradient with respect to (Monaghan alpha, Molteni-Colagrossi delta, gravity magnitude along
 * the configured acceleration), reduced in FP64.  Each k-step segment is recomputed from its
 * checkpoint and reversed stage by stage.  Needs a preceding tp_adjoint_forward on the handle;
 * may be called again with other cotangents.
 */
tp_status tp_adjoint_forward(tp_handle* h, double* v_ode, double* u_ode, double dt,
                             int64_t n_steps, int64_t checkpoint_every);
tp_status tp_adjoint_backward(tp_handle* h, double* v_bar, double* u_bar, double params_bar[3]);
/* Kernel launches issued by the differentiation form on this handle (diagnostics). */
int64_t tp_adjoint_kernel_launches(const tp_handle* h);

/*
 * Batching form: many independent simulations per CUDA-graph launch.  Stands where the
 * reference would run an ensemble as separate `solve` calls (one per simulation); the
 * reference has no batched entry point.  A batch bundles handles -- each a group of instances
 * that share one cell grid (instances of equal spacing side by side, separated by gaps wider
 * than the kernel support, so that they never interact) -- with their device state (v_ode,
 * u_ode in the reference layout, integrated in place) and time step.
 *   tp_batch_autotune: per member, times `trial_steps` steps on scratch copies of the state
 *     for every pair pass (neighbour lists; in the FP32 form also cell tiles staged in shared
 *     memory, TP_PAIR_TILED) x list skins {0.03, 0.05, 0.1, 0.2} x pair-kernel block sizes
 *     {64, 128, 256} (the tiled pass: 256) and keeps the fastest; outputs (per member, optional):
 *     block size, skin, pair mode, ms per step.
 *   tp_batch_capture: sizes every member's lists for `growth` x the densest cell now
 *     (tp_prepare_lists), warms up on scratch state, then records `steps` steps of every member
 *     into one CUDA graph, the members as parallel branches.
 *   tp_batch_launch: replays the graph on `stream` (asynchronous); tp_batch_sync waits and
 *     reports the first member error.
 * The batch owns one stream per member and sets it on the member handles; tp_batch_destroy
 * resets them to the default stream.  Handles must outlive the batch.
 */
typedef struct tp_batch tp_batch;
tp_status tp_batch_create(tp_handle* const* handles, int32_t n, tp_batch** out);
tp_status tp_batch_destroy(tp_batch* b);
tp_status tp_batch_set_state(tp_batch* b, int32_t member, double* v_ode, double* u_ode, double dt);
tp_status tp_batch_autotune(tp_batch* b, int32_t trial_steps, int32_t* pair_block_out,
                            double* skin_out, int32_t* pair_mode_out, double* ms_out);
tp_status tp_batch_capture(tp_batch* b, int64_t steps, double growth);
tp_status tp_batch_launch(tp_batch* b, void* stream);
tp_status tp_batch_sync(tp_batch* b);
int64_t tp_batch_steps(const tp_batch* b);
/*
 * How tp_batch_capture records the members (no counterpart in the reference).
 * TP_BATCH_BRANCHES (default): every member's fused integrator is one parallel branch of the
 * graph.  TP_BATCH_PERSISTENT (FP32 members on neighbour lists, at most 6, one ndims and model
 * setup): the members' neighbour search, pack and Adami passes stay parallel branches, and the
 * pair stage of all members is one persistent launch per Runge-Kutta stage whose blocks take
 * 256-slot tiles of the members (largest member first) from a work counter.  Results equal the
 * branches mode bit for bit.  A mode change drops the captured graph.
 */
enum { TP_BATCH_BRANCHES = 0, TP_BATCH_PERSISTENT = 1 };
tp_status tp_batch_set_mode(tp_batch* b, int32_t mode);
const char* tp_batch_last_error(const tp_batch* b);

/* Last error message of the handle (or of the last failed tp_create when h is NULL). */
const char* tp_last_error(const tp_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* TP_WCSPH_H */
