"""Host-side mirror of the reference's WCSPH drop-in surface for the GB300 backend.

Names, argument meanings and errors follow the reference:
    Semidiscretization(fluid_system, boundary_system; neighborhood_search, parallelization_backend)
        src/general/semidiscretization.jl:106-155
    semidiscretize(semi, tspan)            src/general/semidiscretization.jl:293-396
    kick!(dv_ode, v_ode, u_ode, p, t)      src/general/semidiscretization.jl:589-612  -> `kick`
    drift!(du_ode, v_ode, u_ode, p, t)     src/general/semidiscretization.jl:522-536  -> `drift`
    solve(ode, CarpenterKennedy2N54(williamson_condition=false); dt)  (OrdinaryDiffEq)
The ODE state vectors are CUDA float64 tensors (PyTorch provides device memory and streams only);
every computation runs in libtp_wcsph.so through its C ABI.  Unsupported system combinations
raise ValueError, as the reference raises ArgumentError (docs/src/development.md:96).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .setups import InitialCondition, StateEquationCole


# ------------------------------------------------------------------------------------------
# Model tags (constructor keywords as in the reference)
# ------------------------------------------------------------------------------------------
@dataclass(frozen=True)
class WendlandC2Kernel:
    ndims: int


@dataclass(frozen=True)
class ContinuityDensity:
    pass


@dataclass(frozen=True)
class ArtificialViscosityMonaghan:
    alpha: float
    beta: float = 0.0
    epsilon: float = 0.01


@dataclass(frozen=True)
class DensityDiffusionMolteniColagrossi:
    delta: float


@dataclass(frozen=True)
class AdamiPressureExtrapolation:
    pressure_offset: float = 0.0
    allow_loop_flipping: bool = True


@dataclass
class BoundaryModelDummyParticles:
    initial_density: np.ndarray
    hydrodynamic_mass: np.ndarray
    density_calculator: object
    smoothing_kernel: WendlandC2Kernel
    smoothing_length: float
    viscosity: object = None
    state_equation: StateEquationCole | None = None
    correction: object = None
    clip_negative_pressure: bool = False


@dataclass
class WeaklyCompressibleSPHSystem:
    initial_condition: InitialCondition
    smoothing_kernel: WendlandC2Kernel
    smoothing_length: float
    density_calculator: object
    state_equation: StateEquationCole
    acceleration: tuple | None = None
    viscosity: object = None
    density_diffusion: object = None
    correction: object = None
    surface_tension: object = None
    shifting_technique: object = None

    def __post_init__(self):
        # the constructor's checks and default (weakly_compressible_sph/system.jl:65-174)
        nd = self.ndims
        if self.acceleration is None:
            self.acceleration = (0.0,) * nd
        acc = tuple(float(a) for a in np.atleast_1d(self.acceleration))
        if len(acc) != nd:
            raise _argument_error(f"`acceleration` must be of length {nd} for a {nd}D problem")
        self.acceleration = acc
        if getattr(self.smoothing_kernel, "ndims", nd) != nd:
            raise _argument_error(f"smoothing kernel dimensionality must be {nd} for a {nd}D "
                                  "problem")

    @property
    def ndims(self) -> int:
        return self.initial_condition.ndims


@dataclass
class WallBoundarySystem:
    initial_condition: InitialCondition
    boundary_model: BoundaryModelDummyParticles
    prescribed_motion: object = None


@dataclass
class FullGridCellList:
    min_corner: tuple
    max_corner: tuple


@dataclass
class GridNeighborhoodSearch:
    ndims: int
    cell_list: FullGridCellList | None = None


@dataclass
class GB300Backend:
    """parallelization_backend for the sm_103a library.  precision: "float64" (plain drop-in) or
    "float32" (precision form); device: CUDA device index."""

    precision: str = "float64"
    device: int = 0


# ------------------------------------------------------------------------------------------
# Semidiscretization
# ------------------------------------------------------------------------------------------
def _argument_error(msg: str) -> ValueError:
    return ValueError(f"ArgumentError: {msg}")


class Semidiscretization:
    """Couples one WCSPH fluid system with one Adami dummy-particle wall system."""

    def __init__(self, *systems, neighborhood_search: GridNeighborhoodSearch,
                 parallelization_backend: GB300Backend):
        fluids = [s for s in systems if isinstance(s, WeaklyCompressibleSPHSystem)]
        walls = [s for s in systems if isinstance(s, WallBoundarySystem)]
        if len(fluids) != 1 or len(walls) != 1 or len(systems) != 2:
            raise _argument_error("the GB300 backend supports exactly one "
                                  "WeaklyCompressibleSPHSystem and one WallBoundarySystem")
        self.fluid, self.wall = fluids[0], walls[0]
        self.systems = (self.fluid, self.wall)
        self.neighborhood_search = neighborhood_search
        self.backend = parallelization_backend
        self.config = self._config()
        self._handle = None
        self._lib = None

    # -- validation + C config (check_configuration, semidiscretization.jl:126) --
    def _config(self) -> _abi.TpConfig:
        f, w = self.fluid, self.wall
        bm = w.boundary_model
        nd = f.ndims
        if not isinstance(f.smoothing_kernel, WendlandC2Kernel) or f.smoothing_kernel.ndims != nd:
            raise _argument_error(f"smoothing kernel must be WendlandC2Kernel{{{nd}}}")
        if not isinstance(f.density_calculator, ContinuityDensity):
            raise _argument_error("only ContinuityDensity is supported by the GB300 backend")
        if f.correction is not None or f.surface_tension is not None or \
                f.shifting_technique is not None:
            raise _argument_error("corrections, surface tension and shifting are not supported")
        if f.viscosity is not None and not isinstance(f.viscosity, ArtificialViscosityMonaghan):
            raise _argument_error("only ArtificialViscosityMonaghan is supported")
        if f.density_diffusion is not None and \
                not isinstance(f.density_diffusion, DensityDiffusionMolteniColagrossi):
            raise _argument_error("only DensityDiffusionMolteniColagrossi is supported")
        if not isinstance(bm.density_calculator, AdamiPressureExtrapolation):
            raise _argument_error("the wall model must use AdamiPressureExtrapolation")
        if bm.viscosity is not None or bm.correction is not None or \
                w.prescribed_motion is not None:
            raise _argument_error("wall viscosity, corrections and moving walls are not supported")
        if bm.state_equation is None:  # the reference's check_configuration message
            raise _argument_error("`WeaklyCompressibleSPHSystem` cannot be used without setting "
                                  "a `state_equation` for all boundary models")
        if f.state_equation is None:
            raise _argument_error("ContinuityDensity needs the fluid's `state_equation`")
        if not isinstance(bm.smoothing_kernel, WendlandC2Kernel) or \
                float(bm.smoothing_length) != float(f.smoothing_length):
            raise _argument_error("the wall model must share the fluid's WendlandC2 kernel and "
                                  "smoothing length")
        se, sw = f.state_equation, bm.state_equation
        if (se.sound_speed, se.reference_density, se.exponent, se.background_pressure) != \
                (sw.sound_speed, sw.reference_density, sw.exponent, sw.background_pressure):
            raise _argument_error("fluid and wall must share the state equation")
        nhs = self.neighborhood_search
        if not isinstance(nhs, GridNeighborhoodSearch) or nhs.cell_list is None:
            raise _argument_error("GPU execution requires GridNeighborhoodSearch with a "
                                  "FullGridCellList (docs/src/gpu.md)")
        if not isinstance(self.backend, GB300Backend):
            raise _argument_error("parallelization_backend must be GB300Backend()")
        c = _abi.default_config()
        c.ndims = nd
        c.precision = (_abi.TP_PRECISION_FP32 if self.backend.precision == "float32"
                       else _abi.TP_PRECISION_FP64)
        c.n_fluid = f.initial_condition.n_particles
        c.n_wall = w.initial_condition.n_particles
        c.smoothing_length = float(f.smoothing_length)
        c.reference_density = se.reference_density
        c.sound_speed = se.sound_speed
        c.exponent = se.exponent
        c.background_pressure = se.background_pressure
        c.fluid_clip_negative_pressure = int(bool(se.clip_negative_pressure))
        c.wall_clip_negative_pressure = int(bool(bm.clip_negative_pressure))
        if f.viscosity is None:
            c.viscosity_model = _abi.TP_VISCOSITY_NONE
        else:
            c.viscosity_model = _abi.TP_VISCOSITY_MONAGHAN
            c.viscosity_alpha = f.viscosity.alpha
            c.viscosity_beta = f.viscosity.beta
            c.viscosity_epsilon = f.viscosity.epsilon
        if f.density_diffusion is None:
            c.density_diffusion_model = _abi.TP_DIFFUSION_NONE
        else:
            c.density_diffusion_model = _abi.TP_DIFFUSION_MOLTENI_COLAGROSSI
            c.density_diffusion_delta = f.density_diffusion.delta
        acc = f.acceleration if f.acceleration is not None else (0.0,) * nd
        for d in range(3):
            c.acceleration[d] = float(acc[d]) if d < nd else 0.0
        c.pressure_offset = float(bm.density_calculator.pressure_offset)
        cl = nhs.cell_list
        for d in range(3):
            c.min_corner[d] = float(cl.min_corner[d]) if d < nd else 0.0
            c.max_corner[d] = float(cl.max_corner[d]) if d < nd else 0.0
        return c

    @property
    def ndims(self) -> int:
        return self.fluid.ndims

    @property
    def n_fluid(self) -> int:
        return self.fluid.initial_condition.n_particles

    @property
    def n_wall(self) -> int:
        return self.wall.initial_condition.n_particles

    # -- device side --
    def _ensure_handle(self):
        if self._handle is not None:
            return
        import torch

        self._lib = _abi.load_library()
        if not torch.cuda.is_available():
            raise RuntimeError("GB300Backend needs a CUDA device")
        dev = torch.device("cuda", self.backend.device)
        torch.cuda.set_device(dev)
        h = ctypes.c_void_p()
        st = self._lib.tp_create(ctypes.byref(self.config), ctypes.byref(h))
        _abi.check(self._lib, None, st)
        self._handle = h
        self.device = dev
        nd = self.ndims
        wall = self.wall.initial_condition
        x_w = torch.as_tensor(np.ascontiguousarray(wall.coordinates, dtype=np.float64),
                              device=dev).reshape(-1)
        m_w = torch.as_tensor(np.ascontiguousarray(self.wall.boundary_model.hydrodynamic_mass,
                                                   dtype=np.float64), device=dev)
        m_f = torch.as_tensor(np.ascontiguousarray(self.fluid.initial_condition.mass,
                                                   dtype=np.float64), device=dev)
        self._x_w, self._m_w, self._m_f = x_w, m_w, m_f
        self._set_stream()
        self._call("tp_set_wall", x_w.data_ptr(), m_w.data_ptr())
        self._call("tp_set_fluid_mass", m_f.data_ptr())
        assert x_w.numel() == nd * self.n_wall

    def _set_stream(self):
        import torch

        s = torch.cuda.current_stream(self.device).cuda_stream
        self._lib.tp_set_stream(self._handle, ctypes.c_void_p(s))

    def _call(self, name: str, *args):
        st = getattr(self._lib, name)(self._handle, *args)
        _abi.check(self._lib, self._handle, st)

    def close(self):
        if self._handle is not None and self._lib is not None:
            self._lib.tp_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- wrap_v / wrap_u (semidiscretization.jl:457-488) --
    def wrap_v(self, v_ode):
        return v_ode.view(self.n_fluid, self.ndims + 1)

    def wrap_u(self, u_ode):
        return u_ode.view(self.n_fluid, self.ndims)

    def sync(self):
        """tp_sync: waits for the device and raises latched device errors."""
        self._call("tp_sync")

    def fluid_pressure(self):
        import torch

        p = torch.empty(self.n_fluid, dtype=torch.float64, device=self.device)
        self._set_stream()
        self._call("tp_fluid_pressure", p.data_ptr())
        return p

    def wall_state(self):
        import torch

        out = [torch.empty(self.n_wall, dtype=torch.float64, device=self.device) for _ in range(3)]
        self._set_stream()
        self._call("tp_wall_state", *[t.data_ptr() for t in out])
        return tuple(out)

    def nhs_debug(self, u_ode):
        import torch

        nf, nw = self.n_fluid, self.n_wall
        out = [torch.empty(n, dtype=torch.int32, device=self.device)
               for n in (nf, nf, nf, nf, nw)]
        self._set_stream()
        self._call("tp_nhs_debug", u_ode.data_ptr(), *[t.data_ptr() for t in out])
        return dict(zip(("cell", "order", "nnb_ff", "nnb_fw", "nnb_wf"), out))

    def conservation(self, v_ode):
        out = (ctypes.c_double * 5)()
        self._set_stream()
        self._call("tp_conservation", v_ode.data_ptr(), out)
        return np.array(list(out))

    def grid_info(self):
        dims = (ctypes.c_int32 * 3)()
        cs = ctypes.c_double()
        lo = (ctypes.c_double * 3)()
        self._call("tp_grid_info", dims, ctypes.byref(cs), lo)
        return tuple(dims), cs.value, tuple(lo)


@dataclass
class ODEProblem:
    """DynamicalODEProblem(kick!, drift!, v0, u0, tspan, p) (semidiscretization.jl:391-395)."""

    v0: object
    u0: object
    tspan: tuple
    p: dict = field(default_factory=dict)


def semidiscretize(semi: Semidiscretization, tspan) -> ODEProblem:
    """Allocate v0/u0 on the device, write the initial conditions (fluid.jl:79-97,
    weakly_compressible_sph/system.jl:440-445: density in the last v row) and set up the
    library handle (cell grid, static wall cell list, masses)."""
    import torch

    semi._ensure_handle()
    ic = semi.fluid.initial_condition
    nd = semi.ndims
    v0 = np.empty((ic.n_particles, nd + 1), dtype=np.float64)
    v0[:, :nd] = ic.velocity
    v0[:, nd] = ic.density
    u0 = np.ascontiguousarray(ic.coordinates, dtype=np.float64)
    v0_t = torch.as_tensor(v0.reshape(-1), device=semi.device).contiguous()
    u0_t = torch.as_tensor(u0.reshape(-1), device=semi.device).contiguous()
    return ODEProblem(v0=v0_t, u0=u0_t, tspan=tuple(tspan), p={"semi": semi})


def kick(dv_ode, v_ode, u_ode, p, t):
    """kick!: dv_ode <- RHS(v_ode, u_ode).  Asynchronous on the current torch stream."""
    semi = p["semi"]
    semi._set_stream()
    semi._call("tp_kick", dv_ode.data_ptr(), v_ode.data_ptr(), u_ode.data_ptr(),
               ctypes.c_double(float(t)))
    return dv_ode


def drift(du_ode, v_ode, u_ode, p, t):
    """drift!: du_ode <- v_ode[1:ndims, :]."""
    semi = p["semi"]
    semi._set_stream()
    semi._call("tp_drift", du_ode.data_ptr(), v_ode.data_ptr(), u_ode.data_ptr(),
               ctypes.c_double(float(t)))
    return du_ode


@dataclass(frozen=True)
class CarpenterKennedy2N54:
    williamson_condition: bool = False


@dataclass(frozen=True)
class SymplecticPositionVerlet:
    """The reference's SymplecticPositionVerlet (2 kick! evaluations per step, density updated
    by rho_prev (2 - eps) / (2 + eps))."""


def CallbackSet(*callbacks) -> list:
    """CallbackSet(callbacks...) as the reference's examples build it: the callbacks in order,
    `nothing` entries (None here) dropped; `solve` takes the list."""
    return [c for c in callbacks if c is not None]


class InfoCallback:
    """InfoCallback(; interval=0) (src/callbacks/info.jl): a progress line every `interval` steps
    (interval 0: none) with the step count, the step size and the simulation time."""

    def __init__(self, *, interval: int = 0):
        if int(interval) < 0:
            raise _argument_error("`interval` must be non-negative")
        self.interval = int(interval) if int(interval) > 0 else None
        self.lines = []

    def report(self, steps: int, dt: float, t: float) -> None:
        line = f"#timesteps: {steps:10d} | dt: {dt:.4e} | sim. time: {t:.4e}"
        self.lines.append(line)
        print(line, flush=True)


class StepsizeCallback:
    """StepsizeCallback(; cfl) (src/callbacks/stepsize.jl:35-75): at initialisation the
    integrator's fixed step becomes calculate_dt of the semidiscretization, the minimum over its
    systems (semidiscretization.jl:510-520).  The WCSPH fluid's (fluid.jl:199-229) is
    min(0.125 h^2 / nu, 0.25 sqrt(h / |g|), cfl h / c) with nu = alpha h c / (2 ndims + 4) for
    the Monaghan viscosity (viscosity.jl:82-87); the wall's is Inf (wall_boundary/system.jl:
    291-293).  It depends on no state, so the step stays constant, as in the reference."""

    def __init__(self, *, cfl: float):
        self.cfl = float(cfl)

    def calculate_dt(self, semi) -> float:
        f = semi.fluid
        h = float(f.smoothing_length)
        c = float(f.state_equation.sound_speed)
        dt_viscosity = math.inf
        if isinstance(f.viscosity, ArtificialViscosityMonaghan):
            nu = f.viscosity.alpha * h * c / (2 * f.ndims + 4)
            if nu > 0.0:
                dt_viscosity = 0.125 * h ** 2 / nu
        g = math.sqrt(sum(float(a) ** 2 for a in (f.acceleration or ())))
        dt_acceleration = 0.25 * math.sqrt(h / g) if g > 0.0 else math.inf
        dt_sound_speed = self.cfl * h / c
        return min(dt_viscosity, dt_acceleration, dt_sound_speed)


class SortingCallback:
    """SortingCallback(; interval=-1, dt=0.0, initial_sort=true) (src/callbacks/sorting.jl:
    24-55): reorder the fluid particles by neighbour-search cell at the end of every `interval`
    steps, or at the first step after every `dt` of integration time, and (initial_sort) once
    before the first step.  `sort_masses` (not in the reference) also moves the fluid masses with
    their particles; the reference leaves them in place (a TODO there), which is the default."""

    def __init__(self, *, interval: int = -1, dt: float = 0.0, initial_sort: bool = True,
                 sort_masses: bool = False):
        if dt > 0 and interval > 0:
            raise _argument_error("setting both `interval` and `dt` is not supported")
        if dt <= 0 and interval <= 0:
            raise _argument_error("either `interval` or `dt` must be set to a positive value")
        self.interval = int(interval) if dt <= 0 else None
        self.dt = float(dt) if dt > 0 else None
        self.initial_sort = bool(initial_sort)
        self.sort_masses = bool(sort_masses)
        self.last_t = 0.0

    def sort(self, semi, v, u, perm=None):
        """Sorts (v, u) in place; returns the composed permutation (original index of every
        current particle) when `perm` (the previous one) is given."""
        import torch

        p = torch.empty(semi.n_fluid, dtype=torch.int32, device=v.device)
        semi._set_stream()
        semi._call("tp_sort_particles", v.data_ptr(), u.data_ptr(), int(self.sort_masses),
                   p.data_ptr())
        return p.long() if perm is None else perm[p.long()]


@dataclass
class ODESolution:
    v: object
    u: object
    t: float
    n_steps: int
    retcode: str = "Success"
    perm: object = None  # with a SortingCallback: original index of every particle


def fixed_step_schedule(t0: float, t1: float, dt: float) -> tuple[int, float | None]:
    """The steps OrdinaryDiffEq takes with a fixed `dt` from t0 to the tstop t1: dt = min(dt,
    t1 - t) (the last step shortened to land on t1), and a time within 100 ulp of t1 snapped to it
    (`fixed_t_for_floatingpoint_error!`), so that a span of a whole number of steps takes no extra
    step of rounding size.  Returns (full steps, length of the shortened last step or None)."""
    if not dt > 0.0:
        raise _argument_error("dt must be positive")
    t, n = float(t0), 0
    while t < t1:
        d = min(dt, t1 - t)
        tn = t + d
        if abs(tn - t1) < 100.0 * float(np.spacing(max(abs(t), abs(t1)))):
            tn = t1
        if d < dt:
            return n, d
        n += 1
        t = tn
    return n, None


def solve(ode: ODEProblem, alg: CarpenterKennedy2N54, *, dt: float, n_steps: int | None = None,
          save_everystep: bool = False, callback=None) -> ODESolution:
    """Fixed-step CarpenterKennedy2N54 or SymplecticPositionVerlet from tspan[0], advanced by the
    library's fused integrators; v/u of the result are new tensors.  Without `n_steps` the run
    ends on tspan[1] as OrdinaryDiffEq's does (fixed_step_schedule: the last step shortened);
    with it, exactly `n_steps` steps of `dt`.  `callback`: SortingCallback and/or
    SolutionSavingCallback and InfoCallback (one, a list or a CallbackSet), applied between
    integrator calls at their step / time intervals, and StepsizeCallback, whose step replaces
    `dt`."""
    if not isinstance(alg, (CarpenterKennedy2N54, SymplecticPositionVerlet)):
        raise _argument_error("only CarpenterKennedy2N54 and SymplecticPositionVerlet are "
                              "provided by the GB300 backend")
    semi = ode.p["semi"]
    from .vtk import SolutionSavingCallback

    cbs = callback if isinstance(callback, (list, tuple)) else \
        ([] if callback is None else [callback])
    for c in cbs:
        if not isinstance(c, (SortingCallback, SolutionSavingCallback, StepsizeCallback,
                              InfoCallback)):
            raise _argument_error("only SortingCallback, SolutionSavingCallback, "
                                  "StepsizeCallback and InfoCallback are supported as callbacks")
    for c in cbs:  # the step size callback overwrites `dt` before the first step
        if isinstance(c, StepsizeCallback):
            dt = c.calculate_dt(semi)
    cbs = [c for c in cbs if not isinstance(c, StepsizeCallback) and
           not (isinstance(c, InfoCallback) and c.interval is None)]
    t0, t1 = ode.tspan
    last = None
    if n_steps is None:
        n_steps, last = fixed_step_schedule(t0, t1, dt)
    v = ode.v0.clone()
    u = ode.u0.clone()
    semi._set_stream()
    entry = "tp_integrate_spv" if isinstance(alg, SymplecticPositionVerlet) else \
        "tp_integrate_ck2n54"

    def advance(t, k, step=dt):
        semi._call(entry, v.data_ptr(), u.data_ptr(), ctypes.c_double(t), ctypes.c_double(step),
                   ctypes.c_int64(k))

    def next_step(c, done):
        if c.interval is not None:
            return (done // c.interval + 1) * c.interval
        return max(done + 1, int(math.ceil((c.last_t + c.dt - t0) / dt - 1e-9)))

    perm = None
    for c in cbs:
        c.last_t = t0
        if isinstance(c, SortingCallback) and c.initial_sort:
            perm = c.sort(semi, v, u, perm)
        if isinstance(c, SolutionSavingCallback) and c.save_initial_solution:
            c.save(semi, v, u, t0)
    done = 0
    while done < n_steps:
        nxt = min([n_steps] + [next_step(c, done) for c in cbs])
        advance(t0 + done * dt, nxt - done)
        done = nxt
        t = t0 + done * dt
        for c in cbs:
            if next_step(c, done - 1) != done:
                continue
            if isinstance(c, SortingCallback):
                perm = c.sort(semi, v, u, perm)
                c.last_t = t
            elif isinstance(c, InfoCallback):
                c.report(done, dt, t)
            else:
                c.save(semi, v, u, t)
    t_end = t0 + n_steps * dt
    if last is not None:  # the shortened step that lands on tspan[1]
        advance(t_end, 1, last)
        n_steps += 1
        t_end = t1
    for c in cbs:
        if isinstance(c, SolutionSavingCallback) and c.save_final_solution and \
                c.last_t != t_end:
            c.save(semi, v, u, t_end)
    semi.sync()
    return ODESolution(v=v, u=u, t=t_end, n_steps=n_steps, perm=perm)


def dam_break_semidiscretization(tank, eos, smoothing_length: float, *, precision="float64",
                                 alpha=0.02, delta=0.1, gravity=9.81, wall_clip=True,
                                 beta=0.0, device: int = 0) -> Semidiscretization:
    """The dam-break system pair of examples/fluid/dam_break_2d.jl with a FullGridCellList over
    the tank's wall particles (examples/fluid/dam_break_2d_gpu.jl:30-33).  `beta`: the Monaghan
    beta (0 in the examples); `delta=None`: no density diffusion."""
    nd = tank.fluid.ndims
    kern = WendlandC2Kernel(nd)
    acc = (0.0, -gravity) if nd == 2 else (0.0, -gravity, 0.0)
    fluid = WeaklyCompressibleSPHSystem(
        tank.fluid, smoothing_kernel=kern, smoothing_length=smoothing_length,
        density_calculator=ContinuityDensity(), state_equation=eos, acceleration=acc,
        viscosity=ArtificialViscosityMonaghan(alpha=alpha, beta=beta),
        density_diffusion=None if delta is None else DensityDiffusionMolteniColagrossi(delta=delta))
    bm = BoundaryModelDummyParticles(
        tank.boundary.density, tank.boundary.mass, AdamiPressureExtrapolation(), kern,
        smoothing_length, state_equation=eos, clip_negative_pressure=wall_clip)
    wall = WallBoundarySystem(tank.boundary, bm)
    allc = np.concatenate([tank.boundary.coordinates, tank.fluid.coordinates], axis=0)
    cl = FullGridCellList(tuple(allc.min(axis=0)), tuple(allc.max(axis=0)))
    return Semidiscretization(fluid, wall, neighborhood_search=GridNeighborhoodSearch(nd, cl),
                              parallelization_backend=GB300Backend(precision, device))
