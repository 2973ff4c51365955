"""Batched ensembles of independent 2D dam breaks on one GPU (the batching form).

Instances are drawn from a seed: fluid width U[0.5, 2] m, height U[0.25, 1] m, spacing dx from
{0.005, 0.01, 0.02}, each in the 5.366 x 4.0 m tank with 3 wall layers of the 2D benchmark.
Instances that share a spacing share one cell grid: they are placed side by side along x with
gaps wider than the kernel support, so they never interact, and one set of kernel launches
advances all of them (one library handle per spacing group).  The whole ensemble step is
recorded once into a CUDA graph by the library (tp_batch_capture, the groups as parallel
branches) and replayed; the pair-kernel block size and the neighbour-list skin of every group
are chosen by the library's autotuner (tp_batch_autotune) from timed trial steps.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

from .semidiscretization import (AdamiPressureExtrapolation, ArtificialViscosityMonaghan,
                                 BoundaryModelDummyParticles, ContinuityDensity,
                                 DensityDiffusionMolteniColagrossi, FullGridCellList,
                                 GB300Backend, GridNeighborhoodSearch, Semidiscretization,
                                 WallBoundarySystem, WeaklyCompressibleSPHSystem,
                                 WendlandC2Kernel, semidiscretize)
from . import _abi
from .setups import InitialCondition, dam_break

TANK = (5.366, 4.0)
LAYERS = 3
SPACINGS = (0.005, 0.01, 0.02)


@dataclass
class InstanceSpec:
    width: float
    height: float
    dx: float


def ensemble_specs(n: int = 512, seed: int = 0) -> list[InstanceSpec]:
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.5, 2.0, n)
    h = rng.uniform(0.25, 1.0, n)
    dx = rng.choice(np.array(SPACINGS), n)
    return [InstanceSpec(float(a), float(b), float(c)) for a, b, c in zip(w, h, dx)]


@dataclass
class Group:
    dx: float
    instances: list          # indices into the spec list
    shifts: list             # x shift of every instance
    fluid_ranges: list       # (start, stop) of every instance's fluid particles
    semi: Semidiscretization
    tanks: list
    ode: object = None
    v: object = None
    u: object = None
    tuned: dict = field(default_factory=dict)

    @property
    def n_particles(self) -> int:
        return self.semi.n_fluid + self.semi.n_wall


def _concat(ics: list[InitialCondition], shifts: list[float]) -> InitialCondition:
    coords = []
    for ic, s in zip(ics, shifts):
        c = ic.coordinates.copy()
        c[:, 0] += s
        coords.append(c)
    return InitialCondition(
        coordinates=np.ascontiguousarray(np.concatenate(coords)),
        velocity=np.concatenate([ic.velocity for ic in ics]),
        mass=np.concatenate([ic.mass for ic in ics]),
        density=np.concatenate([ic.density for ic in ics]),
        pressure=np.concatenate([ic.pressure for ic in ics]),
        particle_spacing=ics[0].particle_spacing)


def build_group(specs: list[InstanceSpec], members: list[int], precision: str = "float32",
                h_factor: float = 1.75, device: int = 0) -> Group:
    dx = specs[members[0]].dx
    h = h_factor * dx
    tanks = []
    for i in members:
        tank, eos = dam_break(2, dx, (specs[i].width, specs[i].height), TANK, n_layers=LAYERS)
        tanks.append(tank)
    # side by side with a gap of several kernel supports between neighbouring tanks
    pitch = math.ceil((TANK[0] + 2 * LAYERS * dx + 8 * h) / (2 * h)) * (2 * h)
    shifts = [k * pitch for k in range(len(members))]
    fluid = _concat([t.fluid for t in tanks], shifts)
    wall = _concat([t.boundary for t in tanks], shifts)
    ranges, start = [], 0
    for t in tanks:
        ranges.append((start, start + t.fluid.n_particles))
        start += t.fluid.n_particles
    kern = WendlandC2Kernel(2)
    fsys = WeaklyCompressibleSPHSystem(
        fluid, smoothing_kernel=kern, smoothing_length=h, density_calculator=ContinuityDensity(),
        state_equation=eos, acceleration=(0.0, -9.81),
        viscosity=ArtificialViscosityMonaghan(alpha=0.02),
        density_diffusion=DensityDiffusionMolteniColagrossi(delta=0.1))
    bm = BoundaryModelDummyParticles(wall.density, wall.mass, AdamiPressureExtrapolation(), kern,
                                     h, state_equation=eos, clip_negative_pressure=True)
    wsys = WallBoundarySystem(wall, bm)
    allc = np.concatenate([wall.coordinates, fluid.coordinates])
    cl = FullGridCellList(tuple(allc.min(0)), tuple(allc.max(0)))
    semi = Semidiscretization(fsys, wsys, neighborhood_search=GridNeighborhoodSearch(2, cl),
                              parallelization_backend=GB300Backend(precision, device))
    return Group(dx=dx, instances=list(members), shifts=shifts, fluid_ranges=ranges, semi=semi,
                 tanks=tanks)


def build_ensemble(specs: list[InstanceSpec], precision: str = "float32",
                   device: int = 0) -> list[Group]:
    groups = []
    for dx in SPACINGS:
        members = [i for i, s in enumerate(specs) if s.dx == dx]
        if members:
            groups.append(build_group(specs, members, precision, device=device))
    return groups


def time_step(dx: float) -> float:
    """Fixed step of an instance: 1e-4 s at dx = 0.02 (the 2D dam break's step), scaled with dx
    (acoustic CFL 0.25 h / c at h = 1.75 dx, c = 20 sqrt(9.81) m/s gives 1.4e-4 s there)."""
    return 5e-3 * dx


def _integrate(g: Group, steps: int, dt: float | None = None):
    dt = time_step(g.dx) if dt is None else dt
    g.semi._call("tp_integrate_ck2n54", g.v.data_ptr(), g.u.data_ptr(), ctypes.c_double(0.0),
                 ctypes.c_double(dt), ctypes.c_int64(steps))


def _bind(g: Group, stream) -> None:
    g.semi._ensure_handle()
    st = g.semi._lib.tp_set_stream(g.semi._handle, ctypes.c_void_p(stream.cuda_stream))
    _abi.check(g.semi._lib, g.semi._handle, st)


def prepare(g: Group, stream, growth: float = 1.5) -> None:
    """Initial state, fixed list capacities and the stream of a group (before any capture)."""
    if g.ode is None:
        g.ode = semidiscretize(g.semi, (0.0, 1.0))
    g.v, g.u = g.ode.v0.clone(), g.ode.u0.clone()
    _bind(g, stream)
    g.semi._call("tp_prepare_lists", g.u.data_ptr(), ctypes.c_double(growth))


class Batch:
    """The native batch of the C ABI (tp_batch_*): one member per spacing group, its device
    state integrated in place by every graph launch."""

    def __init__(self, groups: list[Group]):
        self.groups = groups
        for g in groups:
            if g.ode is None:
                g.ode = semidiscretize(g.semi, (0.0, 1.0))
            if g.v is None:
                g.v, g.u = g.ode.v0.clone(), g.ode.u0.clone()
        self.lib = groups[0].semi._lib
        hs = (ctypes.c_void_p * len(groups))(*[g.semi._handle.value for g in groups])
        b = ctypes.c_void_p()
        st = self.lib.tp_batch_create(hs, len(groups), ctypes.byref(b))
        if st != 0:
            raise _abi.TpError(st, "tp_batch_create failed")
        self._b = b
        for k, g in enumerate(groups):
            self._check(self.lib.tp_batch_set_state(self._b, k, g.v.data_ptr(), g.u.data_ptr(),
                                                    ctypes.c_double(time_step(g.dx))))

    def _check(self, st):
        if st != 0:
            raise _abi.TpError(st, (self.lib.tp_batch_last_error(self._b) or b"").decode())

    def autotune(self, trial_steps: int = 3) -> dict:
        n = len(self.groups)
        blk = (ctypes.c_int32 * n)()
        skin = (ctypes.c_double * n)()
        mode = (ctypes.c_int32 * n)()
        ms = (ctypes.c_double * n)()
        self._check(self.lib.tp_batch_autotune(self._b, trial_steps, blk, skin, mode, ms))
        out = {}
        for k, g in enumerate(self.groups):
            g.tuned = {"pair_mode": "tiled" if mode[k] == _abi.TP_PAIR_TILED else "lists",
                       "pair_block": int(blk[k]), "skin": float(skin[k]),
                       "ms_per_step": float(ms[k])}
            out[g.dx] = g.tuned
        return out

    def set_mode(self, persistent: bool) -> None:
        """Graph layout of the next capture: the groups as parallel branches (default), or one
        persistent pair launch per stage for all groups (FP32 groups on neighbour lists)."""
        self._check(self.lib.tp_batch_set_mode(
            self._b, _abi.TP_BATCH_PERSISTENT if persistent else _abi.TP_BATCH_BRANCHES))

    def capture(self, steps: int, growth: float = 1.5) -> None:
        self._check(self.lib.tp_batch_capture(self._b, ctypes.c_int64(steps),
                                              ctypes.c_double(growth)))

    def launch(self, stream=None) -> None:
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        self._check(self.lib.tp_batch_launch(self._b, ctypes.c_void_p(s.cuda_stream)))

    def sync(self) -> None:
        self._check(self.lib.tp_batch_sync(self._b))

    def close(self) -> None:
        if self._b is not None:
            self.lib.tp_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(groups: list[Group], trial_steps: int = 3) -> dict:
    """Picks (pair pass, pair_block, skin) per group with the native autotuner (trial steps on
    scratch copies of the state); leaves each group's handle set to its choice; returns
    {dx: choice}."""
    b = Batch(groups)
    try:
        return b.autotune(trial_steps)
    finally:
        b.close()


class EnsembleGraph:
    """K CarpenterKennedy2N54 steps of every group as one CUDA graph (tp_batch_capture): one
    branch per spacing group (the groups run concurrently), each branch the group's fused
    integrator (neighbour-list upkeep, Adami, pair kernel with the stage update).  With
    `persistent`, the groups' pair passes of a stage are one persistent launch over all groups
    (a work queue of 256-slot tiles) between the branches' neighbour-list upkeep and their
    next stage."""

    def __init__(self, groups: list[Group], steps_per_replay: int, growth: float = 1.5,
                 persistent: bool = False):
        self.groups = groups
        self.k = steps_per_replay
        self.persistent = persistent
        self.batch = Batch(groups)
        if persistent:
            self.batch.set_mode(True)
        self.batch.capture(steps_per_replay, growth)

    @property
    def n_particles(self) -> int:
        return sum(g.n_particles for g in self.groups)

    @property
    def n_fluid(self) -> int:
        return sum(g.semi.n_fluid for g in self.groups)

    def reset(self):
        for g in self.groups:
            g.v.copy_(g.ode.v0)
            g.u.copy_(g.ode.u0)

    def replay(self):
        """Launches the graph on the current torch stream (asynchronous)."""
        self.batch.launch()

    def check(self):
        """Waits for the graph and raises the first error any group reported."""
        self.batch.sync()

    def close(self):
        self.batch.close()


def instance_state(g: Group, j: int):
    """(x, v, rho) of the j-th instance of a group, shifted back to its own tank."""
    nd = 2
    a, b = g.fluid_ranges[j]
    u = g.u.view(-1, nd)[a:b].cpu().numpy().copy()
    u[:, 0] -= g.shifts[j]
    v = g.v.view(-1, nd + 1)[a:b].cpu().numpy()
    return u, v[:, :nd].copy(), v[:, nd].copy()


def single_instance(spec: InstanceSpec, precision: str = "float32", device: int = 0) -> Group:
    """The same instance as its own one-member group (the single-instance path)."""
    return build_group([spec], [0], precision, device=device)
