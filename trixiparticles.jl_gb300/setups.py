"""Dam-break setup: the reference's RectangularTank / RectangularShape, restated with numpy.

Particle arrays use the reference's memory layout: a Julia `(ndims, n)` column-major matrix is
a C-contiguous numpy array of shape `(n, ndims)` (particle-major), the layout the C ABI takes.
Arithmetic follows the reference expressions in order (IEEE double, no fused operations), so the
arrays are identical to the reference's on the same inputs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

EPS = float(np.finfo(np.float64).eps)


def _round_ties_even(x: float) -> int:
    """Julia's round(Int, x) (RoundNearest, ties to even)."""
    return int(np.rint(x))


def round_n_particles(size: float, spacing: float) -> tuple[int, float]:
    """rectangular_tank.jl:406-416."""
    n = _round_ties_even(size / spacing)
    return n, float(n) * spacing


def _isapprox(a: float, b: float) -> bool:
    return abs(a - b) <= math.sqrt(EPS) * max(abs(a), abs(b))


def _shape_indices(n_per_dim, loop_order=None) -> list:
    """The 0-based cartesian index of every particle along each axis, in the order of
    `permutedims(CartesianIndices(n), loop_permutation(loop_order))` (rectangular_shape.jl:
    168-224): first permuted index fastest."""
    nd = len(n_per_dim)
    if nd == 2:
        perm = (1, 0) if loop_order == "x" else (0, 1)
    else:
        perm = {"y": (1, 0, 2), "x": (2, 1, 0)}.get(loop_order, (0, 1, 2))
    sizes = [int(n_per_dim[p]) for p in perm]
    rem = np.arange(int(np.prod(sizes)))
    idx = [None] * nd
    for k in range(nd):
        idx[perm[k]] = rem % sizes[k]
        rem = rem // sizes[k]
    return idx


def rectangular_shape_coords(spacing: float, n_per_dim, min_coords, loop_order=None) -> np.ndarray:
    """rectangular_shape.jl:196-224 with loop_permutation (:168-194).

    Returns an `(n, ndims)` array.  `loop_order` is None, 'x', 'y' or 'z' as in the reference:
    linear iteration over `permutedims(CartesianIndices(n), perm)`, first permuted index fastest.
    """
    nd = len(n_per_dim)
    idx = _shape_indices(n_per_dim, loop_order)
    out = np.empty((len(idx[0]), nd), dtype=np.float64)
    for d in range(nd):
        out[:, d] = float(min_coords[d]) + spacing * ((idx[d] + 1).astype(np.float64) - 0.5)
    return out


@dataclass
class StateEquationCole:
    """StateEquationCole (state_equations.jl:100-139)."""

    sound_speed: float
    reference_density: float
    exponent: float
    background_pressure: float = 0.0
    clip_negative_pressure: bool = False

    @property
    def B(self) -> float:
        return (self.reference_density * (self.sound_speed * self.sound_speed)) / self.exponent

    def __call__(self, density: float) -> float:
        p = self.B * (math.pow(density / self.reference_density, self.exponent) - 1.0)
        p = p + self.background_pressure
        if self.clip_negative_pressure:
            p = p if (p != p or p > 0.0) else 0.0
        return p

    def inverse(self, pressure: float) -> float:
        tmp = (pressure - self.background_pressure) / self.B + 1.0
        return self.reference_density * math.pow(tmp, 1.0 / self.exponent)


@dataclass
class InitialCondition:
    """InitialCondition (initial_condition.jl:114-215): coordinates/velocity `(n, ndims)`,
    mass/density/pressure `(n,)`.  As in the reference, velocity, mass, density and pressure may
    also be given as constants or as functions of a particle's coordinates; without a mass it is
    density * particle_spacing^ndims (particle_spacing required then); the reference's argument
    errors are raised as ValueError("ArgumentError: ...")."""

    coordinates: np.ndarray
    velocity: object = None
    mass: object = None
    density: object = None
    pressure: object = 0.0
    particle_spacing: float = -1.0

    def __post_init__(self):
        x = np.asarray(self.coordinates, dtype=np.float64)
        if x.ndim != 2:
            raise ValueError("ArgumentError: `coordinates` must be an (n, ndims) array")
        self.coordinates = x
        n, nd = x.shape
        if n == 0:
            self.velocity = np.zeros((0, nd))
            self.mass = np.zeros(0)
            self.density = np.zeros(0)
            self.pressure = np.zeros(0)
            return

        def per_particle(value, name):
            if callable(value):
                return np.array([value(r.copy()) for r in x], dtype=np.float64)
            a = np.asarray(value, dtype=np.float64)
            if a.ndim == 0:
                return np.full(n, float(a))
            if a.shape != (n,):
                raise ValueError(f"ArgumentError: Expected: length({name}) == size(coordinates, "
                                 f"2)\nGot: size(coordinates, 2) = {n}, length({name}) = "
                                 f"{a.size}")
            return a

        v = self.velocity
        if v is None:
            v = np.zeros((n, nd))
        elif callable(v) or np.ndim(v) == 1:
            f = v if callable(v) else (lambda _r, c=np.asarray(v, dtype=np.float64): c)
            if np.size(f(x[0].copy())) != nd:
                raise ValueError(f"ArgumentError: `velocity` must be {nd}-dimensional for "
                                 f"{nd}-dimensional `coordinates`")
            v = np.array([np.asarray(f(r.copy()), dtype=np.float64) for r in x])
        v = np.asarray(v, dtype=np.float64)
        if v.shape != x.shape:
            raise ValueError("ArgumentError: `coordinates` and `velocities` must be of the "
                             "same size")
        self.velocity = v
        if self.density is None:
            raise ValueError("ArgumentError: `density` must be given")
        rho = per_particle(self.density, "density")
        if np.any(rho < EPS):
            raise ValueError("ArgumentError: density must be positive and larger than `eps()`")
        self.density = rho
        self.pressure = per_particle(self.pressure, "pressure")
        if self.mass is None:
            if self.particle_spacing < 0:
                raise ValueError("ArgumentError: `mass` must be specified when not using "
                                 "`particle_spacing`")
            dx = float(self.particle_spacing)
            vol = dx * dx if nd == 2 else ((dx * dx) * dx if nd == 3 else dx)
            self.mass = vol * rho
        else:
            self.mass = per_particle(self.mass, "mass")

    @property
    def ndims(self) -> int:
        return self.coordinates.shape[1]

    @property
    def n_particles(self) -> int:
        return self.coordinates.shape[0]


_LOOP_ORDERS = {2: {None: None, "y_first": None, "x_first": "x"},
                3: {None: None, "z_first": None, "y_first": "y", "x_first": "x"}}


def hydrostatic_pressure(spacing: float, acceleration, density_fun, n_per_dim,
                         loop_order=None) -> np.ndarray:
    """initialize_pressure! (rectangular_shape.jl:226-267): explicit Euler from the surface,
    half a step above the first particle, along the one axis the acceleration acts on; the
    levels reversed when it points in the negative direction, then read per particle through
    the shape's index order."""
    acc = [float(a) for a in acceleration]
    if sum(abs(a) > EPS for a in acc) > 1:
        raise ValueError("ArgumentError: hydrostatic pressure calculation is not supported "
                         "with diagonal acceleration")
    ad = next(d for d in range(len(acc)) if abs(acc[d]) > EPS)
    factor = spacing * abs(acc[ad])
    p1d = [0.0] * int(n_per_dim[ad])
    p1d[0] = (0.5 * factor) * density_fun(0.0)
    for i in range(len(p1d) - 1):
        p1d[i + 1] = p1d[i] + factor * density_fun(p1d[i])
    if acc[ad] < 0:
        p1d.reverse()
    return np.asarray(p1d, dtype=np.float64)[_shape_indices(n_per_dim, loop_order)[ad]]


def RectangularShape(particle_spacing, n_particles_per_dimension, min_coordinates, *,
                     velocity=None, mass=None, density=None, pressure=0.0, acceleration=None,
                     state_equation=None, place_on_shell=False,
                     loop_order=None) -> InitialCondition:
    """RectangularShape (rectangular_shape.jl:79-151): particles at min_coordinates +
    (i - 1/2) dx (with place_on_shell the first ones on min_coordinates: the corner moved back by
    dx / 2 first, :205-209), in `loop_order` (None, "x_first", "y_first", "z_first"); with `acceleration`
    a hydrostatic pressure column (hydrostatic_pressure) and, with a state equation, the density
    of every particle from its inverse; mass density dx^d unless given.  Errors as the
    reference's (ArgumentError)."""
    dx = float(particle_spacing)
    if not dx >= EPS:
        raise ValueError(f"ArgumentError: `particle_spacing` needs to be positive and larger "
                         f"than {EPS}")
    n = tuple(int(k) for k in n_particles_per_dimension)
    nd = len(n)
    if len(min_coordinates) != nd:
        raise ValueError(f"ArgumentError: `min_coordinates` must be of length {nd} for a "
                         f"{nd}D problem")
    if loop_order not in _LOOP_ORDERS.get(nd, {None: None}):
        raise ValueError(f"ArgumentError: {loop_order} is not a valid loop order")
    order = _LOOP_ORDERS.get(nd, {None: None})[loop_order]
    if density is not None and np.any(np.asarray(density) < EPS):
        raise ValueError(f"ArgumentError: `density` needs to be positive and larger than {EPS}")
    corner = [float(c) for c in min_coordinates]
    if place_on_shell:
        corner = [c - 0.5 * dx for c in corner]
    coords = rectangular_shape_coords(dx, n, corner, order)
    n_p = coords.shape[0]
    if acceleration is not None:
        if pressure != 0.0:
            raise ValueError("ArgumentError: `pressure` cannot be used together with "
                             "`acceleration` and `state_equation` (hydrostatic pressure "
                             "gradient)")
        if state_equation is None:
            if density is None:
                raise ValueError("ArgumentError: `density` must be specified when not using "
                                 "`acceleration` and `state_equation`")
            rho = float(density)
            p = hydrostatic_pressure(dx, acceleration, lambda _p: rho, n, order)
        else:
            if density is not None:
                raise ValueError("ArgumentError: `density` cannot be used together with "
                                 "`acceleration` and `state_equation` (hydrostatic pressure "
                                 "gradient)")
            p = hydrostatic_pressure(dx, acceleration, state_equation.inverse, n, order)
            density = np.array([state_equation.inverse(x) for x in p], dtype=np.float64)
    else:
        if state_equation is not None:
            raise ValueError("ArgumentError: `state_equation` must be used together with "
                             "`acceleration`")
        p = np.full(n_p, float(pressure))
    if density is None:
        raise ValueError("ArgumentError: `density` must be specified when not using "
                         "`acceleration` and `state_equation` (hydrostatic pressure gradient)")
    rho = np.broadcast_to(np.asarray(density, dtype=np.float64), (n_p,)).copy()
    vol = dx * dx if nd == 2 else ((dx * dx) * dx if nd == 3 else dx)
    m = rho * vol if mass is None else \
        np.broadcast_to(np.asarray(mass, dtype=np.float64), (n_p,)).copy()
    vel = np.zeros_like(coords) if velocity is None else \
        np.broadcast_to(np.asarray(velocity, dtype=np.float64), coords.shape).copy()
    return InitialCondition(coordinates=coords, velocity=vel, mass=m, density=rho, pressure=p,
                            particle_spacing=dx)


@dataclass
class RectangularTank:
    """RectangularTank (rectangular_tank.jl:99-200): fluid block at the tank's min corner with
    `n_layers` of wall particles of spacing particle_spacing / spacing_ratio on the faces
    (-x, +x, -y, +y[, -z, +z]), hydrostatic fluid density from the inverse state equation, fluid
    mass rho dx^d, wall density boundary_density (default fluid_density) and wall mass
    boundary_density (dx / spacing_ratio)^d; the whole tank moved to min_coordinates."""

    particle_spacing: float
    fluid_size: tuple
    tank_size: tuple
    fluid_density: float
    n_layers: int = 1
    acceleration: tuple | None = None
    state_equation: StateEquationCole | None = None
    faces: tuple | None = None
    spacing_ratio: float = 1.0  # particle_spacing / wall particle spacing
    min_coordinates: tuple | None = None  # the tank's corner in the negative directions
    boundary_density: float | None = None  # default: fluid_density
    fluid: InitialCondition = field(init=False)
    boundary: InitialCondition = field(init=False)
    n_particles_per_dimension: tuple = field(init=False)
    tank_size_rounded: tuple = field(init=False)

    def __post_init__(self):
        dx = float(self.particle_spacing)
        nd = len(self.fluid_size)
        if len(self.tank_size) != nd:
            raise ValueError(f"`tank_size` must be of length {nd} for a {nd}D problem")
        if not dx > EPS:
            raise ValueError("`particle_spacing` needs to be positive and larger than eps")
        faces = self.faces if self.faces is not None else (True,) * (2 * nd)
        nfd, fsz = [], []
        for d in range(nd):
            n, s = round_n_particles(float(self.fluid_size[d]), dx)
            nfd.append(n)
            fsz.append(s)
        tsz = [float(t) for t in self.tank_size]
        for d in range(nd):
            if _isapprox(float(self.fluid_size[d]), float(self.tank_size[d])):
                tsz[d] = fsz[d]
        if not float(self.spacing_ratio) > 0.0:
            raise ValueError("`spacing_ratio` must be positive")
        bdx = dx / float(self.spacing_ratio)
        nbd = []
        for d in range(nd):
            n, s = round_n_particles(tsz[d], bdx)
            nbd.append(n)
            tsz[d] = s
        for d in range(nd):  # check_tank_overlap
            if tsz[d] < fsz[d] - 1e-5 * dx:
                nfd[d] -= 1
                fsz[d] = nfd[d] * dx
        self.n_particles_per_dimension = tuple(nfd)
        self.tank_size_rounded = tuple(tsz)
        wall = _initialize_boundaries(bdx, tsz, nbd, self.n_layers, faces)
        bvol = bdx * bdx if nd == 2 else (bdx * bdx) * bdx
        nw = wall.shape[0]
        rho0 = float(self.fluid_density)
        rho_w = rho0 if self.boundary_density is None else float(self.boundary_density)
        shift = np.zeros(nd) if self.min_coordinates is None else \
            np.asarray(self.min_coordinates, dtype=np.float64)
        if shift.shape != (nd,):
            raise ValueError(f"`min_coordinates` must be of length {nd} for a {nd}D problem")
        wall = wall + shift  # the tank's corner moved to min_coordinates
        self.boundary = InitialCondition(
            coordinates=wall,
            velocity=np.zeros_like(wall),
            mass=np.full(nw, rho_w * bvol),
            density=np.full(nw, rho_w),
            pressure=np.zeros(nw),
            particle_spacing=bdx,
        )
        # the fluid: a RectangularShape at the tank's corner (rectangular_tank.jl:171-190), with
        # the hydrostatic column when an acceleration acts (a zero acceleration gives the
        # density of zero pressure everywhere)
        acc = self.acceleration
        eos = self.state_equation
        if acc is not None and any(abs(float(a)) > EPS for a in acc):
            fluid = RectangularShape(dx, nfd, [0.0] * nd, acceleration=acc, state_equation=eos,
                                     density=None if eos is not None else rho0)
        else:
            fluid = RectangularShape(dx, nfd, [0.0] * nd,
                                     density=eos.inverse(0.0) if eos is not None else rho0)
        fluid.coordinates = fluid.coordinates + shift
        self.fluid = fluid


def _initialize_boundaries(bdx, tsz, nbd, n_layers, faces) -> np.ndarray:
    """initialize_boundaries (rectangular_tank.jl:530-690 in 2D, :692-1130 in 3D)."""
    nd = len(tsz)
    lo = -float(n_layers) * bdx
    L = n_layers
    parts = []

    def S(n, m, loop=None):
        parts.append(rectangular_shape_coords(bdx, n, m, loop))

    if nd == 2:
        nx, ny = nbd
        if faces[0]:
            S((L, ny), (lo, 0.0), "x")
        if faces[1]:
            S((L, ny), (tsz[0], 0.0), "x")
        if faces[2]:
            S((nx, L), (0.0, lo), "y")
        if faces[3]:
            S((nx, L), (0.0, tsz[1]), "y")
        if faces[0] and faces[2]:
            S((L, L), (lo, lo))
        if faces[0] and faces[3]:
            S((L, L), (lo, tsz[1]))
        if faces[1] and faces[2]:
            S((L, L), (tsz[0], lo))
        if faces[1] and faces[3]:
            S((L, L), (tsz[0], tsz[1]))
    else:
        nx, ny, nz = nbd
        left, right, bottom, top, front, back = (bool(f) for f in faces)
        if left:
            S((L, ny, nz), (lo, 0.0, 0.0), "x")
        if right:
            S((L, ny, nz), (tsz[0], 0.0, 0.0), "x")
        if bottom:
            S((nx, L, nz), (0.0, lo, 0.0), "y")
        if top:
            S((nx, L, nz), (0.0, tsz[1], 0.0), "y")
        if front:
            S((nx, ny, L), (0.0, 0.0, lo), "z")
        if back:
            S((nx, ny, L), (0.0, 0.0, tsz[2]), "z")
        if left and bottom:
            S((L, L, nz), (lo, lo, 0.0))
        if left and top:
            S((L, L, nz), (lo, tsz[1], 0.0))
        if right and bottom:
            S((L, L, nz), (tsz[0], lo, 0.0))
        if right and top:
            S((L, L, nz), (tsz[0], tsz[1], 0.0))
        if front and bottom:
            S((nx, L, L), (0.0, lo, lo))
        if front and top:
            S((nx, L, L), (0.0, tsz[1], lo))
        if back and bottom:
            S((nx, L, L), (0.0, lo, tsz[2]))
        if back and top:
            S((nx, L, L), (0.0, tsz[1], tsz[2]))
        if left and front:
            S((L, ny, L), (lo, 0.0, lo))
        if left and back:
            S((L, ny, L), (lo, 0.0, tsz[2]))
        if right and front:
            S((L, ny, L), (tsz[0], 0.0, lo))
        if right and back:
            S((L, ny, L), (tsz[0], 0.0, tsz[2]))
        for cx, cy, cz in ((lo, lo, lo), (lo, tsz[1], lo), (lo, lo, tsz[2]), (lo, tsz[1], tsz[2]),
                           (tsz[0], lo, lo), (tsz[0], tsz[1], lo), (tsz[0], lo, tsz[2]),
                           (tsz[0], tsz[1], tsz[2])):
            fx = left if cx == lo else right
            fy = bottom if cy == lo else top
            fz = front if cz == lo else back
            if fx and fy and fz:
                S((L, L, L), (cx, cy, cz))
    if not parts:
        return np.zeros((0, nd))
    return np.ascontiguousarray(np.concatenate(parts, axis=0))


def dam_break(ndims: int, particle_spacing: float, fluid_size, tank_size, n_layers: int = 3,
              gravity: float = 9.81, sound_speed: float | None = None, exponent: float = 7.0,
              reference_density: float = 1000.0) -> tuple[RectangularTank, StateEquationCole]:
    """The dam-break setups of the benchmark configurations: gravity along -y, Cole EOS with
    c = 20 sqrt(g * 1.0) unless given, hydrostatic initial density, zero velocity."""
    c = sound_speed if sound_speed is not None else 20.0 * math.sqrt(gravity * 1.0)
    eos = StateEquationCole(sound_speed=c, reference_density=reference_density, exponent=exponent)
    acc = (0.0, -gravity) if ndims == 2 else (0.0, -gravity, 0.0)
    tank = RectangularTank(particle_spacing, tuple(fluid_size), tuple(tank_size),
                           reference_density, n_layers=n_layers, acceleration=acc,
                           state_equation=eos)
    return tank, eos
