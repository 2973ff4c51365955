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


def rectangular_shape_coords(spacing: float, n_per_dim, min_coords, loop_order=None) -> np.ndarray:
    """rectangular_shape.jl:196-224 with loop_permutation (:168-194).

    Returns an `(n, ndims)` array.  `loop_order` is None, 'x', 'y' or 'z' as in the reference:
    linear iteration over `permutedims(CartesianIndices(n), perm)`, first permuted index fastest.
    """
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
    """InitialCondition: coordinates/velocity `(n, ndims)`, mass/density/pressure `(n,)`."""

    coordinates: np.ndarray
    velocity: np.ndarray
    mass: np.ndarray
    density: np.ndarray
    pressure: np.ndarray
    particle_spacing: float

    @property
    def ndims(self) -> int:
        return self.coordinates.shape[1]

    @property
    def n_particles(self) -> int:
        return self.coordinates.shape[0]


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
        coords = rectangular_shape_coords(dx, nfd, [0.0] * nd) + shift
        nf = coords.shape[0]
        pressure = np.zeros(nf)
        eos = self.state_equation
        density = None
        if self.acceleration is not None:
            acc = [float(a) for a in self.acceleration]
            if sum(abs(a) > EPS for a in acc) > 1:
                raise ValueError("hydrostatic pressure calculation is not supported with "
                                 "diagonal acceleration")
            ad = next((d for d in range(nd) if abs(acc[d]) > EPS), None)
            if ad is not None:
                dens = (lambda p: eos.inverse(p)) if eos is not None else (lambda p: rho0)
                factor = dx * abs(acc[ad])
                p1d = [0.0] * nfd[ad]
                p1d[0] = (0.5 * factor) * dens(0.0)
                for i in range(nfd[ad] - 1):
                    p1d[i + 1] = p1d[i] + factor * dens(p1d[i])
                if acc[ad] < 0:
                    p1d.reverse()
                k = np.arange(nf)
                strides = [1, nfd[0], nfd[0] * nfd[1]]
                idx_ad = (k // strides[ad]) % nfd[ad]
                pressure = np.asarray(p1d, dtype=np.float64)[idx_ad]
                if eos is not None:  # one inverse-EOS evaluation per hydrostatic level
                    d1d = np.array([eos.inverse(p) for p in p1d], dtype=np.float64)
                    density = d1d[idx_ad]
        if density is None:
            density = (np.full(nf, eos.inverse(0.0)) if eos is not None else np.full(nf, rho0))
        fvol = dx * dx if nd == 2 else (dx * dx) * dx
        self.fluid = InitialCondition(
            coordinates=coords,
            velocity=np.zeros_like(coords),
            mass=fvol * density,
            density=density,
            pressure=pressure,
            particle_spacing=dx,
        )


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
