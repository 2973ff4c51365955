"""Shared setups of the tests: dam-break cases and the 2D validation run."""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def dam_break_case(pkg, ndims, dx, fluid, tank, layers=3, precision="float64", h_factor=1.75,
                   jitter=0.0, seed=0, alpha=0.02, delta=0.1, beta=0.0):
    """A dam-break Semidiscretization (not yet on the device) plus its tank."""
    tank_, eos = pkg.dam_break(ndims, dx, fluid, tank, n_layers=layers)
    if jitter:
        rng = np.random.default_rng(seed)
        tank_.fluid.coordinates += rng.uniform(-jitter * dx, jitter * dx,
                                               tank_.fluid.coordinates.shape)
    semi = pkg.dam_break_semidiscretization(tank_, eos, h_factor * dx, precision=precision,
                                            alpha=alpha, delta=delta, beta=beta)
    return semi, tank_


def initial_state(tank):
    nd = tank.fluid.ndims
    v = np.zeros((tank.fluid.n_particles, nd + 1))
    v[:, nd] = tank.fluid.density
    return v, tank.fluid.coordinates.copy()


def oracle_model(orc, semi, tank):
    return orc.Model(semi.config, tank.boundary.coordinates, tank.boundary.mass, tank.fluid.mass)


def load_validation():
    return json.loads((GOLDEN / "validation_wcsph_40.json").read_text())


def validation_case(pkg, precision="float64"):
    """validation/dam_break_2d setup at 40 particles per H (setup_marrone_2011.jl)."""
    g = load_validation()
    P = g["params"]
    H, dx, grav = P["H"], P["particle_spacing"], 9.81
    tank_x = math.floor(5.366 * H / dx) * dx
    eos = pkg.StateEquationCole(sound_speed=P["sound_speed"], reference_density=1000.0,
                                exponent=P["exponent"])
    tank = pkg.RectangularTank(dx, (P["W"], H), (tank_x, 4.0), 1000.0, n_layers=P["n_layers"],
                               acceleration=(0.0, -grav), state_equation=eos)
    semi = pkg.dam_break_semidiscretization(tank, eos, P["smoothing_length"], precision=precision,
                                            alpha=P["alpha"], delta=P["delta"])
    return semi, tank, g


def validation_schedule(g, n_samples):
    """Step sizes of the reference run: dt_max steps, shortened to land on every save time."""
    save = 0.01 / math.sqrt(9.81 / g["params"]["H"])
    dtmax = g["params"]["dt_max"]
    t = 0.0
    sched = []
    for k in range(1, n_samples):
        tstop = k * save
        steps = []
        while t < tstop - 1e-12:
            dt = min(dtmax, tstop - t)
            steps.append(dt)
            t = t + dt
            if abs(t - tstop) < 1e-12:
                t = tstop
        sched.append(steps)
    return sched


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def adami_tank_case(pkg, density, gravity, precision="float64", n_layers=2, wall_clip=True):
    """The static tank of the reference's Adami pressure-extrapolation tests
    (test/schemes/boundary/dummy_particles/dummy_particles.jl:308-333): a 10 x 10 fluid block at
    dx = 0.1 filling the tank, `n_layers` of wall particles on the bottom and sides (no lid),
    Cole EOS with c = 10, rho0 = 257, exponent 7, smoothing length 1.5 dx; `density` is the fluid
    density (hydrostatic from the EOS when `gravity` is set)."""
    dx = 0.1
    eos = pkg.StateEquationCole(sound_speed=10.0, reference_density=257.0, exponent=7.0)
    acc = (0.0, -gravity) if gravity else None
    tank = pkg.RectangularTank(dx, (1.0, 1.0), (1.0, 1.0), density, n_layers=n_layers,
                               acceleration=acc, state_equation=eos if gravity else None,
                               faces=(True, True, True, False))
    semi = pkg.dam_break_semidiscretization(tank, eos, 1.5 * dx, precision=precision,
                                            gravity=gravity, wall_clip=wall_clip)
    return semi, tank, eos


def hydrostatic_fields(pkg, tank, eos, p_f, p_w, n_layers=2, n=10, dx=0.1):
    """Pressure of the tank's fluid and walls on one integer grid, and that of a fluid-only tank
    covering the same area (test/schemes/boundary/dummy_particles/dummy_particles.jl:646-694)."""
    got = np.zeros((n + 2 * n_layers, n + n_layers))
    for coords, p in ((tank.boundary.coordinates, p_w), (tank.fluid.coordinates, p_f)):
        idx = np.rint(coords / dx + n_layers + 0.5).astype(int) - 1
        got[idx[:, 0], idx[:, 1]] = p
    ref_tank = pkg.RectangularTank(dx, (dx * (n + 2 * n_layers), dx * (n + n_layers)),
                                   (dx * (n + 2 * n_layers), dx * (n + n_layers)), 257.0,
                                   n_layers=0, acceleration=(0.0, -9.81), state_equation=eos,
                                   faces=(True, True, True, False))
    ref = np.zeros_like(got)
    idx = np.rint(ref_tank.fluid.coordinates / dx + 0.5).astype(int) - 1
    ref[idx[:, 0], idx[:, 1]] = ref_tank.fluid.pressure
    return got, ref


def random_fluid_case(pkg, nd, seed, n=6, viscosity=True, diffusion=True, precision="float64"):
    """Fluid-only semidiscretization of n^nd particles on a lattice of spacing 0.1 jittered by
    +-0.3 dx, densities 1000 (1 +- 1 %), random velocities, no walls and no gravity: the
    setting of the reference's conservation tests (test/schemes/fluid/rhs.jl:115-264), with the
    path's WendlandC2 kernel at h = 1.2 dx.  Returns (semi, x, v, m)."""
    rng = np.random.default_rng(seed)
    dx = 0.1
    g = np.stack(np.meshgrid(*[np.arange(n)] * nd, indexing="ij"), -1).reshape(-1, nd)
    x = (g + 0.5) * dx + rng.uniform(-0.3 * dx, 0.3 * dx, g.shape)
    rho = 1000.0 * (1 + rng.uniform(-0.01, 0.01, len(x)))
    m = dx ** nd * rho
    v = np.zeros((len(x), nd + 1))
    v[:, :nd] = rng.normal(0, 0.3, (len(x), nd))
    v[:, nd] = rho
    eos = pkg.StateEquationCole(sound_speed=20.0, reference_density=1000.0, exponent=7.0)
    ic = pkg.InitialCondition(x, v[:, :nd], m, rho, np.zeros(len(x)), dx)
    wic = pkg.InitialCondition(np.zeros((0, nd)), np.zeros((0, nd)), np.zeros(0), np.zeros(0),
                               np.zeros(0), dx)
    k = pkg.WendlandC2Kernel(nd)
    fluid = pkg.WeaklyCompressibleSPHSystem(
        ic, smoothing_kernel=k, smoothing_length=1.2 * dx,
        density_calculator=pkg.ContinuityDensity(), state_equation=eos,
        acceleration=(0.0,) * nd,
        viscosity=pkg.ArtificialViscosityMonaghan(alpha=0.02) if viscosity else None,
        density_diffusion=pkg.DensityDiffusionMolteniColagrossi(delta=0.1) if diffusion else None)
    wall = pkg.WallBoundarySystem(wic, pkg.BoundaryModelDummyParticles(
        np.zeros(0), np.zeros(0), pkg.AdamiPressureExtrapolation(), k, 1.2 * dx,
        state_equation=eos))
    cl = pkg.FullGridCellList(tuple(x.min(0) - dx), tuple(x.max(0) + dx))
    semi = pkg.Semidiscretization(fluid, wall,
                                  neighborhood_search=pkg.GridNeighborhoodSearch(nd, cl),
                                  parallelization_backend=pkg.GB300Backend(precision=precision))
    return semi, x, v, m


def conservation_residuals(x, v, m, dv, p):
    """Rates of the conserved quantities of the pair terms and their scales (sums of the
    magnitudes of the summands): linear momentum sum_a m_a dv_a, angular momentum
    sum_a m_a x_a x dv_a, total energy sum_a m_a (v_a . dv_a + p_a / rho_a^2 drho_a)
    (test/schemes/fluid/rhs.jl:192-260)."""
    nd = x.shape[1]
    a, drho = dv[:, :nd], dv[:, nd]
    rho = v[:, nd]
    mom = (m[:, None] * a).sum(0)
    mom_scale = (m[:, None] * np.abs(a)).sum()
    x3 = np.zeros((len(x), 3))
    a3 = np.zeros((len(x), 3))
    x3[:, :nd], a3[:, :nd] = x, a
    ang = (m[:, None] * np.cross(x3, a3)).sum(0)
    ang_scale = (m[:, None] * np.linalg.norm(x3, axis=1)[:, None] * np.abs(a3)).sum()
    work = m * (v[:, :nd] * a).sum(1)
    heat = m * p / rho ** 2 * drho
    energy = (work + heat).sum()
    energy_scale = (np.abs(work) + np.abs(heat)).sum()
    return dict(mom=mom, mom_scale=mom_scale, ang=ang, ang_scale=ang_scale, energy=energy,
                energy_scale=energy_scale)


def gpu_example_dam_break(pkg, precision="float64"):
    """examples/fluid/dam_break_2d.jl as examples/fluid/dam_break_2d_gpu.jl includes it, at the
    fluid particle spacing 0.05 of the reference's GPU interpolation test
    (test/examples/gpu.jl:833-841): H = 0.6, W = 2H, tank length floor(5.366 H / dx) dx by 4,
    4 wall layers, Cole EOS with exponent 1 and c = 20 sqrt(g H), h = 2 dx, Monaghan alpha 0.02,
    Molteni-Colagrossi delta 0.1, clipped wall pressure.  Returns (semi, tank)."""
    H, dx, grav = 0.6, 0.05, 9.81
    eos = pkg.StateEquationCole(sound_speed=20 * math.sqrt(grav * H), reference_density=1000.0,
                                exponent=1.0)
    tank_x = math.floor(5.366 * H / dx) * dx
    tank = pkg.RectangularTank(dx, (2 * H, H), (tank_x, 4.0), 1000.0, n_layers=4,
                               acceleration=(0.0, -grav), state_equation=eos)
    semi = pkg.dam_break_semidiscretization(tank, eos, 2 * dx, precision=precision, alpha=0.02,
                                            delta=0.1, gravity=grav, wall_clip=True)
    return semi, tank


# Fields interpolated by the reference's Float32 GPU run of that setup at t = 0.01
# (StepsizeCallback(cfl=0.9), CarpenterKennedy2N54), test/examples/gpu.jl:843-916, compared
# there with isapprox, i.e. |got - ref| <= sqrt(eps(Float32)) |ref| in the 2-norm.
INTERP_GOLDEN = {
    "line": dict(  # interpolate_line (0.5, 0) -> (0.5, 0.5), 10 points, cut_off_bnd=false
        computed_density=[500.96387, 859.06744, 989.0479, 1001.3735, 1001.30927, 1001.0831,
                          1000.7325, 1000.3575, 999.8011, 975.98553],
        density=[1002.1891, 1002.0748, 1001.8913, 1001.67126, 1001.4529, 1001.2382, 1001.0298,
                 1000.81964, 1000.594, 1000.3878],
        pressure=[5154.1177, 4885.1, 4452.6533, 3934.9075, 3420.5737, 2915.0933, 2424.0908,
                  1929.7888, 1398.8309, 913.2089]),
    "line_h02": dict(  # the same line with smoothing_length = 0.2
        computed_density=[501.10648, 700.15857, 852.81036, 944.48535, 986.2611, 998.96576,
                          997.5659, 980.23236, 929.7254, 825.95825],
        density=[1001.98303, 1001.8848, 1001.7575, 1001.59985, 1001.41754, 1001.2164, 1001.0109,
                 1000.81616, 1000.6457, 1000.5056],
        pressure=[4668.169, 4437.7715, 4137.7075, 3768.1145, 3337.1655, 2863.6277, 2379.349,
                  1921.7727, 1519.3884, 1190.5823]),
    "plane": dict(  # interpolate_plane_2d (0, 0) -> (1, 1), resolution 0.4, cut_off_bnd=false
        computed_density=[250.47523, 500.98248, 500.49924, 253.77109, 500.0491, 1000.0818,
                          999.6527, 503.08704],
        density=[1002.2373, 1002.22516, 1001.4339, 999.3567, 1000.8318, 1000.80237, 1000.3408,
                 999.92017],
        pressure=[5267.867, 5239.2466, 3376.045, -1514.4237, 1958.2637, 1888.739, 802.3146,
                  -187.81871]),
}
INTERP_RTOL = float(np.sqrt(np.finfo(np.float32).eps))


def interp_golden_errors(results: dict) -> dict:
    """2-norm relative differences of the interpolated fields from INTERP_GOLDEN."""
    out = {}
    for case, fields in INTERP_GOLDEN.items():
        for f, ref in fields.items():
            ref = np.asarray(ref, dtype=np.float64)
            got = np.asarray(results[case][f], dtype=np.float64)
            out[f"{case}.{f}"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    return out
