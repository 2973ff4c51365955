"""Forward-mode derivatives through the oracle (dual numbers, oracle/dual.h), the counterpart of a
ForwardDiff gradient through the reference's CPU path (ForwardDiff is a dependency of the
reference and used by its tests, test/general/smoothing_kernels.jl:121).

* The value part of a dual run is the plain oracle run bit for bit: the dual instantiation
  executes the same operations, branches and neighbour sets.
* The derivatives with respect to Monaghan alpha, Molteni-Colagrossi delta, the gravity
  magnitude and the initial velocity along a seeded direction match central differences through
  the plain oracle (h = 1e-4 relative to the parameter, 1e-5 m/s on the velocity direction,
  small enough that no viscosity switch or neighbour set changes between the two runs) to 1e-6
  relative in the 2-norm of the final state's derivative."""
import numpy as np
import pytest

from helpers import oracle_model

DX, N_STEPS = 0.1, 12


def _case(pkg, alpha=0.02, delta=0.1, gravity=9.81):
    tank, eos = pkg.dam_break(2, DX, (1.0, 0.5), (2.0, 1.0), n_layers=3)
    semi = pkg.dam_break_semidiscretization(tank, eos, 1.75 * DX, alpha=alpha, delta=delta,
                                            gravity=gravity)
    return semi, tank


def _start(tank, seed=3):
    rng = np.random.default_rng(seed)
    n = tank.fluid.n_particles
    v = np.zeros((n, 3))
    v[:, :2] = rng.normal(0.0, 0.2, (n, 2))
    v[:, 2] = tank.fluid.density
    return v, tank.fluid.coordinates.copy()


def _plain(orc, pkg, v, u, dt, **params):
    semi, tank = _case(pkg, **params)
    _, tank0 = _case(pkg)
    m = oracle_model(orc, semi, tank0)
    vv, uu, st = m.integrate(v, u, dt, N_STEPS)
    assert st == 0
    return vv, uu


def test_dual_value_part_equals_the_oracle(pkg, orc):
    semi, tank = _case(pkg)
    v, u = _start(tank)
    dt = 5e-3 * DX
    vv, uu = _plain(orc, pkg, v, u, dt)
    vd, ud, dv, du, st = orc.integrate_jvp(semi.config, tank.boundary.coordinates,
                                           tank.boundary.mass, tank.fluid.mass, v, u, dt, N_STEPS)
    assert st == 0
    assert np.array_equal(vd, vv) and np.array_equal(ud, uu)
    assert np.all(np.isfinite(dv)) and np.all(np.isfinite(du))
    assert np.abs(du).max() > 0.0


@pytest.mark.parametrize("k,name", [(0, "alpha"), (1, "delta"), (2, "gravity"), (3, "v0")])
def test_dual_derivatives_match_central_differences(pkg, orc, k, name):
    semi, tank = _case(pkg)
    v, u = _start(tank)
    dt = 5e-3 * DX
    w = np.zeros_like(v)
    w[:, :2] = np.random.default_rng(5).normal(size=(v.shape[0], 2))
    _, _, dv, du, st = orc.integrate_jvp(semi.config, tank.boundary.coordinates,
                                         tank.boundary.mass, tank.fluid.mass, v, u, dt, N_STEPS,
                                         v_dir=w)
    assert st == 0
    base = dict(alpha=0.02, delta=0.1, gravity=9.81)
    if name == "v0":
        h = 1e-5
        vp, up = _plain(orc, pkg, v + h * w, u, dt)
        vm, um = _plain(orc, pkg, v - h * w, u, dt)
    else:
        h = 1e-4 * base[name]
        vp, up = _plain(orc, pkg, v, u, dt, **dict(base, **{name: base[name] + h}))
        vm, um = _plain(orc, pkg, v, u, dt, **dict(base, **{name: base[name] - h}))
    fd_u = (up - um) / (2 * h)
    fd_v = (vp - vm) / (2 * h)
    for got, fd in ((du[k], fd_u), (dv[k], fd_v)):
        assert np.linalg.norm(got - fd) <= 1e-6 * np.linalg.norm(fd), name
