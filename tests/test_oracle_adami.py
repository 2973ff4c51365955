"""Adami pressure extrapolation in the oracle: the properties the reference tests for it
(test/schemes/boundary/dummy_particles/dummy_particles.jl:308-697), restated for the path's
WendlandC2 kernel (support 2h = 3 dx, as the reference test's cubic spline with h = 1.5 dx):

* fluid at the reference density: fluid and wall pressures are exactly zero;
* fluid at another constant density: every wall pressure equals the fluid pressure (atol 1e-12);
* hydrostatic fluid: fluid and wall pressures together equal the hydrostatic pressure of a
  fluid-only tank covering fluid and walls (atol 4 Pa), i.e. the walls continue the gradient;
* fluid below the reference density (negative pressure): with clip_negative_pressure the walls
  get p = 0 and rho = rho0 exactly, without it the fluid's negative pressure and density
  (dummy_particles.jl:13-68).
"""
import numpy as np

from helpers import adami_tank_case, hydrostatic_fields, oracle_model


def _wall_state(pkg, orc, density, gravity, wall_clip=True):
    semi, tank, eos = adami_tank_case(pkg, density, gravity, wall_clip=wall_clip)
    model = oracle_model(orc, semi, tank)
    v = np.zeros((tank.fluid.n_particles, 3))
    v[:, 2] = tank.fluid.density
    _, st = model.kick(v, tank.fluid.coordinates)
    assert st == 0
    return model.last_state(), tank, eos


def test_constant_zero_pressure(pkg, orc):
    s, _, _ = _wall_state(pkg, orc, 257.0, 0.0)
    assert np.all(s["p_f"] == 0.0)
    assert np.all(s["p_w"] == 0.0)
    assert np.all(s["rho_w"] == 257.0)


def test_constant_nonzero_pressure(pkg, orc):
    s, _, eos = _wall_state(pkg, orc, 260.0, 0.0)
    assert np.allclose(s["p_f"], s["p_f"][0], rtol=0.0, atol=1e-12)
    assert s["p_f"][0] == eos(260.0)
    assert np.all(s["vol_w"] > 0.0)  # every wall particle sees fluid
    assert np.allclose(s["p_w"], s["p_f"][0], rtol=0.0, atol=1e-12)


def test_hydrostatic_pressure_gradient(pkg, orc):
    s, tank, eos = _wall_state(pkg, orc, 257.0, 9.81)
    got, ref = hydrostatic_fields(pkg, tank, eos, s["p_f"], s["p_w"])
    assert np.all(ref > 0.0)
    assert np.abs(got - ref).max() <= 4.0


def test_negative_pressure_clipping(pkg, orc):
    s, _, eos = _wall_state(pkg, orc, 250.0, 0.0, wall_clip=True)
    assert eos(250.0) < 0.0 and np.all(s["p_f"] == eos(250.0))
    assert np.all(s["p_w"] == 0.0) and np.all(s["rho_w"] == 257.0)
    s, _, _ = _wall_state(pkg, orc, 250.0, 0.0, wall_clip=False)
    assert np.abs(s["p_w"] - eos(250.0)).max() <= 1e-12
    assert np.abs(s["rho_w"] - 250.0).max() <= 1e-12 * 250.0
