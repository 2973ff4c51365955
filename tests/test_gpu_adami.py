"""Adami pressure extrapolation on the device: the properties the reference tests for it
(test/schemes/boundary/dummy_particles/dummy_particles.jl:308-697), restated for WendlandC2 with
support 3 dx, through tp_kick and the pressure / wall-state accessors, in both precision forms:

* fluid at the reference density: fluid and wall pressures exactly zero, wall density rho0;
* fluid at another constant density: every wall pressure equals the fluid pressure;
* hydrostatic fluid: the walls continue the fluid's hydrostatic gradient (atol 4 Pa against a
  fluid-only tank covering fluid and walls), and the wall state matches the oracle's;
* fluid below the reference density: clipped walls get p = 0 and rho = rho0 exactly, unclipped
  walls the fluid's negative pressure and its density (dummy_particles.jl:13-68).
"""
import numpy as np
import pytest

from helpers import adami_tank_case, hydrostatic_fields, oracle_model

pytestmark = pytest.mark.gpu

PRECISIONS = ["float64", "float32"]


def _device_state(pkg, cuda, density, gravity, precision, wall_clip=True):
    torch = cuda
    semi, tank, eos = adami_tank_case(pkg, density, gravity, precision=precision,
                                      wall_clip=wall_clip)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v = np.zeros((tank.fluid.n_particles, 3))
    v[:, 2] = tank.fluid.density
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    u_t = torch.as_tensor(tank.fluid.coordinates.ravel(), device=semi.device)
    dv = torch.full_like(v_t, float("nan"))
    pkg.kick(dv, v_t, u_t, ode.p, 0.0)
    p_f = semi.fluid_pressure()
    p_w, rho_w, vol_w = semi.wall_state()
    semi.sync()
    out = dict(p_f=p_f.cpu().numpy(), p_w=p_w.cpu().numpy(), rho_w=rho_w.cpu().numpy(),
               vol_w=vol_w.cpu().numpy(), dv=dv.cpu().numpy())
    semi.close()
    return out, semi, tank, eos, v


@pytest.mark.parametrize("precision", PRECISIONS)
def test_constant_zero_pressure(pkg, cuda, precision):
    s, *_ = _device_state(pkg, cuda, 257.0, 0.0, precision)
    assert np.all(np.isfinite(s["dv"]))
    assert np.all(s["p_f"] == 0.0)
    assert np.all(s["p_w"] == 0.0)
    assert np.all(s["rho_w"] == 257.0)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_constant_nonzero_pressure(pkg, cuda, precision):
    s, _, _, eos, _ = _device_state(pkg, cuda, 260.0, 0.0, precision)
    p0 = eos(260.0)
    # FP64: rounding of the normalised sum; FP32 form: float EOS and sums (~10 ulp of p0 ~ 312)
    tol = 1e-12 if precision == "float64" else 1e-5 * p0
    assert np.all(s["vol_w"] > 0.0)
    assert np.abs(s["p_f"] - p0).max() <= tol
    assert np.abs(s["p_w"] - p0).max() <= tol


@pytest.mark.parametrize("precision", PRECISIONS)
def test_hydrostatic_pressure_gradient(pkg, orc, cuda, precision):
    s, semi, tank, eos, v = _device_state(pkg, cuda, 257.0, 9.81, precision)
    got, ref = hydrostatic_fields(pkg, tank, eos, s["p_f"], s["p_w"])
    assert np.all(ref > 0.0)
    assert np.abs(got - ref).max() <= 4.0
    model = oracle_model(orc, semi, tank)
    _, st = model.kick(v, tank.fluid.coordinates)
    assert st == 0
    o = model.last_state()
    if precision == "float64":
        assert np.abs(s["p_w"] - o["p_w"]).max() <= 1e-12 * np.abs(o["p_w"]).max()
        assert np.abs(s["rho_w"] - o["rho_w"]).max() <= 1e-13 * 257.0
    else:
        assert np.abs(s["p_w"] - o["p_w"]).max() <= 1e-5 * np.abs(o["p_w"]).max()
        assert np.abs(s["rho_w"] - o["rho_w"]).max() <= 1e-6 * 257.0


@pytest.mark.parametrize("precision", PRECISIONS)
def test_negative_pressure_clipping(pkg, cuda, precision):
    s, _, _, eos, _ = _device_state(pkg, cuda, 250.0, 0.0, precision, wall_clip=True)
    p0 = eos(250.0)
    assert p0 < 0.0
    assert np.all(s["p_w"] == 0.0) and np.all(s["rho_w"] == 257.0)
    s, *_ = _device_state(pkg, cuda, 250.0, 0.0, precision, wall_clip=False)
    # FP32 form: float EOS, its inverse and sums (a few ulp of |p0| ~ 750 and of rho)
    tol_p = 1e-12 if precision == "float64" else 1e-5 * abs(p0)
    tol_rho = 1e-12 * 250.0 if precision == "float64" else 1e-6 * 250.0
    assert np.abs(s["p_f"] - p0).max() <= tol_p
    assert np.abs(s["p_w"] - p0).max() <= tol_p
    assert np.abs(s["rho_w"] - 250.0).max() <= tol_rho
