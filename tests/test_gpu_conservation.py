"""Conservation properties of the device pair terms, through tp_kick: linear momentum, angular
momentum and total energy (test/schemes/fluid/rhs.jl:115-264; random configurations, three seeds,
no walls, no gravity), in both FP64 pair modes and the FP32 form.

Pressure + continuity (viscosity and diffusion off, as the reference's zero sound speed makes
them): all three rates vanish to rounding.  With the Monaghan viscosity: momentum and angular
momentum only.  Tolerances are relative to the sum of the summands' magnitudes: 1e-14 in FP64
(the CPU oracle reaches ~1e-17), 1e-5 in the FP32 form (FP32 pair arithmetic, compensated sums).
"""
import numpy as np
import pytest

from helpers import conservation_residuals, random_fluid_case

pytestmark = pytest.mark.gpu

FORMS = [("float64", 0), ("float64", 1), ("float32", 0), ("float32", 2)]
FORM_IDS = ["fp64-gather", "fp64-symmetric", "fp32", "fp32-tiled"]


def _device_rates(pkg, cuda, nd, seed, viscosity, precision, pair_mode):
    torch = cuda
    semi, x, v, m = random_fluid_case(pkg, nd, seed, n=8, viscosity=viscosity, diffusion=False,
                                      precision=precision)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    if precision == "float64":
        semi._call("tp_set_pair_mode", pair_mode)
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    dv = torch.full_like(v_t, float("nan"))
    pkg.kick(dv, v_t, ode.u0, ode.p, 0.0)
    p = semi.fluid_pressure()
    semi.sync()
    dv = dv.cpu().numpy().reshape(-1, nd + 1)
    assert np.all(np.isfinite(dv))
    r = conservation_residuals(x, v, m, dv, p.cpu().numpy())
    semi.close()
    return r


@pytest.mark.parametrize("precision,pair_mode", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_pressure_and_continuity_conserve_momentum_and_energy(pkg, cuda, seed, nd, precision,
                                                              pair_mode):
    r = _device_rates(pkg, cuda, nd, seed, False, precision, pair_mode)
    tol = 1e-14 if precision == "float64" else 1e-5
    assert np.all(np.abs(r["mom"]) <= tol * r["mom_scale"])
    assert np.all(np.abs(r["ang"]) <= tol * r["ang_scale"])
    assert abs(r["energy"]) <= tol * r["energy_scale"]


@pytest.mark.parametrize("precision,pair_mode", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("nd", [2, 3])
def test_monaghan_viscosity_conserves_momentum(pkg, cuda, nd, precision, pair_mode):
    r = _device_rates(pkg, cuda, nd, 1, True, precision, pair_mode)
    tol = 1e-14 if precision == "float64" else 1e-5
    assert np.all(np.abs(r["mom"]) <= tol * r["mom_scale"])
    assert np.all(np.abs(r["ang"]) <= tol * r["ang_scale"])
