"""The fluid pressure accessor after each entry point that reorders particles internally: the
pressure of the last right-hand side comes back in the caller's particle order after tp_kick,
after the fused CarpenterKennedy2N54 integrator (whose slots follow cell order, not the caller's)
and after SymplecticPositionVerlet; after an unconditional reordering it is refused until the
next kick.  Distinct per-particle densities make any misordering visible."""
import ctypes

import numpy as np
import pytest
import torch

from helpers import dam_break_case

pytestmark = pytest.mark.gpu


def _cole(rho, c):
    b = c.reference_density * c.sound_speed ** 2 / c.exponent
    return b * ((rho / c.reference_density) ** c.exponent - 1.0) + c.background_pressure


def _setup(pkg, precision):
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=11,
                                precision=precision)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    rng = np.random.default_rng(2)
    v = ode.v0.clone().view(-1, 3)
    v[:, 2] += torch.as_tensor(rng.uniform(-2.0, 2.0, v.shape[0]), device="cuda")
    return semi, ode, v.reshape(-1).contiguous(), ode.u0.clone()


def _pressure(semi):
    p = semi.fluid_pressure()
    semi.sync()
    return p.cpu().numpy()


def _kick_pressure(pkg, semi, ode, v, u):
    dv = torch.zeros_like(v)
    pkg.kick(dv, v, u, ode.p, 0.0)
    return _pressure(semi)


@pytest.mark.parametrize("precision", ["float64", "float32"])
@pytest.mark.parametrize("entry", ["tp_integrate_ck2n54", "tp_integrate_spv"])
def test_pressure_after_integration_is_in_caller_order(pkg, cuda, precision, entry):
    semi, ode, v, u = _setup(pkg, precision)
    # dt = 0: every stage sees the initial state, so the integrator's last right-hand side has
    # exactly the pressure a kick of the same state gives
    semi._call(entry, v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0), ctypes.c_double(0.0),
               ctypes.c_int64(1))
    p_int = _pressure(semi)
    p_kick = _kick_pressure(pkg, semi, ode, v, u)
    rho = v.view(-1, 3)[:, 2].cpu().numpy()
    if precision == "float64":
        assert np.array_equal(p_int, p_kick)
        assert np.allclose(p_int, _cole(rho, semi.config), rtol=1e-12, atol=1e-9)
    else:  # FP32 records: pressure rounded to float
        assert np.allclose(p_int, p_kick, rtol=1e-6, atol=1e-3)
        assert np.allclose(p_int, _cole(rho, semi.config), rtol=1e-5, atol=1e-2)
    # a moving run: the last stage's pressure stays close to that of the final density (one
    # stage of density change), far closer than the spread a misordering would show
    dt = 1e-5
    semi._call(entry, v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0), ctypes.c_double(dt),
               ctypes.c_int64(5))
    p_int = _pressure(semi)
    rho = v.view(-1, 3)[:, 2].cpu().numpy()
    p_final = _cole(rho, semi.config)
    spread = p_final.max() - p_final.min()
    assert np.abs(p_int - p_final).max() < 0.05 * spread
    semi.close()


def test_pressure_refused_after_a_reordering(pkg, cuda):
    semi, ode, v, u = _setup(pkg, "float64")
    _kick_pressure(pkg, semi, ode, v, u)
    semi._call("tp_sort_particles", v.data_ptr(), u.data_ptr(), 0, None)
    with pytest.raises(Exception, match="call tp_kick first"):
        semi.fluid_pressure()
    # the next kick makes the accessor valid again, in the new caller order
    p = _kick_pressure(pkg, semi, ode, v, u)
    rho = v.view(-1, 3)[:, 2].cpu().numpy()
    assert np.allclose(p, _cole(rho, semi.config), rtol=1e-12, atol=1e-9)
    semi.close()
