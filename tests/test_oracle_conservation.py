"""Conservation properties of the pair terms in the oracle: linear momentum, angular momentum and
total energy (test/schemes/fluid/rhs.jl:115-264: random particle configurations, three seeds,
no walls, no gravity).

The reference runs the test with a zero sound speed, which switches the Monaghan viscosity and the
density diffusion off; here they are switched off explicitly, and the densities (so the Cole EOS
pressures) are random.  The pressure term -m_b (p_a + p_b) / (rho_a rho_b) grad W_ab and the
continuity term (rho_a / rho_b) m_b v_ab . grad W_ab then conserve all three to rounding: the
forces are antisymmetric and along x_ab, and the pressure work cancels p_a / rho_a^2 drho_a
pairwise.  With the Monaghan viscosity on, momentum and angular momentum are still conserved (its
force is antisymmetric and along x_ab), energy is not (it dissipates).
"""
import numpy as np
import pytest

from helpers import conservation_residuals, random_fluid_case

SEEDS = [1, 2, 3]


def _oracle_rates(pkg, orc, nd, seed, viscosity):
    semi, x, v, m = random_fluid_case(pkg, nd, seed, viscosity=viscosity, diffusion=False)
    model = orc.Model(semi.config, np.zeros((0, nd)), np.zeros(0), m)
    dv, st = model.kick(v, x)
    assert st == 0
    dv = dv.reshape(-1, nd + 1)
    return conservation_residuals(x, v, m, dv, model.last_state()["p_f"])


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("seed", SEEDS)
def test_pressure_and_continuity_conserve_momentum_and_energy(pkg, orc, nd, seed):
    r = _oracle_rates(pkg, orc, nd, seed, viscosity=False)
    assert np.all(np.abs(r["mom"]) <= 1e-14 * r["mom_scale"])
    assert np.all(np.abs(r["ang"]) <= 1e-14 * r["ang_scale"])
    assert abs(r["energy"]) <= 1e-14 * r["energy_scale"]


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("seed", SEEDS)
def test_monaghan_viscosity_conserves_momentum(pkg, orc, nd, seed):
    r = _oracle_rates(pkg, orc, nd, seed, viscosity=True)
    assert np.all(np.abs(r["mom"]) <= 1e-14 * r["mom_scale"])
    assert np.all(np.abs(r["ang"]) <= 1e-14 * r["ang_scale"])
    # dissipative: the pair terms remove kinetic energy of approaching pairs
    r0 = _oracle_rates(pkg, orc, nd, seed, viscosity=False)
    assert r["energy"] < r0["energy"] - 1e-6 * r["energy_scale"]
