"""SymplecticPositionVerlet on the GPU (tp_integrate_spv, solve with SymplecticPositionVerlet())
against the oracle's restatement: FP64 v within 1e-9, u and rho within 1e-12 relative L2 (the
runs are short enough for rounding differences to stay at that level); FP32 form within the
precision-form tolerances."""
import numpy as np
import pytest

from helpers import dam_break_case, initial_state, oracle_model, rel_l2

pytestmark = pytest.mark.gpu


def _spv(pkg, orc, cuda, nd, dx, fluid, tank, n, dt, precision):
    semi, tank_ = dam_break_case(pkg, nd, dx, fluid, tank, precision=precision, jitter=0.1,
                                 seed=6)
    ode = pkg.semidiscretize(semi, (0.0, n * dt))
    sol = pkg.solve(ode, pkg.SymplecticPositionVerlet(), dt=dt, n_steps=n)
    model = oracle_model(orc, semi, tank_)
    v0, u0 = initial_state(tank_)
    v_ref, u_ref, st = model.integrate_spv(v0, u0, dt, n)
    assert st == 0
    v, u = sol.v.cpu().numpy().reshape(-1, nd + 1), sol.u.cpu().numpy()
    semi.close()
    return v, u, v_ref.reshape(-1, nd + 1), u_ref


def test_spv_fp64_2d(pkg, orc, cuda):
    v, u, vr, ur = _spv(pkg, orc, cuda, 2, 0.02, (2.0, 1.0), (5.366, 4.0), 40, 1e-4, "float64")
    assert rel_l2(u, ur) <= 1e-12
    assert rel_l2(v[:, :2], vr[:, :2]) <= 1e-9
    assert rel_l2(v[:, 2], vr[:, 2]) <= 1e-12


def test_spv_fp64_3d(pkg, orc, cuda):
    v, u, vr, ur = _spv(pkg, orc, cuda, 3, 0.05, (1.0, 0.5, 1.0), (3.2, 1.0, 1.4), 10, 2e-4,
                        "float64")
    assert rel_l2(u, ur) <= 1e-12
    assert rel_l2(v[:, :3], vr[:, :3]) <= 1e-9
    assert rel_l2(v[:, 3], vr[:, 3]) <= 1e-12


def test_spv_fp32_form_2d(pkg, orc, cuda):
    v, u, vr, ur = _spv(pkg, orc, cuda, 2, 0.02, (2.0, 1.0), (5.366, 4.0), 40, 1e-4, "float32")
    assert rel_l2(u, ur) <= 1e-8
    assert rel_l2(v[:, :2], vr[:, :2]) <= 1e-4
    assert rel_l2(v[:, 2], vr[:, 2]) <= 1e-6
