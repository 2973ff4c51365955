"""The fused CarpenterKennedy2N54 integrator on the GPU against the oracle.

FP64 drop-in: relative L2 error of v and u after the run <= 1e-9 (the runs are short enough
for rounding differences to stay at that level).  FP32 form: density and velocity within the
stated precision-form tolerance of the FP64 oracle.
"""
import numpy as np
import pytest

from helpers import dam_break_case, initial_state, oracle_model, rel_l2

pytestmark = pytest.mark.gpu


def _integrate(pkg, orc, cuda, nd, dx, fluid, tank, n_steps, dt, precision, jitter=0.0,
               pair_mode=None):
    torch = cuda
    semi, tank_ = dam_break_case(pkg, nd, dx, fluid, tank, precision=precision, jitter=jitter,
                                 seed=1)
    ode = pkg.semidiscretize(semi, (0.0, n_steps * dt))
    if pair_mode is not None:
        semi._call("tp_set_pair_mode", pair_mode)
    sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=n_steps)
    model = oracle_model(orc, semi, tank_)
    v0, u0 = initial_state(tank_)
    v_ref, u_ref, st = model.integrate(v0, u0, dt, n_steps)
    assert st == 0
    out = (sol.v.cpu().numpy(), sol.u.cpu().numpy(), v_ref, u_ref, semi)
    return out


@pytest.mark.parametrize("mode", [0, 1], ids=["gather", "symmetric"])
def test_integrate_fp64_2d(pkg, orc, cuda, mode):
    v, u, v_ref, u_ref, semi = _integrate(pkg, orc, cuda, 2, 0.02, (2.0, 1.0), (5.366, 4.0),
                                          40, 1e-4, "float64", pair_mode=mode)
    nd = 2
    vr, vg = v_ref.reshape(-1, nd + 1), v.reshape(-1, nd + 1)
    assert rel_l2(u, u_ref) <= 1e-12
    assert rel_l2(vg[:, :nd], vr[:, :nd]) <= 1e-9
    assert rel_l2(vg[:, nd], vr[:, nd]) <= 1e-12
    semi.close()


def test_integrate_2d_dam_break_200_steps(pkg, orc, cuda):
    """The 2D dam break (5000 fluid particles, 3 wall layers, dx = 0.02) over its full 200 steps
    at dt = 1e-4 from rest, FP64 drop-in and FP32 form against the oracle."""
    nd = 2
    v, u, v_ref, u_ref, semi = _integrate(pkg, orc, cuda, 2, 0.02, (2.0, 1.0), (5.366, 4.0),
                                          200, 1e-4, "float64")
    vr, vg = v_ref.reshape(-1, nd + 1), v.reshape(-1, nd + 1)
    assert rel_l2(u, u_ref) <= 1e-11
    assert rel_l2(vg[:, :nd], vr[:, :nd]) <= 1e-8
    assert rel_l2(vg[:, nd], vr[:, nd]) <= 1e-11
    semi.close()
    v, u, _, _, semi = _integrate(pkg, orc, cuda, 2, 0.02, (2.0, 1.0), (5.366, 4.0), 200, 1e-4,
                                  "float32")
    vg = v.reshape(-1, nd + 1)
    assert rel_l2(u, u_ref) <= 1e-7
    assert rel_l2(vg[:, :nd], vr[:, :nd]) <= 1e-4
    assert rel_l2(vg[:, nd], vr[:, nd]) <= 1e-7
    semi.close()


def test_integrate_fp64_3d_jittered(pkg, orc, cuda):
    v, u, v_ref, u_ref, semi = _integrate(pkg, orc, cuda, 3, 0.05, (1.0, 0.5, 1.0),
                                          (3.2, 1.0, 1.4), 10, 2e-4, "float64", jitter=0.1)
    nd = 3
    vr, vg = v_ref.reshape(-1, nd + 1), v.reshape(-1, nd + 1)
    assert rel_l2(u, u_ref) <= 1e-12
    assert rel_l2(vg[:, :nd], vr[:, :nd]) <= 1e-9
    assert rel_l2(vg[:, nd], vr[:, nd]) <= 1e-12
    semi.close()


@pytest.mark.parametrize("mode", [0, 2], ids=["lists", "tiled"])
def test_integrate_fp32_form_2d(pkg, orc, cuda, mode):
    v, u, v_ref, u_ref, semi = _integrate(pkg, orc, cuda, 2, 0.02, (2.0, 1.0), (5.366, 4.0),
                                          40, 1e-4, "float32", pair_mode=mode)
    nd = 2
    vr, vg = v_ref.reshape(-1, nd + 1), v.reshape(-1, nd + 1)
    assert rel_l2(u, u_ref) <= 1e-8
    assert rel_l2(vg[:, :nd], vr[:, :nd]) <= 1e-4
    assert rel_l2(vg[:, nd], vr[:, nd]) <= 1e-6
    semi.close()


def test_fused_integrator_equals_kick_drift_loop(pkg, cuda):
    """The fused stage kernel and a host loop over kick!/drift! with the 2N update agree."""
    torch = cuda
    semi, tank = dam_break_case(pkg, 2, 0.04, (1.0, 0.5), (2.0, 1.0), jitter=0.1, seed=4)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    dt, n = 1e-4, 5
    sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=n)
    import oracle.oracle as O

    A, B, _ = O.ck2n54_coefficients()
    v, u = ode.v0.clone(), ode.u0.clone()
    tv, tu = torch.zeros_like(v), torch.zeros_like(u)
    kv, ku = torch.zeros_like(v), torch.zeros_like(u)
    for _ in range(n):
        for s in range(5):
            pkg.kick(kv, v, u, ode.p, 0.0)
            pkg.drift(ku, v, u, ode.p, 0.0)
            if s == 0:
                tv, tu = dt * kv, dt * ku
            else:
                tv, tu = A[s] * tv + dt * kv, A[s] * tu + dt * ku
            v, u = v + B[s] * tv, u + B[s] * tu
    semi.sync()
    assert rel_l2(sol.u.cpu().numpy(), u.cpu().numpy()) <= 1e-13
    assert rel_l2(sol.v.cpu().numpy(), v.cpu().numpy()) <= 1e-10
    semi.close()


def test_conservation_and_zero_steps(pkg, cuda):
    torch = cuda
    semi, tank = dam_break_case(pkg, 3, 0.06, (0.6, 0.3, 0.6), (1.2, 0.6, 0.8))
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    c0 = semi.conservation(ode.v0)
    assert c0[0] == pytest.approx(tank.fluid.mass.sum(), rel=1e-14)
    assert np.all(c0[1:] == 0.0)
    sol0 = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=1e-4, n_steps=0)
    assert torch.equal(sol0.u, ode.u0) and torch.equal(sol0.v, ode.v0)
    sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=1e-4, n_steps=20)
    c1 = semi.conservation(sol.v)
    assert c1[0] == c0[0]  # masses are constant
    assert c1[2] < 0  # the column starts to fall
    assert np.all(np.isfinite(c1))
    semi.close()
