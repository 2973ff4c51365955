"""SortingCallback on the GPU (tp_sort_particles): the permutation equals the oracle's (the
reference's stable sortperm over cell coordinates) bit for bit, the state moves with it, and a
simulation with sorting equals one without after undoing the permutation (FP64: v within 1e-9,
u within 1e-12 relative; summation order inside cells changes with the particle order)."""
import numpy as np
import pytest
import torch

from helpers import dam_break_case, initial_state, rel_l2

pytestmark = pytest.mark.gpu


def _case(pkg, nd, precision="float64"):
    if nd == 2:
        return dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.3, seed=8,
                              precision=precision)
    return dam_break_case(pkg, 3, 0.05, (1.0, 0.5, 1.0), (3.2, 1.0, 1.4), jitter=0.3, seed=8,
                          precision=precision)


@pytest.mark.parametrize("nd", [2, 3])
def test_sort_perm_matches_oracle(pkg, orc, cuda, nd):
    semi, tank = _case(pkg, nd)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v0, u0 = initial_state(tank)
    rng = np.random.default_rng(2)
    shuffle = rng.permutation(v0.shape[0])
    v0, u0 = v0[shuffle], u0[shuffle]
    v = torch.as_tensor(v0.ravel(), device="cuda")
    u = torch.as_tensor(u0.ravel(), device="cuda")
    cb = pkg.SortingCallback(interval=1)
    perm = cb.sort(semi, v, u).cpu().numpy()
    ref = orc.sort_perm(semi.config, u0)
    assert np.array_equal(perm, ref)
    assert np.array_equal(u.cpu().numpy().reshape(-1, nd), u0[ref])
    assert np.array_equal(v.cpu().numpy().reshape(-1, nd + 1), v0[ref])
    semi.close()


def test_kick_after_sorting_with_masses(pkg, cuda):
    semi, tank = _case(pkg, 2)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v, u = ode.v0.clone(), ode.u0.clone()
    dv0 = torch.zeros_like(v)
    pkg.kick(dv0, v, u, ode.p, 0.0)
    cb = pkg.SortingCallback(interval=1, sort_masses=True)
    perm = cb.sort(semi, v, u)
    dv1 = torch.zeros_like(v)
    pkg.kick(dv1, v, u, ode.p, 0.0)
    semi.sync()
    a = dv1.view(-1, 3).cpu().numpy()
    b = dv0.view(-1, 3).cpu().numpy()[perm.cpu().numpy()]
    assert rel_l2(a, b) <= 1e-12
    semi.close()


def test_reference_mass_behaviour(pkg, cuda):
    """sort_masses=False (the reference): masses stay at their array positions, so with
    hydrostatic (non-uniform) masses the kick after sorting differs from the permuted one."""
    semi, tank = _case(pkg, 2)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v, u = ode.v0.clone(), ode.u0.clone()
    dv0 = torch.zeros_like(v)
    pkg.kick(dv0, v, u, ode.p, 0.0)
    perm = pkg.SortingCallback(interval=1).sort(semi, v, u)
    dv1 = torch.zeros_like(v)
    pkg.kick(dv1, v, u, ode.p, 0.0)
    semi.sync()
    moved = not np.array_equal(perm.cpu().numpy(), np.arange(perm.numel()))
    assert moved
    a = dv1.view(-1, 3).cpu().numpy()
    b = dv0.view(-1, 3).cpu().numpy()[perm.cpu().numpy()]
    assert rel_l2(a, b) > 1e-10
    semi.close()


@pytest.mark.parametrize("alg", ["ck", "spv"])
def test_solve_with_sorting_callback(pkg, cuda, alg):
    n, dt = 30, 1e-4
    A = pkg.CarpenterKennedy2N54() if alg == "ck" else pkg.SymplecticPositionVerlet()
    s1, _ = _case(pkg, 2)
    o1 = pkg.semidiscretize(s1, (0.0, n * dt))
    ref = pkg.solve(o1, A, dt=dt, n_steps=n)
    s2, _ = _case(pkg, 2)
    o2 = pkg.semidiscretize(s2, (0.0, n * dt))
    sol = pkg.solve(o2, A, dt=dt, n_steps=n,
                    callback=pkg.SortingCallback(interval=7, sort_masses=True))
    perm = sol.perm.cpu().numpy()
    assert sorted(perm.tolist()) == list(range(perm.size))
    vr = ref.v.view(-1, 3).cpu().numpy()[perm]
    ur = ref.u.view(-1, 2).cpu().numpy()[perm]
    assert rel_l2(sol.u.view(-1, 2).cpu().numpy(), ur) <= 1e-12
    assert rel_l2(sol.v.view(-1, 3).cpu().numpy(), vr) <= 1e-9
    s1.close()
    s2.close()
