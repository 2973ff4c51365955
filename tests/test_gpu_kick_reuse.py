"""kick! with neighbour-list reuse: successive kicks of a moving state (the calls a
CarpenterKennedy2N54 or SymplecticPositionVerlet stage loop makes) refresh the records through the
last permutation and rebuild only after skin * h of displacement; every kick must still equal a
fresh neighbour search -- the oracle's kick of the same state -- including after rebuilds,
after another entry point has re-sorted the handle, and after the caller reordered its arrays."""
import numpy as np
import pytest
import torch

from helpers import dam_break_case, initial_state, oracle_model, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_kicks_along_a_trajectory_match_oracle(pkg, orc, cuda, precision):
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=3,
                                precision=precision)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    model = oracle_model(orc, semi, tank)
    v0, u0 = initial_state(tank)
    rng = np.random.default_rng(5)
    v0[:, :2] = rng.normal(0.0, 0.3, (v0.shape[0], 2))
    tol = 1e-11 if precision == "float64" else 2e-5
    v, u = v0.copy(), u0.copy()
    moved = 0.0
    for k in range(40):
        # drift the caller state by 0.01 h per call: a rebuild every ~10 calls
        u = u + 0.01 * 0.035 * v[:, :2] / np.maximum(np.abs(v[:, :2]).max(), 1e-12)
        moved += 0.01 * 0.035
        if k == 25:  # the caller reorders its arrays (as a SortingCallback would)
            perm = rng.permutation(u.shape[0])
            u, v = u[perm], v[perm]
            import ctypes
            m = semi.fluid.initial_condition.mass[perm]
            mt = torch.as_tensor(m, device="cuda")
            semi._call("tp_set_fluid_mass", ctypes.c_void_p(mt.data_ptr()))
            model = orc.Model(semi.config, tank.boundary.coordinates, tank.boundary.mass, m)
        if k == 30:  # another entry point re-sorts the handle
            semi.fluid_pressure()
            pkg.interpolate_points(np.array([[1.0], [0.5]]), semi, semi.fluid,
                                   torch.as_tensor(v.ravel(), device="cuda"),
                                   torch.as_tensor(u.ravel(), device="cuda"))
        vt = torch.as_tensor(v.ravel(), device="cuda")
        ut = torch.as_tensor(u.ravel(), device="cuda")
        dv = torch.zeros_like(vt)
        pkg.kick(dv, vt, ut, ode.p, 0.0)
        semi.sync()
        ref, st = model.kick(v, u)
        assert st == 0
        g = dv.cpu().numpy().reshape(-1, 3)
        r = ref.reshape(-1, 3)
        assert rel_l2(g[:, :2], r[:, :2]) <= tol, k
    assert moved > 0.3 * 0.035  # several rebuilds happened along the way
    semi.close()


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_warm_started_integrator_calls(pkg, orc, cuda, precision):
    """Consecutive tp_integrate_ck2n54 calls continue from the previous call's slot order and
    lists (warm start); 4 calls of 10 steps equal 40 steps of the oracle, also when the caller
    hands in a permuted state in between (the gate then rebuilds)."""
    import ctypes

    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=3,
                                precision=precision)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    model = oracle_model(orc, semi, tank)
    v0, u0 = initial_state(tank)
    dt = 1e-4
    v, u = ode.v0.clone(), ode.u0.clone()
    for _ in range(2):
        semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(dt), ctypes.c_int64(10))
    # permute the caller state (and masses) between calls
    rng = np.random.default_rng(7)
    perm = rng.permutation(tank.fluid.n_particles)
    pt = torch.as_tensor(perm, device="cuda")
    v = v.view(-1, 3)[pt].reshape(-1).contiguous()
    u = u.view(-1, 2)[pt].reshape(-1).contiguous()
    m = torch.as_tensor(tank.fluid.mass[perm], device="cuda")
    semi._call("tp_set_fluid_mass", m.data_ptr())
    for _ in range(2):
        semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                   ctypes.c_double(dt), ctypes.c_int64(10))
    semi.sync()
    v_ref, u_ref, st = model.integrate(v0, u0, dt, 40)
    assert st == 0
    vr = v_ref.reshape(-1, 3)[perm]
    ur = u_ref.reshape(-1, 2)[perm]
    vg = v.view(-1, 3).cpu().numpy()
    ug = u.view(-1, 2).cpu().numpy()
    if precision == "float64":
        assert rel_l2(ug, ur) <= 1e-12 and rel_l2(vg[:, :2], vr[:, :2]) <= 1e-9
    else:
        assert rel_l2(ug, ur) <= 1e-8 and rel_l2(vg[:, :2], vr[:, :2]) <= 1e-4
    semi.close()
