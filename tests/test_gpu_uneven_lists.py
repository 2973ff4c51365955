"""Neighbour lists under uneven particle distributions, against the FP64 oracle.

The list builder groups a warp's lanes by cell row, prunes the searched rows and the staged
candidates against the group's bounding box, reaches a second cell along an axis for particles
near a cell face, and writes each slot's list in eight-entry chunks.  The dam-break tests place
particles on a (jittered) lattice; here the fluid is a dense clump (half the lattice spacing), a
sparse random scatter (cells with zero to a few particles, so a warp's lanes span many cells)
and particles pinned within 0.02 h of cell faces, with random velocities.  One kick (both FP64
pair modes and the FP32 form), a few fused CarpenterKennedy2N54 steps and a few
SymplecticPositionVerlet steps (the kick! path with list reuse) must match the oracle, which
searches exactly at every stage: a missed or misplaced list entry shows as an O(1) error.
"""
import ctypes

import numpy as np
import pytest

from helpers import oracle_model, rel_l2

pytestmark = pytest.mark.gpu


def _uneven_case(pkg, nd, precision, seed):
    dx = 0.02 if nd == 2 else 0.05
    fluid = (2.0, 1.0) if nd == 2 else (1.0, 0.5, 1.0)
    tank_size = (5.366, 4.0) if nd == 2 else (3.2, 1.0, 1.4)
    tank, eos = pkg.dam_break(nd, dx, fluid, tank_size, n_layers=3)
    n = tank.fluid.n_particles
    h = 1.75 * dx
    cs = 2.0 * h
    rng = np.random.default_rng(seed)
    lo = np.full(nd, 3.5 * dx)
    hi = lo + np.asarray(fluid) - dx
    n_clump = n // 3
    n_face = n // 6
    n_sparse = n - n_clump - n_face
    # dense clump: half the lattice spacing around the fluid block's centre, jittered
    side = int(np.ceil(n_clump ** (1.0 / nd)))
    g = np.stack(np.meshgrid(*[np.arange(side)] * nd, indexing="ij"), -1).reshape(-1, nd)[:n_clump]
    centre = 0.5 * (lo + hi)
    clump = centre + (g - 0.5 * side) * 0.5 * dx + rng.uniform(-0.1, 0.1, g.shape) * dx
    # sparse scatter over the whole fluid box
    sparse = rng.uniform(lo, hi, (n_sparse, nd))
    # near cell faces: a random point with one coordinate moved to within 0.02 h of a face of
    # the grid (faces at multiples of cs from the grid's lower corner, the wall's minimum)
    wall_min = tank.boundary.coordinates.min(axis=0)
    face = rng.uniform(lo, hi, (n_face, nd))
    axis = rng.integers(0, nd, n_face)
    k = np.floor((face[np.arange(n_face), axis] - wall_min[axis]) / cs)
    side_sign = rng.choice([-1.0, 1.0], n_face)
    off = np.where(side_sign < 0, rng.uniform(1e-4, 0.02, n_face) * h,
                   cs - rng.uniform(1e-4, 0.02, n_face) * h)
    face[np.arange(n_face), axis] = wall_min[axis] + k * cs + off
    tank.fluid.coordinates = np.concatenate([clump, sparse, face])
    semi = pkg.dam_break_semidiscretization(tank, eos, h, precision=precision)
    v = np.zeros((n, nd + 1))
    v[:, :nd] = rng.normal(0.0, 0.5, (n, nd))
    v[:, nd] = tank.fluid.density * (1.0 + rng.uniform(-1e-3, 1e-3, n))
    return semi, tank, v, tank.fluid.coordinates.copy()


@pytest.mark.parametrize("nd", [2, 3])
@pytest.mark.parametrize("precision,pair_mode", [("float64", 0), ("float64", 1), ("float32", 0),
                                                 ("float32", 2)],
                         ids=["fp64-gather", "fp64-symmetric", "fp32", "fp32-tiled"])
def test_uneven_kick_matches_oracle(pkg, orc, cuda, nd, precision, pair_mode):
    torch = cuda
    semi, tank, v, u = _uneven_case(pkg, nd, precision, seed=21 + nd)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    semi._call("tp_set_pair_mode", pair_mode)
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    u_t = torch.as_tensor(u.ravel(), device=semi.device)
    dv = torch.full_like(v_t, float("nan"))
    pkg.kick(dv, v_t, u_t, ode.p, 0.0)
    semi.sync()
    model = oracle_model(orc, semi, tank)
    ref, st = model.kick(v, u)
    assert st == 0
    g = dv.cpu().numpy().reshape(-1, nd + 1)
    r = ref.reshape(-1, nd + 1)
    assert np.all(np.isfinite(g))
    if precision == "float64":
        assert rel_l2(g, r) <= 1e-11
    else:  # FP32 pair arithmetic; a list error would be O(1)
        assert rel_l2(g[:, :nd], r[:, :nd]) <= 1e-4
        assert rel_l2(g[:, nd], r[:, nd]) <= 1e-3
    semi.close()


@pytest.mark.parametrize("nd", [2, 3])
def test_uneven_integration_matches_oracle(pkg, orc, cuda, nd):
    """Fused FP64 steps with list reuse and displacement-gated rebuilds (skin 0.05; 0.5 m/s
    random velocities move particles past the skin within a few steps)."""
    torch = cuda
    semi, tank, v, u = _uneven_case(pkg, nd, "float64", seed=31 + nd)
    pkg.semidiscretize(semi, (0.0, 1.0))
    dt, n = 2e-4, 8
    v_t = torch.as_tensor(v.ravel(), device=semi.device).contiguous()
    u_t = torch.as_tensor(u.ravel(), device=semi.device).contiguous()
    semi._call("tp_integrate_ck2n54", v_t.data_ptr(), u_t.data_ptr(), ctypes.c_double(0.0),
               ctypes.c_double(dt), ctypes.c_int64(n))
    semi.sync()
    model = oracle_model(orc, semi, tank)
    v_ref, u_ref, st = model.integrate(v, u, dt, n)
    assert st == 0
    vg = v_t.view(-1, nd + 1).cpu().numpy()
    ug = u_t.view(-1, nd).cpu().numpy()
    assert rel_l2(ug, u_ref.reshape(-1, nd)) <= 1e-12
    assert rel_l2(vg, v_ref.reshape(-1, nd + 1)) <= 1e-9
    semi.close()


@pytest.mark.parametrize("nd", [2, 3])
def test_uneven_spv_matches_oracle(pkg, orc, cuda, nd):
    """SymplecticPositionVerlet: two kicks per step through the kick! path, whose lists are
    reused across kicks (records refreshed through the last permutation) and rebuilt on
    displacement."""
    torch = cuda
    semi, tank, v, u = _uneven_case(pkg, nd, "float64", seed=41 + nd)
    pkg.semidiscretize(semi, (0.0, 1.0))
    dt, n = 2e-4, 8
    v_t = torch.as_tensor(v.ravel(), device=semi.device).contiguous()
    u_t = torch.as_tensor(u.ravel(), device=semi.device).contiguous()
    semi._call("tp_integrate_spv", v_t.data_ptr(), u_t.data_ptr(), ctypes.c_double(0.0),
               ctypes.c_double(dt), ctypes.c_int64(n))
    semi.sync()
    model = oracle_model(orc, semi, tank)
    v_ref, u_ref, st = model.integrate_spv(v, u, dt, n)
    assert st == 0
    vg = v_t.view(-1, nd + 1).cpu().numpy()
    ug = u_t.view(-1, nd).cpu().numpy()
    vr = v_ref.reshape(-1, nd + 1)
    assert rel_l2(ug, u_ref.reshape(-1, nd)) <= 1e-12
    assert rel_l2(vg[:, :nd], vr[:, :nd]) <= 1e-9
    # the clump's large density rates and the scheme's multiplicative density update amplify the
    # ulp-level differences (FMA contraction, the EOS power) to ~2e-12; a list error is O(1)
    assert rel_l2(vg[:, nd], vr[:, nd]) <= 1e-11
    semi.close()
