"""Neighbour lists with a skin must list pairs two cells apart: cells are 2h wide and the list
radius is 2h (1 + skin), so two particles 2.1h apart across two cells -- not neighbours yet --
can approach to below 2h before any particle has moved far enough to force a rebuild.  The
fused integrators (lists rebuilt only on displacement) must then agree with the oracle, which
rebuilds its exact neighbour search every stage."""
import ctypes

import numpy as np
import pytest
import torch

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _config(pkg, precision):
    c = pkg.default_config()
    c.ndims = 2
    c.precision = precision
    c.n_fluid = 2
    c.n_wall = 0
    c.smoothing_length = 0.035
    c.sound_speed = 62.6
    c.reference_density = 1000.0
    for d in range(2):
        c.min_corner[d] = -0.5
        c.max_corner[d] = 2.0
    return c


def _state(skin):
    h = 0.035
    xa = 0.07 * 10 + 0.001           # 0.029 h inside cell 10
    xb = xa - 2.0 * h * (1.0 + 0.5 * skin)  # cell 8: two cells to the left, inside the list radius
    u = np.array([[xa, 0.5], [xb, 0.5]])
    v = np.array([[-1.0, 0.0, 1000.0], [1.0, 0.0, 1000.0]])
    return v, u


@pytest.mark.parametrize("skin", [0.05, 0.1])
@pytest.mark.parametrize("precision", [0, 1])
def test_pair_two_cells_apart_is_not_missed(lib, pkg, orc, cuda, precision, skin):
    c = _config(pkg, precision)
    v0, u0 = _state(skin)
    assert int(u0[0, 0] // 0.07) - int(u0[1, 0] // 0.07) == 2
    # contact (r < 2h) after 175 skin steps, first rebuild by displacement after 350 skin steps
    n, dt = 30, 1e-4
    model = orc.Model(c, np.zeros((0, 2)), np.zeros(0), np.full(2, 1.2))
    v_ref, u_ref, st = model.integrate(v0, u0, dt, n)
    assert st == 0
    v_ref = v_ref.reshape(-1, 3)
    assert np.all(np.abs(v_ref[:, 2] - 1000.0) > 1e-3)  # the pair did interact (rho rose)

    h = ctypes.c_void_p()
    assert lib.tp_create(ctypes.byref(c), ctypes.byref(h)) == 0
    assert lib.tp_set_skin(h, ctypes.c_double(skin)) == 0
    dummy = torch.zeros(2, dtype=torch.float64, device="cuda")
    mf = torch.full((2,), 1.2, dtype=torch.float64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.tp_set_wall(h, p(dummy), p(dummy)) == 0
    assert lib.tp_set_fluid_mass(h, p(mf)) == 0
    v = torch.as_tensor(v0.ravel(), device="cuda").contiguous()
    u = torch.as_tensor(u0.ravel(), device="cuda").contiguous()
    assert lib.tp_integrate_ck2n54(h, p(v), p(u), 0.0, dt, n) == 0
    assert lib.tp_sync(h) == 0
    vg = v.view(-1, 3).cpu().numpy()
    if precision == 0:
        assert rel_l2(u.cpu().numpy(), u_ref) <= 1e-13
        assert rel_l2(vg, v_ref) <= 1e-11
    else:
        assert rel_l2(vg[:, :2], v_ref[:, :2]) <= 1e-5
        assert rel_l2(vg[:, 2], v_ref[:, 2]) <= 1e-6
    # the differentiation form's per-step lists reach the same pair
    v2 = torch.as_tensor(v0.ravel(), device="cuda").contiguous()
    u2 = torch.as_tensor(u0.ravel(), device="cuda").contiguous()
    assert lib.tp_adjoint_forward(h, p(v2), p(u2), dt, n, 10) == 0
    va = v2.view(-1, 3).cpu().numpy()
    assert rel_l2(va[:, :2], v_ref[:, :2]) <= (1e-9 if precision == 0 else 1e-5)
    assert lib.tp_destroy(h) == 0
