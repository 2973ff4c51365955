"""Edge cases through the C ABI on the GPU: empty fluid, no walls, a single particle, particles
outside the FullGridCellList box or with non-finite coordinates (reported, never an
out-of-bounds access: cell indices are clamped), list-capacity overflow after fixing the lists,
and the cell-grid size limit."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _config(pkg, nf, nw, nd=2, lo=-0.5, hi=2.0, precision=0):
    c = pkg.default_config()
    c.ndims = nd
    c.precision = precision
    c.n_fluid = nf
    c.n_wall = nw
    c.smoothing_length = 0.035
    c.sound_speed = 62.6
    c.reference_density = 1000.0
    c.acceleration[1] = -9.81
    for d in range(nd):
        c.min_corner[d] = lo
        c.max_corner[d] = hi
    return c


def _handle(lib, pkg, c, xw=None, mf=None):
    h = ctypes.c_void_p()
    assert lib.tp_create(ctypes.byref(c), ctypes.byref(h)) == 0
    nd, nf, nw = c.ndims, c.n_fluid, c.n_wall
    xw_t = torch.as_tensor(np.zeros((max(nw, 1), nd)) if xw is None else xw,
                           dtype=torch.float64, device="cuda").reshape(-1).contiguous()
    mw_t = torch.full((max(nw, 1),), 0.5, dtype=torch.float64, device="cuda")
    mf_t = torch.full((max(nf, 1),), 1.2, dtype=torch.float64, device="cuda") if mf is None \
        else torch.as_tensor(mf, device="cuda")
    assert lib.tp_set_wall(h, ctypes.c_void_p(xw_t.data_ptr()), ctypes.c_void_p(mw_t.data_ptr())) == 0
    assert lib.tp_set_fluid_mass(h, ctypes.c_void_p(mf_t.data_ptr())) == 0
    return h, (xw_t, mw_t, mf_t)


def _state(nf, nd, x, rho=1000.0):
    v = np.zeros((max(nf, 1), nd + 1))
    v[:, nd] = rho
    return (torch.as_tensor(v.reshape(-1), device="cuda").contiguous(),
            torch.as_tensor(np.asarray(x, dtype=np.float64).reshape(-1), device="cuda").contiguous())


@pytest.mark.parametrize("precision", [0, 1])
def test_empty_fluid(lib, pkg, cuda, precision):
    nw = 50
    xw = np.stack([np.linspace(0, 1, nw), np.zeros(nw)], 1)
    h, keep = _handle(lib, pkg, _config(pkg, 0, nw, precision=precision), xw=xw)
    v, u = _state(0, 2, np.zeros((1, 2)))
    dv = torch.zeros_like(v)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.tp_kick(h, p(dv), p(v), p(u), 0.0) == 0
    assert lib.tp_integrate_ck2n54(h, p(v), p(u), 0.0, 1e-4, 3) == 0
    assert lib.tp_integrate_spv(h, p(v), p(u), 0.0, 1e-4, 3) == 0
    assert lib.tp_sync(h) == 0
    assert lib.tp_destroy(h) == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_single_particle_without_walls_falls_freely(lib, pkg, cuda, precision):
    h, keep = _handle(lib, pkg, _config(pkg, 1, 0, precision=precision))
    v, u = _state(1, 2, [[0.7, 0.9]])
    dv = torch.zeros_like(v)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.tp_kick(h, p(dv), p(v), p(u), 0.0) == 0
    assert lib.tp_sync(h) == 0
    assert np.array_equal(dv.cpu().numpy(), [0.0, -9.81, 0.0])
    n, dt = 10, 1e-3
    assert lib.tp_integrate_ck2n54(h, p(v), p(u), 0.0, dt, n) == 0
    assert lib.tp_sync(h) == 0
    t = n * dt
    tol = 1e-12 if precision == 0 else 1e-7  # FP32 form: velocity registers are FP32
    assert np.isclose(u.cpu().numpy()[1], 0.9 - 0.5 * 9.81 * t * t, rtol=0, atol=tol)
    assert np.isclose(v.cpu().numpy()[1], -9.81 * t, rtol=0, atol=tol)
    assert lib.tp_destroy(h) == 0


@pytest.mark.parametrize("bad", ["outside", "nan"])
def test_out_of_grid_and_nonfinite_are_reported(lib, pkg, cuda, bad):
    nf = 40
    rng = np.random.default_rng(0)
    x = rng.uniform(0.2, 1.0, (nf, 2))
    x[7] = [5.0, 0.5] if bad == "outside" else [np.nan, 0.5]
    h, keep = _handle(lib, pkg, _config(pkg, nf, 0))
    v, u = _state(nf, 2, x)
    dv = torch.zeros_like(v)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert lib.tp_kick(h, p(dv), p(v), p(u), 0.0) == 0
    want = 3 if bad == "outside" else 6  # TP_ERR_OUT_OF_GRID / TP_ERR_NONFINITE
    assert lib.tp_sync(h) == want
    assert lib.tp_last_error(h)
    assert lib.tp_sync(h) == 0  # the error word is cleared once reported
    assert lib.tp_destroy(h) == 0


def test_list_capacity_overflow_is_reported(lib, pkg, cuda):
    """Lists fixed for a sparse layout, then integrated on a 144x denser one."""
    nf = 400
    g = np.stack(np.meshgrid(np.arange(20), np.arange(20)), -1).reshape(-1, 2)
    sparse = 0.2 + g * 0.06
    dense = 0.5 + g * 0.005
    h, keep = _handle(lib, pkg, _config(pkg, nf, 0))
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    v, u = _state(nf, 2, sparse)
    assert lib.tp_prepare_lists(h, p(u), ctypes.c_double(1.0)) == 0
    v, u = _state(nf, 2, dense)
    assert lib.tp_integrate_ck2n54(h, p(v), p(u), 0.0, 1e-6, 1) == 0
    assert lib.tp_sync(h) == 7  # TP_ERR_CAPACITY
    assert b"capacity" in lib.tp_last_error(h)
    assert lib.tp_destroy(h) == 0


def test_grid_size_limit(lib, pkg, cuda):
    c = _config(pkg, 10, 10, nd=3, lo=-1000.0, hi=1000.0)
    h = ctypes.c_void_p()
    assert lib.tp_create(ctypes.byref(c), ctypes.byref(h)) == 1
    assert b"2^30" in lib.tp_last_error(None)
