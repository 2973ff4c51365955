"""tp_cell_sort_noalloc: the neighbour-search cell sort for callers that cannot allocate device
memory (a host whose memory pool owns every device byte, or a fixed-budget real-time loop).

The entry point keeps its scratch in one fixed device array inside the library.  This file is
collected last so that a failure here does not hide the other GPU tests, and it passes both alone
in a fresh process and after the rest of the suite (the shared scratch is cleared per call).
Its output must equal the handle path's (tp_nhs_debug) bit for bit, on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

from helpers import dam_break_case

pytestmark = pytest.mark.gpu


def _noalloc(lib, cfg, u, n, torch, device, out=None):
    if out is None:
        out = (torch.full((n,), -1, dtype=torch.int32, device=device),
               torch.full((n,), -1, dtype=torch.int32, device=device))
    cell, order = out
    stream = torch.cuda.current_stream(device).cuda_stream
    st = lib.tp_cell_sort_noalloc(ctypes.byref(cfg), ctypes.c_void_p(u.data_ptr()), n,
                                  ctypes.c_void_p(cell.data_ptr()),
                                  ctypes.c_void_p(order.data_ptr()), ctypes.c_void_p(stream))
    return st, cell, order


@pytest.mark.parametrize("nd", [2, 3])
def test_noalloc_sort_matches_handle_twice(pkg, lib, cuda, nd):
    torch = cuda
    if nd == 2:
        semi, tank = dam_break_case(pkg, 2, 0.01, (2.0, 1.0), (5.366, 4.0), jitter=0.3, seed=9)
    else:
        semi, tank = dam_break_case(pkg, 3, 0.02, (0.8, 0.4, 0.6), (1.6, 0.8, 1.0), jitter=0.3,
                                    seed=9)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    n = semi.n_fluid
    assert 0 < n <= pkg._abi.TP_NOALLOC_MAX_PARTICLES
    rng = np.random.default_rng(1)
    u_b = ode.u0 + torch.as_tensor(rng.uniform(-0.2, 0.2, n * nd) * tank.fluid.particle_spacing,
                                   device=semi.device)
    refs = []
    for u in (ode.u0, u_b):
        r = semi.nhs_debug(u)
        semi.sync()
        refs.append((r["cell"].clone(), r["order"].clone()))
    outs = [(torch.full((n,), -1, dtype=torch.int32, device=semi.device),
             torch.full((n,), -1, dtype=torch.int32, device=semi.device)) for _ in range(2)]
    torch.cuda.synchronize()
    free = []
    for k, u in enumerate((ode.u0, u_b)):  # two calls in a row, on different coordinates
        free.append(torch.cuda.mem_get_info(semi.device)[0])
        st, cell, order = _noalloc(lib, semi.config, u, n, torch, semi.device, outs[k])
        assert st == 0
        torch.cuda.synchronize()
        assert torch.equal(cell, refs[k][0])
        assert torch.equal(order, refs[k][1])
    free.append(torch.cuda.mem_get_info(semi.device)[0])
    # the second call takes no device memory (the first may load the library's module)
    assert free[2] == free[1]
    semi.close()


def test_noalloc_rejects_oversize_and_reports_out_of_grid(pkg, lib, cuda):
    torch = cuda
    semi, tank = dam_break_case(pkg, 2, 0.05, (1.0, 0.5), (2.0, 1.0))
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    n = semi.n_fluid
    too_many = pkg._abi.TP_NOALLOC_MAX_PARTICLES + 1
    st = lib.tp_cell_sort_noalloc(ctypes.byref(semi.config), ctypes.c_void_p(ode.u0.data_ptr()),
                                  too_many, ctypes.c_void_p(ode.u0.data_ptr()),
                                  ctypes.c_void_p(ode.u0.data_ptr()), None)
    assert st == pkg._abi.TP_ERR_CAPACITY
    u = ode.u0.clone()
    u[0] = 1.0e3
    st, cell, order = _noalloc(lib, semi.config, u, n, torch, semi.device)
    assert st == pkg._abi.TP_ERR_OUT_OF_GRID
    st, cell, order = _noalloc(lib, semi.config, ode.u0, n, torch, semi.device)
    assert st == 0  # the error word is cleared per call
    semi.close()


def _grid_cells(cfg, nd):
    """Cell count of the grid that tp_create / tp_cell_sort_noalloc lay over cfg's corners."""
    import math

    cs = 2.0 * cfg.smoothing_length
    total = 1
    for d in range(nd):
        lo = math.floor(cfg.min_corner[d] / cs) - 1
        hi = math.floor(cfg.max_corner[d] / cs) + 1
        total *= hi - lo + 1
    return total


def test_noalloc_rejects_too_many_cells(pkg, lib, cuda):
    """A grid one cell row beyond TP_NOALLOC_MAX_CELLS is refused before any GPU work."""
    torch = cuda
    semi, tank = dam_break_case(pkg, 2, 0.05, (1.0, 0.5), (2.0, 1.0))
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    cfg = type(semi.config).from_buffer_copy(semi.config)
    cs = 2.0 * cfg.smoothing_length
    cfg.min_corner[0] = cfg.min_corner[1] = 0.0
    cfg.max_corner[0] = 509.5 * cs   # 512 cells along x (one padding cell each side)
    cfg.max_corner[1] = 1022.5 * cs  # 1025 cells along y
    assert _grid_cells(cfg, 2) == pkg._abi.TP_NOALLOC_MAX_CELLS + 512
    st, cell, order = _noalloc(lib, cfg, ode.u0, semi.n_fluid, torch, semi.device)
    assert st == pkg._abi.TP_ERR_CAPACITY
    assert bool((cell == -1).all()) and bool((order == -1).all())  # nothing was written
    semi.close()


def test_noalloc_grid_at_cell_limit_matches_handle(pkg, lib, cuda):
    """A grid of exactly TP_NOALLOC_MAX_CELLS cells (the cell starts then end at the last slot
    before the scan partials of the fixed array) sorts as the handle path does."""
    import math

    torch = cuda
    semi, tank = dam_break_case(pkg, 2, 0.05, (1.0, 0.5), (2.0, 1.0), jitter=0.3, seed=4)
    cfg = semi.config
    cs = 2.0 * cfg.smoothing_length
    # keep the tank's min corner (walls must lie inside the box) and widen the box to 512 x 1024
    # cells: n = floor(max / cs) - floor(min / cs) + 3 along each axis
    for d, n in ((0, 512), (1, 1024)):
        cfg.max_corner[d] = (math.floor(cfg.min_corner[d] / cs) + n - 3 + 0.5) * cs
    assert _grid_cells(cfg, 2) == pkg._abi.TP_NOALLOC_MAX_CELLS
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    u = ode.u0
    r = semi.nhs_debug(u)
    semi.sync()
    ref_cell, ref_order = r["cell"].clone(), r["order"].clone()
    for _ in range(2):
        st, cell, order = _noalloc(lib, semi.config, u, semi.n_fluid, torch, semi.device)
        assert st == 0
        torch.cuda.synchronize()
        assert torch.equal(cell, ref_cell)
        assert torch.equal(order, ref_order)
    semi.close()
