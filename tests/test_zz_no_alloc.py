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
