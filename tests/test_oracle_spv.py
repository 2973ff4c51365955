"""The oracle's SymplecticPositionVerlet (CPU): second-order convergence and agreement with the
fourth-order CarpenterKennedy2N54 on a short 2D dam-break interval."""
import numpy as np

from helpers import dam_break_case, initial_state, oracle_model, rel_l2


def _run(model, v0, u0, T, n, spv=True):
    f = model.integrate_spv if spv else model.integrate
    v, u, st = f(v0, u0, T / n, n)
    assert st == 0
    return v, u


def test_spv_second_order_and_consistency(pkg, orc):
    semi, tank = dam_break_case(pkg, 2, 0.05, (1.0, 0.5), (2.0, 1.0), jitter=0.1, seed=2)
    model = oracle_model(orc, semi, tank)
    v0, u0 = initial_state(tank)
    rng = np.random.default_rng(4)
    v0[:, :2] = rng.normal(0.0, 0.05, (v0.shape[0], 2))
    T = 4e-3
    ref_v, ref_u = _run(model, v0, u0, T, 64, spv=False)  # CK2N54, 4th order: the reference
    errs = []
    for n in (4, 8, 16):
        v, u = _run(model, v0, u0, T, n)
        errs.append(rel_l2(v.reshape(-1, 3)[:, :2], ref_v.reshape(-1, 3)[:, :2]))
    assert errs[0] / errs[1] > 3.0 and errs[1] / errs[2] > 3.0  # ~4 for second order
    v, u = _run(model, v0, u0, T, 16)
    assert rel_l2(u, ref_u) < 1e-6
    assert rel_l2(v.reshape(-1, 3)[:, 2], ref_v.reshape(-1, 3)[:, 2]) < 2e-5
