"""Differentiation form on the GPU: the hand-written adjoint against central finite differences.

Objective: the mean final height of the particles of the fluid's initial top layer
(adjoint.surface_height_loss), after n CarpenterKennedy2N54 steps of a 2D dam break from a
seeded random initial velocity field v0 ~ N(0, 0.1^2) m/s per component.  Gradients with
respect to Monaghan alpha, Molteni-Colagrossi delta, gravity magnitude and v0 (a seeded random
direction) are compared with central differences of the same objective computed through the
library's own fused integrator (tp_integrate_ck2n54) in FP64:
  * FP64 adjoint, dx = 0.02, 40 steps, checkpoints every 10: relative error <= 1e-5;
  * FP32 adjoint, dx = 0.01 (20 000 fluid particles), 500 steps, checkpoints every 25, FD step
    h = 1e-4: relative error <= 1e-3;
  * FP64 adjoint on the 2000-particle variant (dx = 0.0316) against central differences through
    the FP64 CPU oracle: relative error <= 1e-5, and against forward-mode derivatives through
    the oracle (dual numbers, the counterpart of ForwardDiff): relative error <= 1e-8;
  * gradients do not depend on the checkpoint interval (FP64, relative 1e-10).
The adjoint's forward agrees with the fused integrator (FP64: v within 1e-9, u within 1e-12
relative L2; FP32: the precision-form tolerances).
"""
import numpy as np
import pytest

from helpers import oracle_model, rel_l2

pytestmark = pytest.mark.gpu

FLUID, TANK = (2.0, 1.0), (5.366, 4.0)


def _tank(pkg, dx):
    return pkg.dam_break(2, dx, FLUID, TANK, n_layers=3)


def _semi(pkg, tank, eos, dx, precision, alpha=0.02, delta=0.1, gravity=9.81):
    return pkg.dam_break_semidiscretization(tank, eos, 1.75 * dx, precision=precision,
                                            alpha=alpha, delta=delta, gravity=gravity)


def _initial(tank, seed=7, sigma=0.1):
    rng = np.random.default_rng(seed)
    n = tank.fluid.n_particles
    v = np.zeros((n, 3))
    v[:, :2] = rng.normal(0.0, sigma, (n, 2))
    v[:, 2] = tank.fluid.density
    return v, tank.fluid.coordinates.copy()


def _dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a).reshape(-1), device="cuda")


def _loss_fd(pkg, torch, tank, eos, dx, v0, u0, dt, n, idx, **params):
    """Objective through the fused FP64 integrator (the product forward path)."""
    semi = _semi(pkg, tank, eos, dx, "float64", **params)
    ode = pkg.semidiscretize(semi, (0.0, n * dt))
    ode.v0.copy_(_dev(torch, v0))
    ode.u0.copy_(_dev(torch, u0))
    sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=n)
    u = sol.u.view(-1, 2).cpu().numpy()
    semi.close()
    return float(u[idx, 1].mean())


def _adjoint(pkg, torch, tank, eos, dx, precision, v0, u0, dt, n, k, idx, **params):
    semi = _semi(pkg, tank, eos, dx, precision, **params)
    pkg.semidiscretize(semi, (0.0, n * dt))
    traj = pkg.adjoint.Trajectory(semi, _dev(torch, v0), _dev(torch, u0), dt=dt, n_steps=n,
                                  checkpoint_every=k)
    loss, ubar = pkg.adjoint.surface_height_loss(traj.u, idx, 2)
    vbar = torch.zeros_like(traj.v)
    vb, ub, pbar = traj.pullback(vbar, ubar)
    out = (float(loss), vb.view(-1, 3).cpu().numpy(), ub.view(-1, 2).cpu().numpy(), pbar,
           traj.v.view(-1, 3).cpu().numpy(), traj.u.view(-1, 2).cpu().numpy())
    semi.close()
    return out


def _fd_all(pkg, torch, tank, eos, dx, v0, u0, dt, n, idx, h, w):
    base = dict(alpha=0.02, delta=0.1, gravity=9.81)
    fd = {}
    for name in ("alpha", "delta", "gravity"):
        hi = dict(base, **{name: base[name] + h})
        lo = dict(base, **{name: base[name] - h})
        fd[name] = (_loss_fd(pkg, torch, tank, eos, dx, v0, u0, dt, n, idx, **hi)
                    - _loss_fd(pkg, torch, tank, eos, dx, v0, u0, dt, n, idx, **lo)) / (2 * h)
    vp, vm = v0.copy(), v0.copy()
    vp[:, :2] += h * w
    vm[:, :2] -= h * w
    fd["v0"] = (_loss_fd(pkg, torch, tank, eos, dx, vp, u0, dt, n, idx, **base)
                - _loss_fd(pkg, torch, tank, eos, dx, vm, u0, dt, n, idx, **base)) / (2 * h)
    return fd


def _compare(grad, fd, tol):
    for name, ref in fd.items():
        err = abs(grad[name] - ref) / max(abs(ref), 1e-300)
        assert err <= tol, (name, grad[name], ref, err)


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_adjoint_forward_matches_integrator(pkg, cuda, precision):
    torch = cuda
    dx, dt, n = 0.02, 1e-4, 40
    tank, eos = _tank(pkg, dx)
    v0, u0 = _initial(tank)
    idx = pkg.adjoint.top_layer_indices(tank)
    _, _, _, _, v_adj, u_adj = _adjoint(pkg, torch, tank, eos, dx, precision, v0, u0, dt, n, 10,
                                        idx)
    semi = _semi(pkg, tank, eos, dx, precision)
    ode = pkg.semidiscretize(semi, (0.0, n * dt))
    ode.v0.copy_(_dev(torch, v0))
    sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=n)
    v = sol.v.view(-1, 3).cpu().numpy()
    u = sol.u.view(-1, 2).cpu().numpy()
    semi.close()
    if precision == "float64":
        assert rel_l2(u_adj, u) <= 1e-12
        assert rel_l2(v_adj[:, :2], v[:, :2]) <= 1e-9
        assert rel_l2(v_adj[:, 2], v[:, 2]) <= 1e-12
    else:
        assert rel_l2(u_adj, u) <= 1e-8
        assert rel_l2(v_adj[:, :2], v[:, :2]) <= 1e-4
        assert rel_l2(v_adj[:, 2], v[:, 2]) <= 1e-6


def test_adjoint_fp64_against_finite_differences(pkg, cuda):
    torch = cuda
    dx, dt, n, k = 0.02, 1e-4, 40, 10
    tank, eos = _tank(pkg, dx)
    v0, u0 = _initial(tank)
    idx = pkg.adjoint.top_layer_indices(tank)
    w = np.random.default_rng(11).normal(size=(tank.fluid.n_particles, 2))
    loss, vb, ub, pbar, _, _ = _adjoint(pkg, torch, tank, eos, dx, "float64", v0, u0, dt, n, k,
                                        idx)
    grad = dict(pbar, v0=float((vb[:, :2] * w).sum()))
    fd = _fd_all(pkg, torch, tank, eos, dx, v0, u0, dt, n, idx, 1e-5, w)
    _compare(grad, fd, 1e-5)


def test_adjoint_checkpoint_interval_invariance(pkg, cuda):
    torch = cuda
    dx, dt, n = 0.02, 1e-4, 30
    tank, eos = _tank(pkg, dx)
    v0, u0 = _initial(tank)
    idx = pkg.adjoint.top_layer_indices(tank)
    res = [_adjoint(pkg, torch, tank, eos, dx, "float64", v0, u0, dt, n, k, idx)
           for k in (1, 7, 30)]
    for r in res[1:]:
        assert rel_l2(r[1], res[0][1]) <= 1e-10
        assert rel_l2(r[2], res[0][2]) <= 1e-10
        for name in ("alpha", "delta", "gravity"):
            assert abs(r[3][name] - res[0][3][name]) <= 1e-10 * abs(res[0][3][name])


def test_adjoint_fp32_differentiated_dam_break(pkg, cuda):
    """The differentiated 2D dam break: dx = 0.01 (20 000 fluid), 500 steps, checkpoints every
    25, FP32 forward and adjoint, FP64 parameter reduction; FD step h = 1e-4."""
    torch = cuda
    dx, dt, n, k = 0.01, 5e-5, 500, 25
    tank, eos = _tank(pkg, dx)
    assert tank.fluid.n_particles == 20000
    v0, u0 = _initial(tank)
    idx = pkg.adjoint.top_layer_indices(tank)
    w = np.random.default_rng(11).normal(size=(tank.fluid.n_particles, 2))
    loss, vb, ub, pbar, _, _ = _adjoint(pkg, torch, tank, eos, dx, "float32", v0, u0, dt, n, k,
                                        idx)
    grad = dict(pbar, v0=float((vb[:, :2] * w).sum()))
    fd = _fd_all(pkg, torch, tank, eos, dx, v0, u0, dt, n, idx, 1e-4, w)
    _compare(grad, fd, 1e-3)


def test_adjoint_against_oracle_finite_differences(pkg, orc, cuda):
    """2000-particle variant (dx = 0.0316): FP64 adjoint vs central differences through the
    FP64 CPU oracle."""
    torch = cuda
    dx, n, k = 0.0316, 60, 20
    dt = 5e-3 * dx
    tank, eos = _tank(pkg, dx)
    assert abs(tank.fluid.n_particles - 2000) < 100
    v0, u0 = _initial(tank)
    idx = pkg.adjoint.top_layer_indices(tank)
    w = np.random.default_rng(11).normal(size=(tank.fluid.n_particles, 2))
    loss, vb, ub, pbar, _, _ = _adjoint(pkg, torch, tank, eos, dx, "float64", v0, u0, dt, n, k,
                                        idx)
    grad = dict(pbar, v0=float((vb[:, :2] * w).sum()))

    def oracle_loss(v, **params):
        semi = _semi(pkg, tank, eos, dx, "float64", **params)
        model = oracle_model(orc, semi, tank)
        _, uu, st = model.integrate(v.copy(), u0.copy(), dt, n)
        assert st == 0
        return float(uu.reshape(-1, 2)[idx, 1].mean())

    h = 1e-5
    base = dict(alpha=0.02, delta=0.1, gravity=9.81)
    fd = {}
    for name in ("alpha", "delta", "gravity"):
        fd[name] = (oracle_loss(v0, **dict(base, **{name: base[name] + h}))
                    - oracle_loss(v0, **dict(base, **{name: base[name] - h}))) / (2 * h)
    vp, vm = v0.copy(), v0.copy()
    vp[:, :2] += h * w
    vm[:, :2] -= h * w
    fd["v0"] = (oracle_loss(vp, **base) - oracle_loss(vm, **base)) / (2 * h)
    assert abs(loss - oracle_loss(v0, **base)) <= 1e-12
    _compare(grad, fd, 1e-5)


def test_adjoint_against_oracle_forward_mode(pkg, orc, cuda):
    """2000-particle variant (dx = 0.0316): FP64 adjoint vs forward-mode derivatives through the
    FP64 CPU oracle (dual numbers carried through the oracle's right-hand side and CK2N54 steps,
    the counterpart of a ForwardDiff gradient through the reference's CPU path).  Both are exact
    derivatives of the same discrete map up to rounding: relative error <= 1e-8 for alpha, delta,
    |g| and the v0 direction."""
    torch = cuda
    dx, n, k = 0.0316, 60, 20
    dt = 5e-3 * dx
    tank, eos = _tank(pkg, dx)
    v0, u0 = _initial(tank)
    idx = pkg.adjoint.top_layer_indices(tank)
    w = np.random.default_rng(11).normal(size=(tank.fluid.n_particles, 2))
    loss, vb, ub, pbar, _, _ = _adjoint(pkg, torch, tank, eos, dx, "float64", v0, u0, dt, n, k,
                                        idx)
    grad = dict(pbar, v0=float((vb[:, :2] * w).sum()))
    semi = _semi(pkg, tank, eos, dx, "float64")
    vdir = np.zeros_like(v0)
    vdir[:, :2] = w
    _, uu, dv, du, st = orc.integrate_jvp(semi.config, tank.boundary.coordinates,
                                          tank.boundary.mass, tank.fluid.mass, v0, u0, dt, n,
                                          v_dir=vdir)
    assert st == 0
    assert abs(loss - float(uu.reshape(-1, 2)[idx, 1].mean())) <= 1e-12
    fwd = {name: float(du[kk].reshape(-1, 2)[idx, 1].mean())
           for kk, name in enumerate(("alpha", "delta", "gravity", "v0"))}
    print(f"\nADJOINT vs forward mode: " + ", ".join(
        f"{k_}: {grad[k_]:.9e} / {fwd[k_]:.9e} (rel {abs(grad[k_] - fwd[k_]) / abs(fwd[k_]):.2e})"
        for k_ in fwd))
    _compare(grad, fwd, 1e-8)
