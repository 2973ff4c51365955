"""Batched ensemble of independent 2D dam breaks on the GPU (FP32 precision form).

- A replay of the captured graph (K steps of every spacing group, one branch per group) equals
  the same K steps issued eagerly through tp_integrate_ck2n54, bit for bit: every kernel of the
  integrator is deterministic and the graph holds the same launches.
- Every instance checked agrees with the same instance run alone (its own Semidiscretization):
  the neighbour sets are identical, only the FP32 rounding of shifted coordinates differs.
  Tolerance after K steps: rel L2 <= 1e-9 (x), 1e-4 (v), 1e-6 (rho) -- the precision-form
  tolerances of the single-instance FP32 tests.
- The instance also stays within those tolerances of the FP64 oracle.
- The autotuner only returns shapes from its grid and its choice leaves results unchanged
  within the same tolerances.
"""
import numpy as np
import pytest

from helpers import initial_state, oracle_model, rel_l2

pytestmark = pytest.mark.gpu

K = 20


def _specs(pkg, n=6, seed=3):
    e = pkg.ensemble
    specs = e.ensemble_specs(n, seed=seed)
    for i, s in enumerate(specs):
        s.dx = e.SPACINGS[i % len(e.SPACINGS)]
    return specs


def _eager(pkg, g, steps):
    import torch

    e = pkg.ensemble
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        e.prepare(g, s)
        e._integrate(g, steps)
    s.synchronize()
    g.semi._call("tp_sync")


def _close(a, b, tol_x=1e-9, tol_v=1e-4, tol_rho=1e-6):
    (xa, va, ra), (xb, vb, rb) = a, b
    assert rel_l2(xa, xb) <= tol_x
    assert rel_l2(va, vb) <= tol_v
    assert rel_l2(ra, rb) <= tol_rho


def test_graph_replay_equals_eager(pkg, cuda):
    e = pkg.ensemble
    specs = _specs(pkg)
    groups = e.build_ensemble(specs)
    eg = e.EnsembleGraph(groups, K)
    eg.reset()
    eg.replay()
    cuda.cuda.synchronize()
    eg.check()
    got = [(g.v.cpu().numpy(), g.u.cpu().numpy()) for g in groups]
    for g, (v, u) in zip(e.build_ensemble(specs), got):  # fresh handles, eager launches
        _eager(pkg, g, K)
        assert np.array_equal(g.v.cpu().numpy(), v)
        assert np.array_equal(g.u.cpu().numpy(), u)
        g.semi.close()
    # a second replay from the reset state reproduces the first
    eg.reset()
    eg.replay()
    cuda.cuda.synchronize()
    for g, (v, u) in zip(groups, got):
        assert np.array_equal(g.v.cpu().numpy(), v)
    for g in groups:
        g.semi.close()


def test_instances_match_single_instance_path(pkg, orc, cuda):
    e = pkg.ensemble
    specs = _specs(pkg)
    groups = e.build_ensemble(specs)
    eg = e.EnsembleGraph(groups, K)
    eg.reset()
    eg.replay()
    cuda.cuda.synchronize()
    eg.check()
    for g in groups:
        for j in (0, len(g.instances) - 1):
            spec = specs[g.instances[j]]
            ens = e.instance_state(g, j)
            one = e.single_instance(spec)
            _eager(pkg, one, K)
            alone = e.instance_state(one, 0)
            _close(ens, alone)
            if j == 0 and g.dx >= 0.01:
                tank = one.tanks[0]
                model = oracle_model(orc, one.semi, tank)
                v0, u0 = initial_state(tank)
                v_ref, u_ref, st = model.integrate(v0, u0, e.time_step(g.dx), K)
                assert st == 0
                vr = v_ref.reshape(-1, 3)
                _close(ens, (u_ref.reshape(-1, 2), vr[:, :2], vr[:, 2]), tol_x=1e-8)
            one.semi.close()
    for g in groups:
        g.semi.close()


def test_autotune_choice_keeps_results(pkg, cuda):
    e = pkg.ensemble
    specs = _specs(pkg, n=3, seed=5)
    groups = e.build_ensemble(specs)
    ref = []
    for g in groups:
        _eager(pkg, g, K)
        ref.append([e.instance_state(g, j) for j in range(len(g.instances))])
    choice = e.autotune(groups, trial_steps=2)
    for g in groups:
        c = choice[g.dx]
        assert c["pair_block"] in (64, 128, 256)
        assert c["skin"] in (0.03, 0.05, 0.1, 0.2)
        assert c["pair_mode"] in ("lists", "tiled")
        assert c["pair_mode"] == "lists" or c["pair_block"] == 256
        assert c["ms_per_step"] > 0.0
        _eager(pkg, g, K)
    for g, r in zip(groups, ref):
        for j in range(len(g.instances)):
            _close(e.instance_state(g, j), r[j])
        g.semi.close()


def test_persistent_batch_equals_branches(pkg, cuda):
    """The persistent capture (one pair launch per stage for every group, a work queue of
    256-slot tiles) runs the same per-slot list pass as the branch capture: equal bit for bit."""
    e = pkg.ensemble
    specs = _specs(pkg)
    runs = []
    for persistent in (False, True):
        groups = e.build_ensemble(specs)
        eg = e.EnsembleGraph(groups, K, persistent=persistent)
        eg.reset()
        eg.replay()
        cuda.cuda.synchronize()
        eg.check()
        runs.append([(g.v.cpu().numpy(), g.u.cpu().numpy()) for g in groups])
        eg.close()
        for g in groups:
            g.semi.close()
    for (vb, ub), (vp, up) in zip(*runs):
        assert np.array_equal(vb, vp)
        assert np.array_equal(ub, up)


def test_persistent_mode_rejects_tiled_members(pkg, cuda):
    e = pkg.ensemble
    _abi = pkg._abi
    groups = e.build_ensemble(_specs(pkg, n=3, seed=5))
    b = e.Batch(groups)  # binds the handles
    groups[0].semi._call("tp_set_pair_mode", _abi.TP_PAIR_TILED)
    b.set_mode(True)
    with pytest.raises(_abi.TpError):
        b.capture(2)
    b.set_mode(False)
    b.capture(2)
    b.close()
    for g in groups:
        g.semi.close()


def test_persistent_batch_3d_equals_branches(pkg, cuda):
    """Two 3D FP32 dam breaks of different sizes in one batch: the persistent pair launch (the
    packed 3D list pass over a work queue of both members' tiles) equals the branch capture bit
    for bit, and both equal the eager integrator."""
    from helpers import dam_break_case

    e = pkg.ensemble
    cases = [(0.05, (0.6, 0.4, 0.5), (1.2, 0.8, 0.7)), (0.04, (0.6, 0.32, 0.44), (1.0, 0.6, 0.6))]

    def groups():
        out = []
        for dx, fluid, tank in cases:
            semi, tank_ = dam_break_case(pkg, 3, dx, fluid, tank, precision="float32")
            out.append(e.Group(dx=dx, instances=[0], shifts=[0.0],
                               fluid_ranges=[(0, tank_.fluid.n_particles)], semi=semi,
                               tanks=[tank_]))
        return out

    runs = []
    for persistent in (False, True):
        gs = groups()
        eg = e.EnsembleGraph(gs, 8, persistent=persistent)
        eg.reset()
        eg.replay()
        cuda.cuda.synchronize()
        eg.check()
        runs.append([(g.v.cpu().numpy(), g.u.cpu().numpy()) for g in gs])
        eg.close()
        for g in gs:
            g.semi.close()
    for (vb, ub), (vp, up) in zip(*runs):
        assert np.array_equal(vb, vp)
        assert np.array_equal(ub, up)
    for g, (v, u) in zip(groups(), runs[0]):  # eager launches on fresh handles
        _eager(pkg, g, 8)
        assert np.array_equal(g.v.cpu().numpy(), v)
        assert np.array_equal(g.u.cpu().numpy(), u)
        g.semi.close()
