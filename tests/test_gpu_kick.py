"""kick!/drift! on the GPU against the FP64 oracle.

Tolerances: the FP64 drop-in differs from the CPU oracle only by FMA contraction in the pair
sums, the Cole EOS power by repeated multiplication and its inverse by Newton's method, the
reference's CUDA `div_fast` (relative error < 1e-15
per division, ext/TrixiParticlesCUDAExt.jl), ulp-level rearrangements of reciprocals and square
roots, and -- in the symmetric pair mode -- the summation order: relative L2 error of
dv <= 1e-11 in both pair modes; the gather mode is bitwise reproducible.  The FP32
precision form is held to 2e-5 relative L2 on the velocity rows and 1e-4 on the density rate.
"""
import numpy as np
import pytest

from helpers import dam_break_case, initial_state, oracle_model, rel_l2

pytestmark = pytest.mark.gpu

CASES = [
    dict(ndims=2, dx=0.02, fluid=(2.0, 1.0), tank=(5.366, 4.0), jitter=0.0, vel=0.0),
    dict(ndims=2, dx=0.02, fluid=(2.0, 1.0), tank=(5.366, 4.0), jitter=0.2, vel=0.5),
    dict(ndims=3, dx=0.05, fluid=(1.0, 0.5, 1.0), tank=(3.2, 1.0, 1.4), jitter=0.2, vel=0.5),
]


def _state(tank, case, seed=11):
    v, u = initial_state(tank)
    if case["vel"]:
        rng = np.random.default_rng(seed)
        nd = tank.fluid.ndims
        v[:, :nd] = rng.normal(0.0, case["vel"], (v.shape[0], nd))
        v[:, nd] *= 1.0 + rng.uniform(-1e-3, 1e-3, v.shape[0])
    return v, u


def _run(pkg, orc, cuda, case, precision, pair_mode=None):
    torch = cuda
    semi, tank = dam_break_case(pkg, case["ndims"], case["dx"], case["fluid"], case["tank"],
                                jitter=case["jitter"], seed=5, precision=precision)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    if pair_mode is not None:
        semi._call("tp_set_pair_mode", pair_mode)
    v, u = _state(tank, case)
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    u_t = torch.as_tensor(u.ravel(), device=semi.device)
    dv = torch.full_like(v_t, float("nan"))
    pkg.kick(dv, v_t, u_t, ode.p, 0.0)
    p_f = semi.fluid_pressure()
    p_w, rho_w, vol_w = semi.wall_state()
    semi.sync()
    model = oracle_model(orc, semi, tank)
    dv_ref, st = model.kick(v, u)
    assert st == 0
    ref = model.last_state()
    out = dict(dv=dv.cpu().numpy(), p_f=p_f.cpu().numpy(), p_w=p_w.cpu().numpy(),
               rho_w=rho_w.cpu().numpy(), vol_w=vol_w.cpu().numpy())
    semi.close()
    return out, dv_ref, ref, case["ndims"]


@pytest.mark.parametrize("mode", [0, 1], ids=["gather", "symmetric"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['ndims']}d-j{c['jitter']}-v{c['vel']}")
def test_kick_fp64_matches_oracle(pkg, orc, cuda, case, mode):
    out, dv_ref, ref, nd = _run(pkg, orc, cuda, case, "float64", pair_mode=mode)
    assert np.all(np.isfinite(out["dv"]))
    assert rel_l2(out["dv"], dv_ref) <= 1e-11
    g = out["dv"].reshape(-1, nd + 1)
    r = dv_ref.reshape(-1, nd + 1)
    assert rel_l2(g[:, nd], r[:, nd]) <= 1e-9 or np.abs(g[:, nd] - r[:, nd]).max() < 1e-9
    assert rel_l2(out["p_f"], ref["p_f"]) <= 1e-13
    assert rel_l2(out["p_w"], ref["p_w"]) <= 1e-12
    assert rel_l2(out["rho_w"], ref["rho_w"]) <= 1e-14
    assert rel_l2(out["vol_w"], ref["vol_w"]) <= 1e-14
    # walls without fluid neighbours keep p = 0 and rho = rho0 exactly
    lone = ref["vol_w"] == 0.0
    assert lone.any()
    assert np.all(out["p_w"][lone] == 0.0)


@pytest.mark.parametrize("mode", [0, 2], ids=["lists", "tiled"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['ndims']}d-j{c['jitter']}-v{c['vel']}")
def test_kick_fp32_form_matches_oracle(pkg, orc, cuda, case, mode):
    out, dv_ref, ref, nd = _run(pkg, orc, cuda, case, "float32", pair_mode=mode)
    g = out["dv"].reshape(-1, nd + 1)
    r = dv_ref.reshape(-1, nd + 1)
    assert rel_l2(g[:, :nd], r[:, :nd]) <= 2e-5
    drho_scale = max(np.abs(r[:, nd]).max(), 1.0)
    assert np.abs(g[:, nd] - r[:, nd]).max() <= 1e-4 * drho_scale
    assert rel_l2(out["p_w"], ref["p_w"]) <= 1e-5


FULL = dict(ndims=3, dx=0.008, fluid=(1.0, 0.5, 1.0), tank=(3.2, 1.0, 1.4), jitter=0.2, vel=0.5)


@pytest.mark.parametrize("precision,mode", [("float64", 0), ("float32", 0), ("float32", 2)],
                         ids=["fp64", "fp32-lists", "fp32-tiled"])
def test_kick_full_3d_workload(pkg, orc, cuda, precision, mode):
    """One right-hand side of the full 3D benchmark workload (968 750 fluid + 876 666 wall
    particles, jittered, random velocities) against the oracle."""
    out, dv_ref, ref, nd = _run(pkg, orc, cuda, FULL, precision, pair_mode=mode)
    g = out["dv"].reshape(-1, nd + 1)
    r = dv_ref.reshape(-1, nd + 1)
    if precision == "float64":
        assert rel_l2(out["dv"], dv_ref) <= 1e-11
        assert rel_l2(out["p_w"], ref["p_w"]) <= 1e-12
    else:
        assert rel_l2(g[:, :nd], r[:, :nd]) <= 2e-5
        assert np.abs(g[:, nd] - r[:, nd]).max() <= 1e-4 * max(np.abs(r[:, nd]).max(), 1.0)


def test_drift_copies_velocity(pkg, cuda):
    # test/general/semidiscretization.jl:608-631
    torch = cuda
    semi, tank = dam_break_case(pkg, 3, 0.1, (0.5, 0.3, 0.4), (1.0, 0.6, 0.6))
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v = torch.randn_like(ode.v0)
    du = torch.full_like(ode.u0, float("nan"))
    pkg.drift(du, v, ode.u0, ode.p, 0.0)
    semi.sync()
    assert torch.equal(du.view(-1, 3), v.view(-1, 4)[:, :3])
    semi.close()


def test_fluid_momentum_conservation(pkg, orc, cuda):
    # test/schemes/fluid/rhs.jl:115-264: without walls and gravity the pair terms conserve
    # linear momentum: sum_a m_a dv_a = 0 to rounding.
    torch = cuda
    rng = np.random.default_rng(2)
    nd, dx = 3, 0.1
    n = 6
    g = np.stack(np.meshgrid(*[np.arange(n)] * nd, indexing="ij"), -1).reshape(-1, nd)
    x = (g + 0.5) * dx + rng.uniform(-0.3 * dx, 0.3 * dx, g.shape)
    rho = 1000.0 * (1 + rng.uniform(-0.01, 0.01, len(x)))
    m = dx ** 3 * rho
    v = np.zeros((len(x), nd + 1))
    v[:, :nd] = rng.normal(0, 0.3, (len(x), nd))
    v[:, nd] = rho
    eos = pkg.StateEquationCole(sound_speed=20.0, reference_density=1000.0, exponent=7.0)
    ic = pkg.InitialCondition(x, v[:, :nd], m, rho, np.zeros(len(x)), dx)
    wic = pkg.InitialCondition(np.zeros((0, nd)), np.zeros((0, nd)), np.zeros(0), np.zeros(0),
                               np.zeros(0), dx)
    k = pkg.WendlandC2Kernel(nd)
    fluid = pkg.WeaklyCompressibleSPHSystem(
        ic, smoothing_kernel=k, smoothing_length=1.2 * dx, density_calculator=pkg.ContinuityDensity(),
        state_equation=eos, acceleration=(0.0,) * nd,
        viscosity=pkg.ArtificialViscosityMonaghan(alpha=0.02),
        density_diffusion=pkg.DensityDiffusionMolteniColagrossi(delta=0.1))
    wall = pkg.WallBoundarySystem(wic, pkg.BoundaryModelDummyParticles(
        np.zeros(0), np.zeros(0), pkg.AdamiPressureExtrapolation(), k, 1.2 * dx,
        state_equation=eos))
    cl = pkg.FullGridCellList(tuple(x.min(0) - dx), tuple(x.max(0) + dx))
    semi = pkg.Semidiscretization(fluid, wall, neighborhood_search=pkg.GridNeighborhoodSearch(nd, cl),
                                  parallelization_backend=pkg.GB300Backend())
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    dv = torch.zeros_like(v_t)
    pkg.kick(dv, v_t, ode.u0, ode.p, 0.0)
    semi.sync()
    a = dv.cpu().numpy().reshape(-1, nd + 1)[:, :nd]
    mom = (m[:, None] * a).sum(0)
    scale = (m[:, None] * np.abs(a)).sum()
    assert np.all(np.abs(mom) <= 1e-13 * scale)
    semi.close()


def test_kick_fp64_gather_mode_is_reproducible(pkg, orc, cuda):
    case = CASES[1]
    a, _, _, _ = _run(pkg, orc, cuda, case, "float64", pair_mode=0)
    b, _, _, _ = _run(pkg, orc, cuda, case, "float64", pair_mode=0)
    assert np.array_equal(a["dv"], b["dv"])


def test_pair_mode_argument_check(pkg, cuda):
    case = CASES[0]
    for precision, bad in (("float64", (7, 2)), ("float32", (7, 1))):
        semi, _ = dam_break_case(pkg, case["ndims"], case["dx"], case["fluid"], case["tank"],
                                 precision=precision)
        pkg.semidiscretize(semi, (0.0, 1.0))
        for mode in bad:  # the tiled pass is an FP32 mode, the symmetric one an FP64 mode
            with pytest.raises(pkg.TpError):
                semi._call("tp_set_pair_mode", mode)
        semi.close()


def test_fp32_modes_switch_back_and_forth(pkg, orc, cuda):
    """Switching an FP32 handle between the list and the tiled pass between kicks hands the
    lists back: every kick matches the oracle."""
    torch = cuda
    case = CASES[1]
    semi, tank = dam_break_case(pkg, case["ndims"], case["dx"], case["fluid"], case["tank"],
                                jitter=case["jitter"], seed=5, precision="float32")
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v, u = _state(tank, case)
    model = oracle_model(orc, semi, tank)
    dv_ref, st = model.kick(v, u)
    assert st == 0
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    u_t = torch.as_tensor(u.ravel(), device=semi.device)
    nd = case["ndims"]
    r = dv_ref.reshape(-1, nd + 1)
    for mode in (0, 2, 0, 2):
        semi._call("tp_set_pair_mode", mode)
        dv = torch.full_like(v_t, float("nan"))
        pkg.kick(dv, v_t, u_t, ode.p, 0.0)
        semi.sync()
        g = dv.cpu().numpy().reshape(-1, nd + 1)
        assert rel_l2(g[:, :nd], r[:, :nd]) <= 2e-5
    semi.close()


@pytest.mark.parametrize("switches", [dict(beta=0.5), dict(delta=None), dict(beta=0.5, delta=None)],
                         ids=["beta", "no-diffusion", "beta-no-diffusion"])
def test_kick_fp32_model_switches_match_oracle(pkg, orc, cuda, switches):
    """The FP32 list pass outside the dam-break configuration (Monaghan beta != 0, no density
    diffusion: the kernels' general path, in 3D through the packed two-candidate evaluation)
    against the oracle, with the FP32 form's tolerances."""
    torch = cuda
    case = CASES[2]
    semi, tank = dam_break_case(pkg, case["ndims"], case["dx"], case["fluid"], case["tank"],
                                jitter=case["jitter"], seed=5, precision="float32", **switches)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v, u = _state(tank, case)
    v_t = torch.as_tensor(v.ravel(), device=semi.device)
    u_t = torch.as_tensor(u.ravel(), device=semi.device)
    dv = torch.full_like(v_t, float("nan"))
    pkg.kick(dv, v_t, u_t, ode.p, 0.0)
    semi.sync()
    model = oracle_model(orc, semi, tank)
    dv_ref, st = model.kick(v, u)
    assert st == 0
    nd = case["ndims"]
    g = dv.cpu().numpy().reshape(-1, nd + 1)
    r = dv_ref.reshape(-1, nd + 1)
    assert np.all(np.isfinite(g))
    assert rel_l2(g[:, :nd], r[:, :nd]) <= 2e-5
    assert rel_l2(g[:, nd], r[:, nd]) <= 1e-4
    semi.close()
