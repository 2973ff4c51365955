"""The oracle against the reference's own known-answer tests (CPU)."""
import math

import numpy as np
import pytest


def test_monaghan_viscosity_golden(orc):
    # test/schemes/fluid/viscosity.jl:1-42: SchoenbergCubicSplineKernel{2}, h = 1.2 * 0.2,
    # c = 10 sqrt(9.81 * 0.9), alpha = 0.02, beta = 0, explicit pos_diff / v_diff.
    h = 1.2 * 0.2
    c = 10 * math.sqrt(9.81 * 0.9)
    pd = [-0.25 * h, 0.375 * h]
    dv = orc.monaghan_pair(2, h, c, 0.02, 0.0, 0.01, pd, [0.3, -1.0], [0.0, 0.0], 1.0,
                           1000.0, 1000.0)
    assert dv[0] == pytest.approx(-0.02049217623299368, abs=6e-15)
    assert dv[1] == pytest.approx(0.03073826434949052, abs=6e-15)


ATM = 101_325.0


@pytest.mark.parametrize("gamma,golden", [
    # test/schemes/fluid/weakly_compressible_sph/state_equation.jl:24-37 (exact equality there)
    (7.15, [(1, 998.34), (100, 1002.8323123356663), (500, 1019.8235062499685),
            (1000, 1038.8747989986027), (3000, 1099.0607413267035), (9000, 1210.4689472510186)]),
    # :84-97 (linear Cole EOS)
    (1.0, [(1, 998.34), (100, 1002.8949541016121), (500, 1021.298809057621),
           (1000, 1044.3036277526319), (3000, 1136.3229025326757), (9000, 1412.380726872807)]),
])
def test_cole_inverse_golden(orc, pkg, gamma, golden):
    # the oracle's and the host setup's state equation (used for the hydrostatic initial state)
    eos = pkg.StateEquationCole(sound_speed=1484.0, reference_density=998.34, exponent=gamma,
                                background_pressure=1 * ATM)
    for p_atm, rho in golden:
        assert orc.cole_inverse(1484.0, 998.34, gamma, 1 * ATM, p_atm * ATM) == rho
        assert eos.inverse(p_atm * ATM) == rho


@pytest.mark.parametrize("c,gamma,p_bg", [(1484.0, 7.15, 101_325.0), (10.0, 7.0, 10_000.0),
                                          (10.0, 7.0, 0.0), (10.0, 7.0, -100_000.0),
                                          (10.0, 1.0, 100_000.0), (10.0, 1.0, 0.0)])
def test_cole_roundtrip(orc, c, gamma, p_bg):
    # state_equation.jl:103-139: inverse(EOS(rho)) ~ rho and EOS(inverse(p)) ~ p.
    rho0 = 998.34 if c == 1484.0 else 1000.0
    for rho in [100.0, 500.0, 900.0, 990.0, 1000.0, 1005.0, 1100.0, 1600.0]:
        p = orc.cole_pressure(c, rho0, gamma, p_bg, 0, rho)
        # Julia `≈`: rtol = sqrt(eps)
        assert orc.cole_inverse(c, rho0, gamma, p_bg, p) == pytest.approx(rho, rel=1.5e-8)
    for p in [-100.0, 0.0, 100.0, 10_000.0, 100_000.0, 100_000_000.0]:
        rho = orc.cole_inverse(c, rho0, gamma, p_bg, p)
        if math.isnan(rho):
            continue
        assert orc.cole_pressure(c, rho0, gamma, p_bg, 0, rho) == pytest.approx(p, abs=2e-7,
                                                                                rel=1e-10)


def test_cole_clipping(orc):
    # state_equation.jl:41-61
    assert orc.cole_pressure(10.0, 1000.0, 7.0, 0.0, 1, 999.0) == 0.0
    assert orc.cole_pressure(10.0, 1000.0, 7.0, 0.0, 1, 900.0) == 0.0
    for p_bg in [0.0, 10_000.0, 100_000.0, 200_000.0]:
        assert orc.cole_pressure(10.0, 1000.0, 7.0, p_bg, 0, 1000.0) == p_bg
        assert orc.cole_pressure(10.0, 1000.0, 7.0, p_bg, 0, 1001.0) > p_bg + 10
        assert orc.cole_pressure(10.0, 1000.0, 7.0, p_bg, 0, 999.0) < p_bg - 10


@pytest.mark.parametrize("nd", [2, 3])
def test_wendland_normalisation(orc, nd):
    # test/general/smoothing_kernels.jl:3-74: integral of W over the support is 1.
    h = 0.7
    r = np.linspace(0.0, 2 * h, 20001)
    w = np.array([orc.wendland_c2(nd, x, h) for x in r])
    shell = 2 * math.pi * r if nd == 2 else 4 * math.pi * r * r
    integral = np.trapezoid(w * shell, r)
    assert integral == pytest.approx(1.0, abs=1e-8)


@pytest.mark.parametrize("nd", [2, 3])
def test_wendland_derivative(orc, nd):
    # smoothing_kernels.jl:77-133: analytic derivative vs a numerical one.
    h = 0.3
    for r in np.linspace(0.01, 2 * h - 0.01, 37):
        eps = 1e-6
        num = (orc.wendland_c2(nd, r + eps, h) - orc.wendland_c2(nd, r - eps, h)) / (2 * eps)
        ana = orc.wendland_c2_deriv_div_r(nd, r, h) * r
        assert ana == pytest.approx(num, rel=1e-7, abs=1e-9)
    assert orc.wendland_c2(nd, 2 * h, h) == 0.0


def test_ck2n54_coefficients(orc):
    # Carpenter & Kennedy (1994) 2N scheme: the abscissae follow from A and B
    # (c_i = sum of the effective Butcher weights), and the weights of the final stage sum to 1.
    A, B, C = orc.ck2n54_coefficients()
    # effective Butcher tableau of a 2N scheme: b_j = sum_{i>=j} B_i prod_{k=j+1..i} A_k
    s = 5
    b = np.zeros(s)
    for j in range(s):
        acc = 0.0
        for i in range(j, s):
            prod = 1.0
            for k in range(j + 1, i + 1):
                prod *= A[k]
            acc += B[i] * prod
        b[j] = acc
    assert b.sum() == pytest.approx(1.0, abs=1e-12)
    # c_i = sum_{j<i} a_ij with a_ij built the same way from stages j..i-1
    for i in range(1, s):
        ci = 0.0
        for j in range(i):
            acc = 0.0
            for m in range(j, i):
                prod = 1.0
                for k in range(j + 1, m + 1):
                    prod *= A[k]
                acc += B[m] * prod
            ci += acc
        assert ci == pytest.approx(C[i], abs=1e-12)
