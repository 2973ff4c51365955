"""The oracle against the reference's GPU interpolation goldens (test/examples/gpu.jl:831-916):
the 2D dam break of examples/fluid/dam_break_2d_gpu.jl at dx = 0.05 advanced to t = 0.01 with
StepsizeCallback(cfl=0.9) and CarpenterKennedy2N54 (five steps of cfl h / c and one shortened
step onto the end time), then interpolated along a line (two smoothing lengths) and on a plane.
The reference ran in Float32 on a GPU and compares with isapprox (sqrt(eps(Float32)) in the
2-norm); the FP64 oracle is within 1e-7 (densities) and 2e-5 (pressures) of it, the FP32
rounding of that run.  This pins the setup, the right-hand side, the integrator with its step
size rule and the interpolation together.
"""
import math

import numpy as np
import pytest

from helpers import INTERP_RTOL, gpu_example_dam_break, initial_state, interp_golden_errors, \
    oracle_model


def test_stepsize_callback_and_schedule(pkg):
    # src/callbacks/stepsize.jl + fluid.jl:199-229: dt_sound_speed = cfl h / c is the smallest
    semi, _ = gpu_example_dam_break(pkg)
    dt = pkg.StepsizeCallback(cfl=0.9).calculate_dt(semi)
    c = 20 * math.sqrt(9.81 * 0.6)
    assert dt == 0.9 * 0.1 / c
    sched = pkg.semidiscretization.fixed_step_schedule
    n, last = sched(0.0, 0.01, dt)
    assert n == 5 and abs(last - (0.01 - 5 * dt)) < 1e-15
    assert sched(0.0, 1.0, 0.1) == (10, None)  # lands on the end within 100 ulp: no extra step
    assert sched(0.0, 0.25, 0.1)[0] == 2
    assert sched(0.5, 0.5, 0.1) == (0, None)  # empty span
    assert sched(0.0, 0.05, 0.1) == (0, 0.05)  # one shortened step
    n, last = sched(0.0, 1.0, 0.1 * (1 - 1e-15))  # ends within 100 ulp of tspan[1]: snapped
    assert n == 10 and last is None
    with pytest.raises(ValueError, match="dt must be positive"):
        sched(0.0, 1.0, 0.0)


def test_oracle_matches_reference_interpolation(pkg, orc):
    semi, tank = gpu_example_dam_break(pkg)
    model = oracle_model(orc, semi, tank)
    v, u = initial_state(tank)
    v, u = v.ravel(), u.ravel()
    dt = pkg.StepsizeCallback(cfl=0.9).calculate_dt(semi)
    n, last = pkg.semidiscretization.fixed_step_schedule(0.0, 0.01, dt)
    v, u, st = model.integrate(v, u, dt, n)
    assert st == 0
    v, u, st = model.integrate(v, u, last, 1)
    assert st == 0
    line = pkg.interpolation.line_points((0.5, 0.0), (0.5, 0.5), 10).T.copy()
    plane = pkg.interpolation.plane_points_2d((0.0, 0.0), (1.0, 1.0), 0.4).T.copy()
    res = {
        "line": model.interpolate(v, u, line, 0.1, cut_off_bnd=False,
                                  clip_negative_pressure=False),
        "line_h02": model.interpolate(v, u, line, 0.2, cut_off_bnd=False,
                                      clip_negative_pressure=False),
    }
    p = model.interpolate(v, u, plane, 0.1, cut_off_bnd=False, clip_negative_pressure=False)
    keep = np.asarray(p["neighbor_count"]) > 0
    assert keep.sum() == 8
    res["plane"] = {k: np.asarray(p[k])[keep] for k in ("computed_density", "density",
                                                         "pressure")}
    err = interp_golden_errors(res)
    assert max(err.values()) <= INTERP_RTOL, err
    # the FP64 oracle sits at the FP32 rounding of the reference run
    assert max(e for k, e in err.items() if "density" in k) <= 1e-6, err
