"""The device path against the reference's GPU interpolation goldens (test/examples/gpu.jl:
831-916), through the reference-facing surface: semidiscretize, solve(ode,
CarpenterKennedy2N54(); dt=1.0, callback=StepsizeCallback(cfl=0.9)) to t = 0.01 (the last step
shortened onto the end time, as OrdinaryDiffEq does), interpolate_line and interpolate_plane_2d.
Criterion: the reference's own isapprox (sqrt(eps(Float32)) in the 2-norm), for the FP64
drop-in and the FP32 form; the FP64 drop-in's densities are also within 1e-6 (the FP32 rounding
of the reference's run).
"""
import numpy as np
import pytest

from helpers import INTERP_RTOL, gpu_example_dam_break, interp_golden_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_reference_interpolation_goldens(pkg, cuda, precision):
    semi, _ = gpu_example_dam_break(pkg, precision)
    ode = pkg.semidiscretize(semi, (0.0, 0.01))
    if precision == "float64":
        sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=1.0,
                        callback=pkg.StepsizeCallback(cfl=0.9))
    else:  # the examples' form: CallbackSet with an InfoCallback and `nothing` entries
        info = pkg.InfoCallback(interval=2)
        sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(williamson_condition=False), dt=1.0,
                        callback=pkg.CallbackSet(info, None, pkg.StepsizeCallback(cfl=0.9)))
        assert len(info.lines) == 2  # after steps 2 and 4 of the five full ones
    assert sol.n_steps == 6 and sol.t == 0.01
    kw = dict(cut_off_bnd=False)
    res = {
        "line": pkg.interpolate_line((0.5, 0.0), (0.5, 0.5), 10, semi, semi.fluid, sol.v, sol.u,
                                     **kw),
        "line_h02": pkg.interpolate_line((0.5, 0.0), (0.5, 0.5), 10, semi, semi.fluid, sol.v,
                                         sol.u, smoothing_length=0.2, **kw),
        "plane": pkg.interpolate_plane_2d((0.0, 0.0), (1.0, 1.0), 0.4, semi, semi.fluid, sol.v,
                                          sol.u, **kw),
    }
    assert len(res["plane"]["pressure"]) == 8
    assert np.all(res["plane"]["neighbor_count"] > 0)
    err = interp_golden_errors(res)
    assert max(err.values()) <= INTERP_RTOL, err
    if precision == "float64":
        assert max(e for k, e in err.items() if "density" in k) <= 1e-6, err
    semi.close()
