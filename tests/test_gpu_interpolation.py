"""interpolate_points on the GPU (tp_interpolate_points) against the oracle, and the validation
pressure sensors along the GPU run against the reference's series.

Tolerances: the library sums in its own cell order (the oracle in the reference's), so finite
fields agree to 1e-12 relative; NaN patterns and neighbour counts agree exactly.  Sensors: the
same statistical bounds as the oracle's test against the fixture.
"""
import ctypes

import numpy as np
import pytest

from helpers import dam_break_case, initial_state, oracle_model, validation_case, \
    validation_schedule

pytestmark = pytest.mark.gpu


def _moved_state(pkg, cuda, semi, steps=20, dt=1e-4):
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    v, u = ode.v0.clone(), ode.u0.clone()
    semi._set_stream()
    semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
               ctypes.c_double(dt), ctypes.c_int64(steps))
    semi.sync()
    return v, u


def _compare(a, b, tol=1e-12):
    for key in ("computed_density", "pressure", "density"):
        x, y = np.asarray(a[key]), np.asarray(b[key])
        assert np.array_equal(np.isnan(x), np.isnan(y)), key
        m = ~np.isnan(y)
        assert np.allclose(x[m], y[m], rtol=tol, atol=tol * max(1.0, np.abs(y[m]).max())), key
    assert np.array_equal(a["neighbor_count"], b["neighbor_count"])


@pytest.mark.parametrize("nd", [2, 3])
def test_interpolation_matches_oracle(pkg, orc, cuda, nd):
    if nd == 2:
        semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=3)
        lo, hi = np.array([-0.05, -0.05]), np.array([2.5, 1.3])
    else:
        semi, tank = dam_break_case(pkg, 3, 0.05, (1.0, 0.5, 1.0), (3.2, 1.0, 1.4), jitter=0.1,
                                    seed=3)
        lo, hi = np.array([-0.1, -0.1, -0.1]), np.array([1.4, 0.7, 1.2])
    v, u = _moved_state(pkg, cuda, semi)
    rng = np.random.default_rng(9)
    pts = lo + (hi - lo) * rng.random((300, nd))
    model = oracle_model(orc, semi, tank)
    vn, un = v.cpu().numpy(), u.cpu().numpy()
    h = semi.fluid.smoothing_length
    for hi_ in (h, 2.0 * h):
        for cut, clip, wallv in ((True, False, False), (False, True, False), (True, True, True)):
            got = pkg.interpolate_points(pts.T, semi, semi.fluid, v, u, smoothing_length=hi_,
                                         cut_off_bnd=cut, clip_negative_pressure=clip,
                                         include_wall_velocity=wallv)
            ref = model.interpolate(vn, un, pts, hi_, cut_off_bnd=cut,
                                    clip_negative_pressure=clip, include_wall_velocity=wallv)
            _compare(got, ref)
            gv, rv = got["velocity"].T, ref["velocity"]
            m = ~np.isnan(rv[:, 0])
            assert np.allclose(gv[m], rv[m], rtol=1e-10, atol=1e-12)
    semi.close()


def test_interpolate_line_endpoints(pkg, cuda):
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0))
    v, u = _moved_state(pkg, cuda, semi, steps=1)
    r = pkg.interpolate_line([1.0, 0.05], [1.0, 0.95], 5, semi, semi.fluid, v, u)
    assert r["point_coords"].shape == (2, 5)
    r2 = pkg.interpolate_line([1.0, 0.05], [1.0, 0.95], 5, semi, semi.fluid, v, u,
                              endpoint=False)
    assert r2["point_coords"].shape == (2, 3)
    assert np.allclose(r2["pressure"], r["pressure"][1:-1], rtol=1e-14)
    # hydrostatic column: pressure decreases upwards
    assert np.all(np.diff(r["pressure"]) < 0)
    semi.close()


def test_gpu_validation_pressure_sensors(pkg, cuda):
    n = 340
    semi, tank, g = validation_case(pkg, "float64")
    ode = pkg.semidiscretize(semi, (0.0, 2.0))
    v, u = ode.v0.clone(), ode.u0.clone()
    segs = pkg.interpolation.dam_break_sensor_segments(g["params"]["H"], tank.tank_size_rounded[0])

    def sensors():
        return [pkg.interpolation.interpolated_pressure(a, b, v, u, semi) for a, b in segs]

    res = [sensors()]
    for steps in validation_schedule(g, n):
        i = 0
        while i < len(steps):
            j = i
            while j < len(steps) and steps[j] == steps[i]:
                j += 1
            semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                       ctypes.c_double(steps[i]), ctypes.c_int64(j - i))
            i = j
        res.append(sensors())
    semi.close()
    res = np.array(res)
    for k in range(4):
        ref = np.array(g["series"][f"pressure_P{k + 1}_fluid_1"]["values"][:n])
        got = res[:, k]
        assert np.nonzero(got)[0][0] == np.nonzero(ref)[0][0]
        assert abs(got.max() - ref.max()) <= 1e-3 * ref.max()
        assert np.mean((got - ref) ** 2) <= 1e-5 * np.mean(ref ** 2)
