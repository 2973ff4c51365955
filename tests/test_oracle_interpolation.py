"""The oracle's interpolate_points against the reference's own outputs and semantics (CPU).

* Pressure sensors P1-P4 of the 2D dam-break validation (sensors.jl: interpolate_line over 10
  points at the right wall, smoothing length 2h, clipped pressure, no boundary cut-off) along the
  oracle's validation run, against the fixture's pressure series: the surge front reaches every
  sensor at the same sample as in the reference, the impact peaks agree to 1e-3 and the mean
  squared difference is below 1e-5 of the signal's mean square (measured: 7e-8 for P1-P3,
  1.2e-6 for P4; the run is chaotic after the wall impact, so agreement is statistical there).
* Semantics of interpolation.jl:540-697: Shepard-normalised fields reproduce a constant field,
  points without fluid return NaN and a zero count, cut_off_bnd removes points where the walls
  add more kernel-weighted mass than the fluid, neighbour counts equal a brute-force count.
"""
import numpy as np
import pytest

from helpers import dam_break_case, initial_state, load_validation, oracle_model, \
    validation_case, validation_schedule


def sensor_segments(pkg, tank, g):
    return pkg.interpolation.dam_break_sensor_segments(g["params"]["H"],
                                                       tank.tank_size_rounded[0])


def oracle_sensors(pkg, model, v, u, segments, h):
    out = []
    for top, bottom in segments:
        pts = pkg.interpolation.line_points(top, bottom, 10).T
        r = model.interpolate(v, u, pts, 2.0 * h, cut_off_bnd=False, clip_negative_pressure=True)
        p = np.where(np.isnan(r["pressure"]), 0.0, r["pressure"])
        out.append(p.sum() / 10)
    return out


def test_oracle_pressure_sensors_match_reference(pkg, orc):
    n = 340  # to t = 0.84 s: the front reaches P1-P4 between samples 232 and 244
    semi, tank, g = validation_case(pkg)
    model = oracle_model(orc, semi, tank)
    v, u = initial_state(tank)
    v, u = v.ravel(), u.ravel()
    segs = sensor_segments(pkg, tank, g)
    h = g["params"]["smoothing_length"]
    res = [oracle_sensors(pkg, model, v, u, segs, h)]
    for steps in validation_schedule(g, n):
        for dt in steps:
            v, u, st = model.integrate(v, u, dt, 1)
            assert st == 0
        res.append(oracle_sensors(pkg, model, v, u, segs, h))
    res = np.array(res)
    for k in range(4):
        ref = np.array(g["series"][f"pressure_P{k + 1}_fluid_1"]["values"][:n])
        got = res[:, k]
        assert np.nonzero(got)[0][0] == np.nonzero(ref)[0][0]
        assert abs(got.max() - ref.max()) <= 1e-3 * ref.max()
        assert np.mean((got - ref) ** 2) <= 1e-5 * np.mean(ref ** 2)


@pytest.fixture(scope="module")
def rest_case(pkg, orc):
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0))
    model = oracle_model(orc, semi, tank)
    v, u = initial_state(tank)
    return semi, tank, model, v, u


def test_constant_density_is_reproduced(rest_case):
    semi, tank, model, v, u = rest_case
    v = v.copy()
    v[:, 2] = 1000.0  # uniform density
    pts = np.array([[0.5, 0.3], [1.0, 0.5], [1.5, 0.2], [0.31, 0.77]])
    r = model.interpolate(v, u, pts, 0.035, cut_off_bnd=False)
    assert np.allclose(r["density"], 1000.0, rtol=1e-13)
    assert np.allclose(r["velocity"], 0.0)
    assert np.all(r["neighbor_count"] > 0)


def test_outside_points_and_counts(rest_case):
    semi, tank, model, v, u = rest_case
    h = 0.035
    pts = np.array([[4.0, 3.0], [1.0, 0.5], [2.5, 0.2], [0.02, 0.02]])
    for walls in (False, True):
        r = model.interpolate(v, u, pts, h, cut_off_bnd=walls)
        assert r["neighbor_count"][0] == 0 and np.isnan(r["pressure"][0])
        assert np.isnan(r["computed_density"][0]) and np.all(np.isnan(r["velocity"][0]))
        # brute-force neighbour count of the inside point
        xf = tank.fluid.coordinates
        xw = tank.boundary.coordinates
        nf = np.sum(((xf - pts[1]) ** 2).sum(1) <= (2 * h) ** 2)
        nw = np.sum(((xw - pts[1]) ** 2).sum(1) <= (2 * h) ** 2)
        assert r["neighbor_count"][1] == nf + (nw if walls else 0)


def test_cut_off_bnd(rest_case):
    semi, tank, model, v, u = rest_case
    # a point inside the bottom wall layers: walls dominate the kernel-weighted mass
    pts = np.array([[1.0, -0.03]])
    cut = model.interpolate(v, u, pts, 0.035, cut_off_bnd=True)
    keep = model.interpolate(v, u, pts, 0.035, cut_off_bnd=False)
    assert np.isnan(cut["pressure"][0]) and cut["neighbor_count"][0] == 0
    assert np.isfinite(keep["pressure"][0]) and keep["neighbor_count"][0] > 0


def test_plane_point_grids(pkg):
    """The point sets of interpolate_plane_2d (interpolation.jl:183-209) and interpolate_plane_3d
    (sample_face_with_fixed_size, :787-824) and their argument errors."""
    I = pkg.interpolation
    p = I.plane_points_2d((0.0, 0.0), (1.0, 1.0), 0.4)
    assert p.shape == (2, 16)
    assert np.allclose(p[:, :4], [[0.0, 0.4, 0.8, 1.2], [0.0] * 4], rtol=0, atol=1e-15)
    assert np.allclose(p[:, 4], [0.0, 0.4], rtol=0, atol=1e-15)  # x fastest
    with pytest.raises(ValueError, match="2D coordinates only"):
        I.plane_points_2d((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.4)
    with pytest.raises(ValueError, match="smaller than `max_corner`"):
        I.plane_points_2d((1.0, 0.0), (0.0, 1.0), 0.4)
    f = I.face_points((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.0, 0.5, 0.5), 0.25)
    n2 = int(np.ceil(np.sqrt(0.5) / 0.25))
    assert f.shape == (3, 5 * (n2 + 1))
    assert np.array_equal(f[:, 0], [0.0, 0.0, 0.0]) and np.allclose(f[:, -1], [1.0, 0.5, 0.5])
    assert np.allclose(f[:, n2], [0.0, 0.5, 0.5])  # the second edge runs fastest
    with pytest.raises(ValueError, match="must not be collinear"):
        I.face_points((0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (2.0, 0.0, 0.0), 0.25)
    with pytest.raises(ValueError, match="3D coordinates"):
        I.face_points((0.0, 0.0), (1.0, 0.0), (0.0, 1.0), 0.25)
