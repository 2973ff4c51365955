"""RectangularShape against the reference's tests (test/setups/rectangular_shape.jl): coordinates
for several corners and loop orders (exact equality, fixture from tests/golden/make_golden.py),
and the hydrostatic initialisation -- incompressible (density fixed) and compressible (density
from an inverse state equation, here the reference's mock rho(p) = 1000 + 10 p) -- for vertical,
horizontal and positive accelerations and every loop order, in 2D and 3D."""
import json
from pathlib import Path

import numpy as np
import pytest

RTOL = float(np.sqrt(np.finfo(np.float64).eps))

# loop_permutation (rectangular_shape.jl:157-196), 0-based
PERM = {2: {"y_first": (0, 1), "x_first": (1, 0)},
        3: {"z_first": (0, 1, 2), "y_first": (1, 0, 2), "x_first": (2, 1, 0)}}


def approx(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a.shape == b.shape and np.linalg.norm(a - b) <= RTOL * max(np.linalg.norm(a),
                                                                     np.linalg.norm(b))


def vec(a):
    return np.asarray(a).ravel(order="F")  # Julia's column-major vec


class MockEOS:
    """The reference's mock inverse_state_equation (rectangular_shape.jl:132-135)."""

    @staticmethod
    def inverse(p):
        return 1000.0 + 10 * p


def test_shape_coordinates_golden(pkg):
    d = json.loads((Path(__file__).parent / "golden" / "rectangular_shape_coordinates.json")
                   .read_text())
    for c in d["cases"]:
        s = pkg.RectangularShape(c["particle_spacing"], tuple(c["n"]),
                                 tuple(c["min_coordinates"]), density=1.0,
                                 loop_order=c["loop_order"], place_on_shell=c["place_on_shell"])
        assert np.array_equal(s.coordinates.T, np.array(c["coordinates"])), c


def test_incompressible_hydrostatic_2d(pkg):
    # rectangular_shape.jl:54-125
    levels = np.array([0.95, 0.85, 0.75, 0.65, 0.55, 0.45, 0.35, 0.25, 0.15, 0.05])
    pressure = np.stack([levels, levels])  # (2, 10): x, y
    S = pkg.RectangularShape
    s = S(0.1, (2, 10), (0.0, 0.0), density=1000.0, acceleration=(0.0, -9.81))
    assert approx(s.pressure, 9.81 * 1000.0 * vec(pressure))
    assert np.all(s.density == 1000.0) and np.all(s.mass == 1000 * 0.1 ** 2)
    s = S(0.1, (2, 10), (0.0, 0.0), density=1000.0, acceleration=(0.0, -9.81),
          loop_order="x_first")
    assert approx(s.pressure, 9.81 * 1000.0 * vec(pressure.T))
    s = S(0.1, (2, 10), (0.0, 0.0), density=1000.0, acceleration=(0.0, 9.81))
    assert approx(s.pressure, 9.81 * 1000.0 * vec(pressure[::-1, ::-1]))
    s = S(0.1, (10, 2), (0.0, 0.0), density=1000.0, acceleration=(-3.73, 0.0))
    assert approx(s.pressure, 3.73 * 1000.0 * vec(pressure.T))
    assert np.all(s.mass == 1000 * 0.1 ** 2)
    s = S(0.1, (10, 2), (0.0, 0.0), density=1000.0, acceleration=(-3.73, 0.0),
          loop_order="x_first")
    assert approx(s.pressure, 3.73 * 1000.0 * vec(pressure))
    s = S(0.1, (10, 2), (0.0, 0.0), density=1000.0, acceleration=(4.71, 0.0))
    assert approx(s.pressure, 4.71 * 1000.0 * vec(pressure.T[::-1, ::-1]))


def test_compressible_hydrostatic_2d(pkg):
    # rectangular_shape.jl:128-189
    pressure = np.array([[2300.0, 1100.0, 500.0, 200.0, 50.0]] * 2)  # (2, 5): x, y
    S = pkg.RectangularShape
    for order, expected in ((None, vec(pressure)), ("x_first", vec(pressure.T))):
        s = S(0.1, (2, 5), (0.0, 0.0), acceleration=(0.0, -1.0), state_equation=MockEOS,
              loop_order=order)
        assert approx(s.pressure, expected)
        assert np.array_equal(s.density, [MockEOS.inverse(p) for p in s.pressure])
        assert np.array_equal(s.mass, 0.1 ** 2 * s.density)
    s = S(0.1, (2, 5), (0.0, 0.0), acceleration=(0.0, 1.0), state_equation=MockEOS)
    assert approx(s.pressure, vec(pressure[::-1, ::-1]))
    s = S(0.1, (5, 2), (0.0, 0.0), acceleration=(-1.0, 0.0), state_equation=MockEOS)
    assert approx(s.pressure, vec(pressure.T))
    assert np.array_equal(s.mass, 0.1 ** 2 * s.density)


def _column_3d(levels):
    p = np.zeros((2, 5, 3))
    p[:, :, :] = np.asarray(levels)[None, :, None]  # gravity along -y: levels along y
    return p


@pytest.mark.parametrize("permutation", [(0, 1, 2), (1, 0, 2), (0, 2, 1)])
def test_hydrostatic_3d(pkg, permutation):
    # rectangular_shape.jl:242-356: the (2, 5, 3) column and gravity permuted onto every axis
    n = tuple(np.array((2, 5, 3))[list(permutation)])
    S = pkg.RectangularShape
    pressure = _column_3d([0.9, 0.7, 0.5, 0.3, 0.1])
    acc = tuple(np.array((0.0, -9.81, 0.0))[list(permutation)])
    for order in ("z_first", "y_first", "x_first"):
        s = S(0.2, n, (0.0, 0.0, 0.0), density=1000.0, loop_order=order, acceleration=acc)
        p = np.transpose(np.transpose(pressure, permutation), PERM[3][order])
        assert approx(s.pressure, 9.81 * 1000.0 * vec(p))
        assert np.all(s.density == 1000.0)
        assert np.all(s.mass == 1000 * ((0.2 * 0.2) * 0.2))
    pressure = _column_3d([2300.0, 1100.0, 500.0, 200.0, 50.0])
    acc = tuple(np.array((0.0, -1.0, 0.0))[list(permutation)])
    s = S(0.1, n, (0.0, 0.0, 0.0), acceleration=acc, state_equation=MockEOS)
    assert approx(s.pressure, vec(np.transpose(pressure, permutation)))
    assert np.array_equal(s.density, [MockEOS.inverse(p) for p in s.pressure])
    assert np.array_equal(s.mass, ((0.1 * 0.1) * 0.1) * s.density)


def test_shape_argument_errors(pkg):
    S = pkg.RectangularShape
    with pytest.raises(ValueError, match="not a valid loop order"):
        S(0.1, (2, 2), (0.0, 0.0), density=1.0, loop_order="z_first")
    with pytest.raises(ValueError, match="`pressure` cannot be used together"):
        S(0.1, (2, 2), (0.0, 0.0), density=1.0, pressure=1.0, acceleration=(0.0, -1.0))
    with pytest.raises(ValueError, match="`density` cannot be used together"):
        S(0.1, (2, 2), (0.0, 0.0), density=1.0, acceleration=(0.0, -1.0),
          state_equation=MockEOS)
    with pytest.raises(ValueError, match="must be used together with `acceleration`"):
        S(0.1, (2, 2), (0.0, 0.0), state_equation=MockEOS)
    with pytest.raises(ValueError, match="diagonal acceleration"):
        S(0.1, (2, 2), (0.0, 0.0), density=1.0, acceleration=(1.0, -1.0))
    with pytest.raises(ValueError, match="`density` must be specified"):
        S(0.1, (2, 2), (0.0, 0.0))
    with pytest.raises(ValueError, match="`min_coordinates` must be of length 2"):
        S(0.1, (2, 2), (0.0, 0.0, 0.0), density=1.0)
