"""InitialCondition against the reference's constructor tests (test/general/initial_condition.jl:
42-156): argument errors with the reference's messages, constant quantities, quantities as
functions of the coordinates, and the mass from the particle spacing.  Arrays are in this
package's layout: coordinates (n, ndims), i.e. the transpose of the reference's (ndims, n)."""
import numpy as np
import pytest

COORDS = np.array([[88.3, 10.4, 5.2, 48.3, 58.9],
                   [23.6, 92.5, 92.1, 96.7, 84.8],
                   [77.5, 44.1, 18.2, 30.5, 44.0]]).T


def test_illegal_inputs(pkg):
    IC = pkg.InitialCondition
    with pytest.raises(ValueError, match="`coordinates` and `velocities` must be of the same"):
        IC(coordinates=np.zeros((3, 2)), velocity=np.zeros((4, 2)), mass=np.ones(3),
           density=np.ones(3))
    with pytest.raises(ValueError, match="`velocity` must be 2-dimensional for 2-dimensional"):
        IC(coordinates=np.zeros((3, 2)), velocity=lambda x: (1, 2, 3), mass=np.ones(3),
           density=np.ones(3))
    for name, kw in (("mass", dict(mass=np.ones(3), density=np.ones(2))),
                     ("density", dict(mass=np.ones(2), density=np.ones(3))),
                     ("pressure", dict(mass=np.ones(2), density=np.ones(2),
                                       pressure=np.ones(3)))):
        msg = (f"Expected: length\\({name}\\) == size\\(coordinates, 2\\)\nGot: "
               f"size\\(coordinates, 2\\) = 2, length\\({name}\\) = 3")
        with pytest.raises(ValueError, match=msg):
            IC(coordinates=np.zeros((2, 2)), velocity=np.zeros((2, 2)), **kw)
    with pytest.raises(ValueError, match="`mass` must be specified when not using"):
        IC(coordinates=np.zeros((2, 2)), velocity=np.zeros((2, 2)), density=np.ones(2))
    with pytest.raises(ValueError, match="density must be positive and larger than `eps\\(\\)`"):
        IC(coordinates=np.zeros((2, 2)), velocity=np.zeros((2, 2)), density=np.zeros(2),
           mass=np.ones(2))


def test_constant_quantities(pkg):
    IC = pkg.InitialCondition
    a = IC(coordinates=np.zeros((5, 2)), velocity=(1.0, 2.0), mass=3.0, density=4.0,
           pressure=5.0)
    b = IC(coordinates=np.zeros((5, 2)), velocity=[1.0, 2.0], mass=3.0, density=4.0,
           pressure=5.0)
    for ic in (a, b):
        assert np.array_equal(ic.velocity, np.tile([1.0, 2.0], (5, 1)))
        assert np.array_equal(ic.mass, 3 * np.ones(5))
        assert np.array_equal(ic.density, 4 * np.ones(5))
        assert np.array_equal(ic.pressure, 5 * np.ones(5))


def test_automatic_mass_and_functions(pkg):
    IC = pkg.InitialCondition
    dx = 0.13
    a = IC(coordinates=COORDS, velocity=lambda x: 2 * x, density=lambda x: 4 * x[1],
           pressure=lambda x: 5 * x[2], particle_spacing=dx)
    assert np.array_equal(a.velocity, 2 * COORDS)
    assert np.array_equal(a.density, 4 * COORDS[:, 1])
    assert np.array_equal(a.pressure, 5 * COORDS[:, 2])
    assert np.array_equal(a.mass, ((dx * dx) * dx) * (4 * COORDS[:, 1]))  # dx^3 as Julia's x*x*x
    b = IC(coordinates=COORDS, velocity=lambda x: 2 * x, mass=lambda x: 3 * x[0],
           density=lambda x: 4 * x[1], pressure=lambda x: 5 * x[2])
    assert np.array_equal(b.mass, 3 * COORDS[:, 0])
    assert np.array_equal(b.velocity, 2 * COORDS)


def test_empty_initial_condition(pkg):
    ic = pkg.InitialCondition(coordinates=np.zeros((0, 3)), density=1000.0, particle_spacing=0.1)
    assert ic.n_particles == 0 and ic.velocity.shape == (0, 3) and ic.mass.shape == (0,)
