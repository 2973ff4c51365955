"""Host-side dam-break setup (numpy) against the oracle's restatement, and the particle counts of
the benchmark configurations."""
import numpy as np
import pytest


@pytest.mark.parametrize("nd,dx,fluid,tank,layers", [
    (2, 0.02, (2.0, 1.0), (5.366, 4.0), 3),
    (2, 0.015, (1.2, 0.6), (3.21, 4.0), 4),
    (3, 0.05, (1.0, 0.5, 1.0), (3.2, 1.0, 1.4), 3),
    (3, 0.04, (0.4, 0.3, 0.2), (0.8, 0.5, 0.5), 2),
])
def test_setup_matches_oracle(pkg, orc, nd, dx, fluid, tank, layers):
    t, eos = pkg.dam_break(nd, dx, fluid, tank, n_layers=layers)
    acc = (0.0, -9.81) if nd == 2 else (0.0, -9.81, 0.0)
    o = orc.tank(nd, dx, fluid, tank, layers, 1000.0, eos.sound_speed, 7.0, 0.0, acc)
    assert np.array_equal(t.fluid.coordinates, o["x_f"])
    assert np.array_equal(t.fluid.density, o["rho_f"])
    assert np.array_equal(t.fluid.mass, o["m_f"])
    assert np.array_equal(t.boundary.coordinates, o["x_w"])
    assert np.array_equal(t.boundary.mass, o["m_w"])
    assert np.array_equal(t.boundary.density, o["rho_w"])


def test_benchmark_counts(pkg):
    # 2D dam break at dx = 0.02 and the 3D dam break at dx = 0.008 (literal geometry).
    t, _ = pkg.dam_break(2, 0.02, (2.0, 1.0), (5.366, 4.0), n_layers=3)
    assert (t.fluid.n_particles, t.boundary.n_particles) == (5000, 2844)
    t, _ = pkg.dam_break(3, 0.008, (1.0, 0.5, 1.0), (3.2, 1.0, 1.4), n_layers=3)
    assert t.fluid.n_particles == 968_750
    assert t.boundary.n_particles == 876_666


def test_hydrostatic_profile(pkg):
    t, eos = pkg.dam_break(2, 0.02, (2.0, 1.0), (5.366, 4.0), n_layers=3)
    y = t.fluid.coordinates[:, 1]
    rho = t.fluid.density
    # density decreases with height, top particle sits half a step below the surface
    top = rho[np.argmax(y)]
    assert top == pytest.approx(eos.inverse((0.5 * 0.02 * 9.81) * eos.inverse(0.0)), rel=0)
    assert np.all(np.diff(rho[np.argsort(y)]) <= 0)


def test_tank_boundary_faces_golden(pkg):
    """The reference's "Boundary Faces" test (test/setups/rectangular_tank.jl:185-270, fixture
    from tests/golden/make_golden.py): wall coordinates, in order, for one and three layers and
    every face selection, with the reference's isapprox (sqrt(eps) relative, 2-norm)."""
    import json
    from pathlib import Path

    d = json.loads((Path(__file__).parent / "golden" / "rectangular_tank_faces.json").read_text())
    t = d["tank"]
    rtol = float(np.sqrt(np.finfo(np.float64).eps))
    for case in d["cases"]:
        tank = pkg.RectangularTank(t["particle_spacing"], tuple(t["fluid_size"]),
                                   tuple(t["tank_size"]), t["fluid_density"],
                                   n_layers=case["n_layers"], faces=tuple(case["faces"]))
        got = tank.boundary.coordinates.T
        exp = np.array(case["boundary_coordinates"])
        assert got.shape == exp.shape, case
        assert np.linalg.norm(got - exp) <= rtol * max(np.linalg.norm(got), np.linalg.norm(exp))


def test_tank_coordinates_golden(pkg):
    """The reference's RectangularTank "Coordinates" tests in 2D and 3D (test/setups/
    rectangular_tank.jl:1-58, 125-141, 274-340, 373-387; fixture from tests/golden/
    make_golden.py): fluid and wall coordinates for two spacings, spacing ratios 1 and 3 and two
    tank corners with one layer, and three layers, with the reference's isapprox."""
    import json
    from pathlib import Path

    d = json.loads((Path(__file__).parent / "golden" / "rectangular_tank_coordinates.json")
                   .read_text())
    rtol = float(np.sqrt(np.finfo(np.float64).eps))

    def close(got, exp):
        return got.shape == exp.shape and np.linalg.norm(got - exp) <= rtol * max(
            np.linalg.norm(got), np.linalg.norm(exp))

    for c in d["cases"]:
        corner = np.array(c["min_coordinates"])
        tank = pkg.RectangularTank(c["particle_spacing"], tuple(c["fluid_size"]),
                                   tuple(c["tank_size"]), c["fluid_density"],
                                   n_layers=c["n_layers"], spacing_ratio=c["spacing_ratio"],
                                   min_coordinates=tuple(corner))
        exp_b = np.array(c["boundary_coordinates"]) + corner[:, None]
        assert close(tank.boundary.coordinates.T, exp_b), c
        if c["fluid_coordinates"] is not None:
            exp_f = np.array(c["fluid_coordinates"]) + corner[:, None]
            assert close(tank.fluid.coordinates.T, exp_f), c
        bdx = c["particle_spacing"] / c["spacing_ratio"]
        assert np.allclose(tank.boundary.mass, c["fluid_density"] * bdx ** c["ndims"],
                           rtol=1e-15)
