"""Host-side mirror of the reference surface: configuration checks without a GPU."""
import numpy as np
import pytest

from helpers import dam_break_case


def test_config_from_dam_break(pkg):
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0))
    c = semi.config
    assert (c.ndims, c.n_fluid, c.n_wall) == (2, 5000, 2844)
    assert c.smoothing_length == 1.75 * 0.02
    assert c.sound_speed == 20 * np.sqrt(9.81)
    assert c.viscosity_alpha == 0.02 and c.density_diffusion_delta == 0.1
    assert c.wall_clip_negative_pressure == 1 and c.fluid_clip_negative_pressure == 0
    assert c.min_corner[0] == tank.boundary.coordinates[:, 0].min()
    assert c.max_corner[1] == tank.boundary.coordinates[:, 1].max()


def _systems(pkg):
    semi, tank = dam_break_case(pkg, 2, 0.05, (1.0, 0.5), (2.0, 1.0))
    return semi.fluid, semi.wall, semi.neighborhood_search


def test_rejects_single_system(pkg):
    f, w, nhs = _systems(pkg)
    with pytest.raises(ValueError, match="ArgumentError"):
        pkg.Semidiscretization(f, neighborhood_search=nhs,
                               parallelization_backend=pkg.GB300Backend())


def test_rejects_other_kernel_and_models(pkg):
    import dataclasses

    f, w, nhs = _systems(pkg)
    for change in [dict(smoothing_kernel=pkg.WendlandC2Kernel(3)), dict(correction="shepard"),
                   dict(viscosity="morris"), dict(density_diffusion="antuono"),
                   dict(density_calculator=None)]:
        with pytest.raises(ValueError, match="ArgumentError"):
            f2 = dataclasses.replace(f, **change)
            pkg.Semidiscretization(f2, w, neighborhood_search=nhs,
                                   parallelization_backend=pkg.GB300Backend())


def test_wcsph_constructor_checks(pkg):
    """test/systems/wcsph_system.jl:3-68: the reference's messages for a wrong acceleration
    length and kernel dimension; the acceleration defaults to zeros."""
    import dataclasses

    f, _, _ = _systems(pkg)
    with pytest.raises(ValueError, match="`acceleration` must be of length 2 for a 2D problem"):
        dataclasses.replace(f, acceleration=0.0)
    with pytest.raises(ValueError, match="smoothing kernel dimensionality must be 2 for a 2D"):
        dataclasses.replace(f, smoothing_kernel=pkg.WendlandC2Kernel(3))
    assert dataclasses.replace(f, acceleration=None).acceleration == (0.0, 0.0)


def test_rejects_missing_cell_list_and_wall_eos(pkg):
    import dataclasses

    f, w, nhs = _systems(pkg)
    with pytest.raises(ValueError, match="FullGridCellList"):
        pkg.Semidiscretization(f, w, neighborhood_search=pkg.GridNeighborhoodSearch(2),
                               parallelization_backend=pkg.GB300Backend())
    bm = dataclasses.replace(w.boundary_model, state_equation=None)
    w2 = dataclasses.replace(w, boundary_model=bm)
    # test/general/semidiscretization.jl:209-227: the reference's message
    msg = ("`WeaklyCompressibleSPHSystem` cannot be used without setting a `state_equation` "
           "for all boundary models")
    with pytest.raises(ValueError, match=msg.replace("`", ".")):
        pkg.Semidiscretization(f, w2, neighborhood_search=nhs,
                               parallelization_backend=pkg.GB300Backend())
    f2 = dataclasses.replace(f, state_equation=None)
    with pytest.raises(ValueError, match="needs the fluid's `state_equation`"):
        pkg.Semidiscretization(f2, w, neighborhood_search=nhs,
                               parallelization_backend=pkg.GB300Backend())


def test_callback_mirrors(pkg):
    """CallbackSet drops `nothing` entries; InfoCallback's interval; StepsizeCallback's rule
    without viscosity and gravity is the sound-speed limit cfl h / c (fluid.jl:199-229)."""
    import dataclasses

    info = pkg.InfoCallback(interval=100)
    st = pkg.StepsizeCallback(cfl=0.5)
    assert pkg.CallbackSet(None, info, None, st) == [info, st]
    assert pkg.InfoCallback().interval is None
    with pytest.raises(ValueError, match="non-negative"):
        pkg.InfoCallback(interval=-1)
    f, w, nhs = _systems(pkg)
    f0 = dataclasses.replace(f, viscosity=None, acceleration=(0.0, 0.0))
    semi = pkg.Semidiscretization(f0, w, neighborhood_search=nhs,
                                  parallelization_backend=pkg.GB300Backend())
    h, c = f0.smoothing_length, f0.state_equation.sound_speed
    assert st.calculate_dt(semi) == 0.5 * h / c
