"""Host side of the batched ensemble: seeded instance draws and the side-by-side layout that keeps
instances from interacting (no GPU needed)."""
import math

import numpy as np


def test_specs_are_seeded_and_in_range(pkg):
    e = pkg.ensemble
    a = e.ensemble_specs(512, seed=0)
    b = e.ensemble_specs(512, seed=0)
    assert a == b
    assert len(a) == 512
    w = np.array([s.width for s in a])
    h = np.array([s.height for s in a])
    assert w.min() >= 0.5 and w.max() <= 2.0
    assert h.min() >= 0.25 and h.max() <= 1.0
    assert {s.dx for s in a} == set(e.SPACINGS)
    assert e.ensemble_specs(512, seed=1) != a


def test_group_layout_separates_instances(pkg):
    e = pkg.ensemble
    specs = e.ensemble_specs(6, seed=4)
    for s in specs:
        s.dx = 0.02
    g = e.build_group(specs, list(range(6)))
    h = g.semi.config.smoothing_length
    cs = 2.0 * h
    # shifts are whole numbers of cells, so every instance sees the same cell boundaries
    for s in g.shifts:
        assert abs(s / cs - round(s / cs)) < 1e-9
    # particle blocks of consecutive instances are further apart than any list radius (skin <= 1)
    x = np.concatenate([g.semi.wall.initial_condition.coordinates[:, 0]])
    n_wall_each = g.tanks[0].boundary.n_particles
    for k in range(5):
        lo_next = g.shifts[k + 1] + g.tanks[k + 1].boundary.coordinates[:, 0].min()
        hi_this = g.shifts[k] + g.tanks[k].boundary.coordinates[:, 0].max()
        assert lo_next - hi_this > 2.0 * cs
    assert x.shape[0] == sum(t.boundary.n_particles for t in g.tanks)
    assert n_wall_each > 0
    # fluid ranges tile the fluid array in instance order
    assert g.fluid_ranges[0][0] == 0
    assert g.fluid_ranges[-1][1] == g.semi.n_fluid
    for (a0, a1), (b0, _) in zip(g.fluid_ranges, g.fluid_ranges[1:]):
        assert a1 == b0


def test_full_ensemble_size(pkg):
    e = pkg.ensemble
    specs = e.ensemble_specs(512, seed=0)
    groups = e.build_ensemble(specs)
    assert sorted(i for g in groups for i in g.instances) == list(range(512))
    n_fluid = sum(g.semi.n_fluid for g in groups)
    # ~8M particles in total over the 512 instances
    assert 6e6 < n_fluid < 9e6
    per = [g.tanks[j].fluid.n_particles for g in groups for j in range(len(g.instances))]
    assert min(per) >= 0.5 * 0.25 / 0.02**2 - 1 and max(per) <= 2.0 * 1.0 / 0.005**2 + 1
    for g in groups:
        assert math.isclose(e.time_step(g.dx) / g.dx, 5e-3)
