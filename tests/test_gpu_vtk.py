"""VTK snapshots, SolutionSavingCallback and restart on the GPU: a snapshot holds the device
state exactly, solve writes the expected numbered files and collections, and a run restarted
from a file continues the uninterrupted run (FP64: 1e-12 relative; the neighbour lists of the
restarted call are rebuilt at a different time, which changes only the in-cell summation order)."""
import os

import numpy as np
import pytest
import torch

from helpers import dam_break_case, rel_l2

pytestmark = pytest.mark.gpu


def test_snapshot_and_files(pkg, cuda, tmp_path):
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=1)
    ode = pkg.semidiscretize(semi, (0.0, 1.0))
    sol = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=1e-4, n_steps=10)
    files = pkg.trixi2vtk(semi, sol.v, sol.u, sol.t, output_directory=str(tmp_path))
    assert [os.path.basename(f) for f in files] == ["fluid_1.vtu", "boundary_1.vtu"]
    d = pkg.vtk2trixi(files[0])
    v = sol.v.view(-1, 3).cpu().numpy()
    assert np.array_equal(d["coordinates"], sol.u.view(-1, 2).cpu().numpy())
    assert np.array_equal(d["velocity"], v[:, :2]) and np.array_equal(d["density"], v[:, 2])
    assert d["time"] == pytest.approx(sol.t) and d["particle_spacing"] == 0.02
    p = semi.fluid_pressure()
    semi.sync()
    assert np.array_equal(d["pressure"], p.cpu().numpy())
    w = pkg.vtk.read_vtu(files[1])
    assert w["points"].shape[0] == tank.boundary.n_particles
    assert "hydrodynamic_density" in w["point_data"]
    semi.close()


def test_saving_callback_and_restart(pkg, cuda, tmp_path):
    n, dt = 20, 1e-4
    semi, tank = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=1)
    ode = pkg.semidiscretize(semi, (0.0, n * dt))
    full = pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=n)
    cb = pkg.SolutionSavingCallback(interval=5, output_directory=str(tmp_path))
    pkg.solve(ode, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=10, callback=cb)
    names = sorted(os.path.basename(f) for f in cb.files)
    assert "fluid_1_0.vtu" in names and "fluid_1_2.vtu" in names  # steps 0, 5, 10
    assert len([f for f in names if f.startswith("fluid_1_")]) == 3
    assert os.path.exists(tmp_path / "fluid_1.pvd")
    # restart from the step-10 file and finish the run
    semi2, _ = dam_break_case(pkg, 2, 0.02, (2.0, 1.0), (5.366, 4.0), jitter=0.1, seed=1)
    ode2 = pkg.semidiscretize(semi2, (0.0, n * dt))
    ode2, t = pkg.vtk.restart_from(ode2, semi2, [str(tmp_path / "fluid_1_2.vtu"),
                                                 str(tmp_path / "boundary_1_2.vtu")])
    assert t == pytest.approx(10 * dt)
    rest = pkg.solve(ode2, pkg.CarpenterKennedy2N54(), dt=dt, n_steps=n - 10)
    assert rel_l2(rest.u.cpu().numpy(), full.u.cpu().numpy()) <= 1e-12
    assert rel_l2(rest.v.cpu().numpy(), full.v.cpu().numpy()) <= 1e-10
    semi.close()
    semi2.close()
