"""The GPU FP64 drop-in against the reference's own 2D dam-break validation trajectory
(validation_reference_wcsph_40.json): surge-front position max_x over 701 samples."""
import numpy as np
import pytest

from helpers import rel_l2, validation_case, validation_schedule

pytestmark = pytest.mark.gpu


def run_gpu(pkg, precision, n_samples):
    semi, tank, g = validation_case(pkg, precision)
    ode = pkg.semidiscretize(semi, (0.0, 2.0))
    v, u = ode.v0.clone(), ode.u0.clone()
    out = [float(u.view(-1, 2)[:, 0].max())]
    import ctypes

    for steps in validation_schedule(g, n_samples):
        # consecutive equal steps go in one fused call
        i = 0
        while i < len(steps):
            j = i
            while j < len(steps) and steps[j] == steps[i]:
                j += 1
            semi._call("tp_integrate_ck2n54", v.data_ptr(), u.data_ptr(), ctypes.c_double(0.0),
                       ctypes.c_double(steps[i]), ctypes.c_int64(j - i))
            i = j
        out.append(float(u.view(-1, 2)[:, 0].max()))
    semi.sync()
    semi.close()
    return np.array(out), np.array(g["series"]["max_x_coord_fluid_1"]["values"][:n_samples])


def test_fp64_validation_trajectory(pkg, cuda):
    got, ref = run_gpu(pkg, "float64", 701)
    assert np.abs(got[:60] - ref[:60]).max() < 1e-9   # smooth collapse phase
    assert np.abs(got[:140] - ref[:140]).max() < 1e-6
    assert rel_l2(got, ref) < 1e-3                      # whole run incl. the chaotic impact


def test_fp32_validation_trajectory(pkg, cuda):
    got, ref = run_gpu(pkg, "float32", 701)
    assert np.abs(got[:60] - ref[:60]).max() < 1e-5
    assert rel_l2(got, ref) < 5e-3
