"""The pair kernels' divisions on the device against IEEE division, as the reference tests its
`div_fast` on the GPU (test/examples/gpu.jl:30-78): x = pi divided by 1024 random y in [1, 2).
FP64 drop-in (x * fast_inv(y), the reference's CUDA Float64 definition): maximum error below
1e-15 and not zero (a fast division is in use); FP32 form (__fdividef): below 1e-6 and not zero.
Also the argument checks of tp_div_fast.
"""
import ctypes

import numpy as np
import pytest

from helpers import dam_break_case

pytestmark = pytest.mark.gpu


def test_div_fast_matches_reference_bounds(pkg, cuda):
    torch = cuda
    semi, _ = dam_break_case(pkg, 2, 0.1, (0.5, 0.3), (1.0, 0.6))
    pkg.semidiscretize(semi, (0.0, 1.0))
    rng = np.random.default_rng(7)
    y64 = rng.random(1024) + 1.0
    y32 = (rng.random(1024).astype(np.float32) + np.float32(1.0)).astype(np.float32)
    y64_t = torch.as_tensor(y64, device=semi.device)
    y32_t = torch.as_tensor(y32, device=semi.device)
    o64 = torch.full_like(y64_t, float("nan"))
    o32 = torch.full_like(y32_t, float("nan"))
    x32 = np.float32(np.pi)
    semi._call("tp_div_fast", ctypes.c_double(np.pi), y64_t.data_ptr(), o64.data_ptr(),
               ctypes.c_float(x32), y32_t.data_ptr(), o32.data_ptr(), ctypes.c_int64(1024))
    semi.sync()
    err64 = np.abs(o64.cpu().numpy() - np.pi / y64).max()
    err32 = np.abs(o32.cpu().numpy() - x32 / y32).max()  # numpy: IEEE FP32 division
    assert 0.0 < err64 < 1e-15
    assert 0.0 < err32 < 1e-6
    with pytest.raises(Exception, match="without its output"):
        semi._call("tp_div_fast", ctypes.c_double(1.0), y64_t.data_ptr(), None,
                   ctypes.c_float(1.0), None, None, ctypes.c_int64(4))
    with pytest.raises(Exception, match="bad element count"):
        semi._call("tp_div_fast", ctypes.c_double(1.0), None, None, ctypes.c_float(1.0), None,
                   None, ctypes.c_int64(-1))
    semi.close()


def test_pair_distance_within_two_ulp_of_sqrt(pkg, cuda):
    """The FP64 kernels' pair distance (approximate reciprocal square root + one third-order
    step, times d2) against the rounded sqrt the reference takes: within 2 ulp over d2 spanning
    the pair scales of every workload (log-uniform in [1e-30, 1e6]) and exact squares."""
    torch = cuda
    semi, _ = dam_break_case(pkg, 2, 0.1, (0.5, 0.3), (1.0, 0.6))
    pkg.semidiscretize(semi, (0.0, 1.0))
    rng = np.random.default_rng(11)
    d2 = np.concatenate([10.0 ** rng.uniform(-30.0, 6.0, 200_000),
                         np.arange(1, 1001, dtype=np.float64) ** 2 * 1e-6])
    d2_t = torch.as_tensor(d2, device=semi.device)
    r_t = torch.full_like(d2_t, float("nan"))
    semi._call("tp_pair_distance", d2_t.data_ptr(), r_t.data_ptr(), ctypes.c_int64(d2.size))
    semi.sync()
    r = r_t.cpu().numpy()
    ref = np.sqrt(d2)
    ulp = np.abs(r - ref) / np.spacing(ref)
    assert np.all(np.isfinite(r))
    assert ulp.max() <= 2.0
    with pytest.raises(Exception, match="null array"):
        semi._call("tp_pair_distance", None, r_t.data_ptr(), ctypes.c_int64(4))
    with pytest.raises(Exception, match="bad element count"):
        semi._call("tp_pair_distance", d2_t.data_ptr(), r_t.data_ptr(), ctypes.c_int64(-1))
    semi.close()
