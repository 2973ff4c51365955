"""ctypes binding of the C ABI declared in include/tp_wcsph.h.

Only plain pointers, sizes and the POD `tp_config` cross the boundary.  The shared library is
built in-tree (build.py); loading fails loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_float, c_int32, c_int64, c_void_p
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libtp_wcsph.so"

TP_OK = 0
TP_ERR_ARGUMENT = 1
TP_ERR_CUDA = 2
TP_ERR_OUT_OF_GRID = 3
TP_ERR_NOT_READY = 4
TP_ERR_UNSUPPORTED = 5
TP_ERR_NONFINITE = 6
TP_ERR_CAPACITY = 7

STATUS_NAMES = {
    TP_OK: "TP_OK",
    TP_ERR_ARGUMENT: "TP_ERR_ARGUMENT",
    TP_ERR_CUDA: "TP_ERR_CUDA",
    TP_ERR_OUT_OF_GRID: "TP_ERR_OUT_OF_GRID",
    TP_ERR_NOT_READY: "TP_ERR_NOT_READY",
    TP_ERR_UNSUPPORTED: "TP_ERR_UNSUPPORTED",
    TP_ERR_NONFINITE: "TP_ERR_NONFINITE",
    TP_ERR_CAPACITY: "TP_ERR_CAPACITY",
}

TP_PRECISION_FP64 = 0
TP_PRECISION_FP32 = 1
TP_VISCOSITY_NONE = 0
TP_VISCOSITY_MONAGHAN = 1
TP_DIFFUSION_NONE = 0
TP_DIFFUSION_MOLTENI_COLAGROSSI = 1


class TpConfig(ctypes.Structure):
    """Mirror of `tp_config` (include/tp_wcsph.h)."""

    _fields_ = [
        ("ndims", c_int32),
        ("precision", c_int32),
        ("n_fluid", c_int64),
        ("n_wall", c_int64),
        ("smoothing_length", c_double),
        ("reference_density", c_double),
        ("sound_speed", c_double),
        ("exponent", c_double),
        ("background_pressure", c_double),
        ("fluid_clip_negative_pressure", c_int32),
        ("wall_clip_negative_pressure", c_int32),
        ("viscosity_model", c_int32),
        ("density_diffusion_model", c_int32),
        ("viscosity_alpha", c_double),
        ("viscosity_beta", c_double),
        ("viscosity_epsilon", c_double),
        ("density_diffusion_delta", c_double),
        ("acceleration", c_double * 3),
        ("pressure_offset", c_double),
        ("min_corner", c_double * 3),
        ("max_corner", c_double * 3),
    ]


class TpError(RuntimeError):
    """A non-zero tp_status returned by the library."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


# (name, restype, argtypes) of every exported entry point, in header order.
PROTOTYPES = [
    ("tp_abi_version", c_int32, []),
    ("tp_config_default", None, [POINTER(TpConfig)]),
    ("tp_create", c_int32, [POINTER(TpConfig), POINTER(c_void_p)]),
    ("tp_destroy", c_int32, [c_void_p]),
    ("tp_set_stream", c_int32, [c_void_p, c_void_p]),
    ("tp_set_wall", c_int32, [c_void_p, c_void_p, c_void_p]),
    ("tp_set_fluid_mass", c_int32, [c_void_p, c_void_p]),
    ("tp_kick", c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_double]),
    ("tp_drift", c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_double]),
    ("tp_integrate_ck2n54", c_int32, [c_void_p, c_void_p, c_void_p, c_double, c_double, c_int64]),
    ("tp_fluid_pressure", c_int32, [c_void_p, c_void_p]),
    ("tp_wall_state", c_int32, [c_void_p, c_void_p, c_void_p, c_void_p]),
    ("tp_nhs_debug", c_int32, [c_void_p] + [c_void_p] * 6),
    ("tp_div_fast", c_int32, [c_void_p, c_double, c_void_p, c_void_p, c_float, c_void_p,
                             c_void_p, c_int64]),
    ("tp_pair_distance", c_int32, [c_void_p, c_void_p, c_void_p, c_int64]),
    ("tp_grid_info", c_int32, [c_void_p, POINTER(c_int32), POINTER(c_double), POINTER(c_double)]),
    ("tp_conservation", c_int32, [c_void_p, c_void_p, POINTER(c_double)]),
    ("tp_sync", c_int32, [c_void_p]),
    ("tp_phase_times", c_int32, [c_void_p, POINTER(c_double), c_int32]),
    ("tp_enable_timing", c_int32, [c_void_p, c_int32]),
    ("tp_prepare_lists", c_int32, [c_void_p, c_void_p, c_double]),
    ("tp_set_launch", c_int32, [c_void_p, c_int32]),
    ("tp_set_skin", c_int32, [c_void_p, c_double]),
    ("tp_kernel_launches", c_int64, [c_void_p]),
    ("tp_rebuild_count", c_int32, [c_void_p, POINTER(c_int64)]),
    ("tp_cell_sort_noalloc", c_int32,
     [POINTER(TpConfig), c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    ("tp_adjoint_forward", c_int32,
     [c_void_p, c_void_p, c_void_p, c_double, c_int64, c_int64]),
    ("tp_adjoint_backward", c_int32, [c_void_p, c_void_p, c_void_p, POINTER(c_double)]),
    ("tp_adjoint_kernel_launches", c_int64, [c_void_p]),
    ("tp_get_config", c_int32, [c_void_p, POINTER(TpConfig)]),
    ("tp_set_pair_mode", c_int32, [c_void_p, c_int32]),
    ("tp_integrate_spv", c_int32, [c_void_p, c_void_p, c_void_p, c_double, c_double, c_int64]),
    ("tp_sort_particles", c_int32, [c_void_p, c_void_p, c_void_p, c_int32, c_void_p]),
    ("tp_interpolate_points", c_int32,
     [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_double, c_int32, c_int32, c_int32,
      c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    ("tp_batch_create", c_int32, [c_void_p, c_int32, c_void_p]),
    ("tp_batch_destroy", c_int32, [c_void_p]),
    ("tp_batch_set_state", c_int32, [c_void_p, c_int32, c_void_p, c_void_p, c_double]),
    ("tp_batch_autotune", c_int32,
     [c_void_p, c_int32, POINTER(c_int32), POINTER(c_double), POINTER(c_int32),
      POINTER(c_double)]),
    ("tp_batch_capture", c_int32, [c_void_p, c_int64, c_double]),
    ("tp_batch_set_mode", c_int32, [c_void_p, c_int32]),
    ("tp_batch_launch", c_int32, [c_void_p, c_void_p]),
    ("tp_batch_sync", c_int32, [c_void_p]),
    ("tp_batch_steps", c_int64, [c_void_p]),
    ("tp_batch_last_error", c_char_p, [c_void_p]),
    ("tp_last_error", c_char_p, [c_void_p]),
]

TP_PAIR_GATHER = 0
TP_PAIR_SYMMETRIC = 1
TP_PAIR_TILED = 2
TP_BATCH_BRANCHES = 0
TP_BATCH_PERSISTENT = 1
TP_NOALLOC_MAX_PARTICLES = 262144
TP_NOALLOC_MAX_CELLS = 524288

_LIB = None


def load_library(path: Path | str | None = None) -> ctypes.CDLL:
    """Load libtp_wcsph.so (once).  Raises if it has not been built."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; "
            "g.build()'); the WCSPH path has no CPU fallback"
        )
    lib = ctypes.CDLL(str(p))
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.tp_abi_version() != 1:
        raise RuntimeError("libtp_wcsph.so ABI version mismatch")
    if path is None:
        _LIB = lib
    return lib


def check(lib: ctypes.CDLL, handle, status: int) -> None:
    if status != TP_OK:
        msg = lib.tp_last_error(handle)
        raise TpError(status, msg.decode() if msg else "")


def default_config() -> TpConfig:
    """tp_config_default, restated in Python so that it is usable without the library."""
    c = TpConfig()
    c.ndims = 3
    c.precision = TP_PRECISION_FP64
    c.reference_density = 1000.0
    c.exponent = 7.0
    c.viscosity_model = TP_VISCOSITY_MONAGHAN
    c.viscosity_alpha = 0.02
    c.viscosity_beta = 0.0
    c.viscosity_epsilon = 0.01
    c.density_diffusion_model = TP_DIFFUSION_MOLTENI_COLAGROSSI
    c.density_diffusion_delta = 0.1
    return c
