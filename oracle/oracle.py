"""ctypes wrapper of the FP64 CPU oracle (tp_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU-baseline leg
of bench.py as the checker.  The product library never imports or calls it.

Parity status: the oracle restates the reference's Float64 CPU path (see tp_oracle.cpp); it is
pinned by the reference's own known-answer tests (Monaghan viscosity, Cole EOS inverse, kernel
normalisation/derivative, Adami constant-pressure exactness, drift copy) and by the 2D dam-break
validation trajectory validation/dam_break_2d/validation_reference_wcsph_40.json, carried as the
fixture tests/golden/validation_wcsph_40_max_x.json.
"""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libtp_oracle.so"
_lib = None


def build(force: bool = False) -> Path:
    """make -C oracle (g++ -O2 -fopenmp -ffp-contract=off)."""
    args = ["make", "-s", "-C", str(HERE)]
    if force:
        args.append("-B")
    res = subprocess.run(args, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        dp = POINTER(c_double)
        ip = POINTER(c_int32)
        L.orc_create.restype = c_void_p
        L.orc_create.argtypes = [c_void_p, dp, dp, dp]
        L.orc_destroy.argtypes = [c_void_p]
        L.orc_kick.restype = c_int
        L.orc_kick.argtypes = [c_void_p, dp, dp, dp]
        L.orc_drift.argtypes = [c_void_p, dp, dp]
        L.orc_last_state.argtypes = [c_void_p, dp, dp, dp, dp]
        L.orc_integrate_ck2n54.restype = c_int
        L.orc_integrate_ck2n54.argtypes = [c_void_p, dp, dp, c_double, c_int64]
        L.orc_integrate_ck2n54_jvp.restype = c_int
        L.orc_integrate_ck2n54_jvp.argtypes = [c_void_p, dp, dp, dp, dp, dp, dp, dp, c_double,
                                               c_int64, dp, dp]
        L.orc_ck2n54_coefficients.argtypes = [dp, dp, dp]
        L.orc_sort_perm.restype = c_int
        L.orc_sort_perm.argtypes = [c_void_p, dp, c_int64, ip]
        L.orc_integrate_spv.restype = c_int
        L.orc_integrate_spv.argtypes = [c_void_p, dp, dp, c_double, c_int64]
        L.orc_interpolate.argtypes = [c_void_p, dp, dp, dp, c_int64, c_double, c_int, c_int,
                                      c_int, dp, dp, dp, dp, ip]
        L.orc_nhs.restype = c_int
        L.orc_nhs.argtypes = [c_void_p, dp, dp, ip, ip, ip, ip, ip]
        for name in ("orc_wendland_c2", "orc_wendland_c2_deriv_div_r"):
            getattr(L, name).restype = c_double
            getattr(L, name).argtypes = [c_int, c_double, c_double]
        L.orc_cole_pressure.restype = c_double
        L.orc_cole_pressure.argtypes = [c_double, c_double, c_double, c_double, c_int, c_double]
        L.orc_cole_inverse.restype = c_double
        L.orc_cole_inverse.argtypes = [c_double, c_double, c_double, c_double, c_double]
        L.orc_monaghan_pair.argtypes = [c_int, c_double, c_double, c_double, c_double, c_double,
                                        dp, dp, dp, c_double, c_double, c_double, dp]
        L.orc_tank.restype = c_int
        L.orc_tank.argtypes = [c_int, c_double, dp, dp, c_int, ip, c_double, c_double, c_double,
                               c_double, dp, POINTER(c_int64), POINTER(c_int64), dp, dp, dp, dp,
                               dp, dp]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(POINTER(c_double))


def _ip(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(POINTER(c_int32))


def tank(ndims, dx, fluid_size, tank_size, n_layers, rho0, c, gamma, p_bg=0.0, accel=None,
         faces=None):
    """RectangularTank restatement; returns dict of (n, nd) / (n,) arrays."""
    L = lib()
    fs = np.array(fluid_size, dtype=np.float64)
    ts = np.array(tank_size, dtype=np.float64)
    fc = np.array(faces if faces is not None else [1] * (2 * ndims), dtype=np.int32)
    acc = np.zeros(3) if accel is None else np.array(list(accel) + [0.0] * (3 - len(accel)))
    nf, nw = c_int64(), c_int64()
    L.orc_tank(ndims, dx, _dp(fs), _dp(ts), n_layers, _ip(fc), rho0, c, gamma, p_bg, _dp(acc),
               ctypes.byref(nf), ctypes.byref(nw), None, None, None, None, None, None)
    nf, nw = nf.value, nw.value
    out = dict(x_f=np.zeros((nf, ndims)), rho_f=np.zeros(nf), m_f=np.zeros(nf),
               x_w=np.zeros((nw, ndims)), rho_w=np.zeros(nw), m_w=np.zeros(nw))
    L.orc_tank(ndims, dx, _dp(fs), _dp(ts), n_layers, _ip(fc), rho0, c, gamma, p_bg, _dp(acc),
               ctypes.byref(c_int64()), ctypes.byref(c_int64()), _dp(out["x_f"]),
               _dp(out["rho_f"]), _dp(out["m_f"]), _dp(out["x_w"]), _dp(out["rho_w"]),
               _dp(out["m_w"]))
    return out


class Model:
    """The oracle's FP64 system pair: kick!, drift!, CK2N54 integration."""

    def __init__(self, cfg, x_w: np.ndarray, m_w: np.ndarray, m_f: np.ndarray):
        self.L = lib()
        self.cfg = cfg
        self.nd, self.nf, self.nw = cfg.ndims, cfg.n_fluid, cfg.n_wall
        self._keep = [np.ascontiguousarray(x_w, dtype=np.float64).reshape(-1),
                      np.ascontiguousarray(m_w, dtype=np.float64),
                      np.ascontiguousarray(m_f, dtype=np.float64)]
        self.h = self.L.orc_create(ctypes.byref(cfg), *[_dp(a) for a in self._keep])
        if not self.h:
            raise RuntimeError("oracle: bad configuration")

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def kick(self, v: np.ndarray, u: np.ndarray) -> tuple[np.ndarray, int]:
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        dv = np.zeros_like(v)
        st = self.L.orc_kick(self.h, _dp(dv), _dp(v), _dp(u))
        return dv, st

    def last_state(self):
        pf, pw, rw, vw = np.zeros(self.nf), np.zeros(self.nw), np.zeros(self.nw), np.zeros(self.nw)
        self.L.orc_last_state(self.h, _dp(pf), _dp(pw), _dp(rw), _dp(vw))
        return dict(p_f=pf, p_w=pw, rho_w=rw, vol_w=vw)

    def drift(self, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        du = np.zeros(self.nf * self.nd)
        self.L.orc_drift(self.h, _dp(du), _dp(v))
        return du

    def interpolate(self, v, u, points, smoothing_length, cut_off_bnd=True,
                    clip_negative_pressure=False, include_wall_velocity=False):
        """interpolate_points at `points` (n, nd): dict of computed_density, velocity (n, nd),
        pressure, density, neighbor_count."""
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1)
        pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, self.nd)
        n = pts.shape[0]
        cd, pr, de = np.zeros(n), np.zeros(n), np.zeros(n)
        ve = np.zeros((n, self.nd))
        cnt = np.zeros(n, dtype=np.int32)
        self.L.orc_interpolate(self.h, _dp(v), _dp(u), _dp(pts), n, smoothing_length,
                               int(cut_off_bnd), int(clip_negative_pressure),
                               int(include_wall_velocity), _dp(cd), _dp(ve), _dp(pr), _dp(de),
                               _ip(cnt))
        return dict(computed_density=cd, velocity=ve, pressure=pr, density=de,
                    neighbor_count=cnt)

    def integrate_spv(self, v: np.ndarray, u: np.ndarray, dt: float, n_steps: int):
        """SymplecticPositionVerlet steps (2 RHS evaluations per step)."""
        v = np.array(v, dtype=np.float64).reshape(-1)
        u = np.array(u, dtype=np.float64).reshape(-1)
        st = self.L.orc_integrate_spv(self.h, _dp(v), _dp(u), dt, n_steps)
        return v, u, st

    def integrate(self, v: np.ndarray, u: np.ndarray, dt: float, n_steps: int):
        v = np.array(v, dtype=np.float64).reshape(-1)
        u = np.array(u, dtype=np.float64).reshape(-1)
        st = self.L.orc_integrate_ck2n54(self.h, _dp(v), _dp(u), dt, n_steps)
        return v, u, st


def integrate_jvp(cfg, x_w, m_w, m_f, v, u, dt: float, n_steps: int, v_dir=None, u_dir=None):
    """Forward-mode derivatives (dual numbers through the oracle's own CK2N54 and right-hand
    side) of n_steps steps from (v, u): returns (v, u, dv, du, status) where dv[k], du[k] are the
    derivatives of the final state along direction k = Monaghan alpha, Molteni-Colagrossi delta,
    gravity magnitude, initial state along (v_dir, u_dir)."""
    L = lib()
    v = np.array(v, dtype=np.float64).reshape(-1)
    u = np.array(u, dtype=np.float64).reshape(-1)
    keep = [np.ascontiguousarray(x_w, dtype=np.float64).reshape(-1),
            np.ascontiguousarray(m_w, dtype=np.float64), np.ascontiguousarray(m_f, np.float64)]
    vd = None if v_dir is None else np.ascontiguousarray(v_dir, np.float64).reshape(-1)
    ud = None if u_dir is None else np.ascontiguousarray(u_dir, np.float64).reshape(-1)
    dv = np.zeros((4, v.size))
    du = np.zeros((4, u.size))
    null = ctypes.POINTER(c_double)()
    st = L.orc_integrate_ck2n54_jvp(ctypes.byref(cfg), *[_dp(a) for a in keep], _dp(v), _dp(u),
                                    _dp(vd) if vd is not None else null,
                                    _dp(ud) if ud is not None else null, dt, n_steps, _dp(dv),
                                    _dp(du))
    return v, u, dv, du, st


def nhs(cfg, x_f: np.ndarray, x_w: np.ndarray):
    L = lib()
    nf, nw = cfg.n_fluid, cfg.n_wall
    xf = np.ascontiguousarray(x_f, dtype=np.float64).reshape(-1)
    xw = np.ascontiguousarray(x_w, dtype=np.float64).reshape(-1)
    out = dict(cell=np.zeros(nf, np.int32), order=np.zeros(nf, np.int32),
               nnb_ff=np.zeros(nf, np.int32), nnb_fw=np.zeros(nf, np.int32),
               nnb_wf=np.zeros(nw, np.int32))
    st = L.orc_nhs(ctypes.byref(cfg), _dp(xf), _dp(xw), _ip(out["cell"]), _ip(out["order"]),
                   _ip(out["nnb_ff"]), _ip(out["nnb_fw"]), _ip(out["nnb_wf"]))
    return out, st


def sort_perm(cfg, x: np.ndarray) -> np.ndarray:
    """SortingCallback permutation of coordinates x (n, nd)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    perm = np.zeros(x.shape[0], dtype=np.int32)
    st = lib().orc_sort_perm(ctypes.byref(cfg), _dp(x.reshape(-1)), x.shape[0], _ip(perm))
    if st != 0:
        raise RuntimeError("oracle: bad configuration")
    return perm


def ck2n54_coefficients():
    A, B, C = (c_double * 5)(), (c_double * 5)(), (c_double * 5)()
    lib().orc_ck2n54_coefficients(A, B, C)
    return np.array(A), np.array(B), np.array(C)


def wendland_c2(nd, r, h):
    return lib().orc_wendland_c2(nd, r, h)


def wendland_c2_deriv_div_r(nd, r, h):
    return lib().orc_wendland_c2_deriv_div_r(nd, r, h)


def cole_pressure(c, rho0, gamma, p_bg, clip, rho):
    return lib().orc_cole_pressure(c, rho0, gamma, p_bg, int(clip), rho)


def cole_inverse(c, rho0, gamma, p_bg, p):
    return lib().orc_cole_inverse(c, rho0, gamma, p_bg, p)


def monaghan_pair(nd, h, c, alpha, beta, eps, pos_diff, v_a, v_b, m_b, rho_a, rho_b):
    pd = np.array(list(pos_diff) + [0.0] * (3 - len(pos_diff)))
    va = np.array(list(v_a) + [0.0] * (3 - len(v_a)))
    vb = np.array(list(v_b) + [0.0] * (3 - len(v_b)))
    out = np.zeros(3)
    lib().orc_monaghan_pair(nd, h, c, alpha, beta, eps, _dp(pd), _dp(va), _dp(vb), m_b, rho_a,
                            rho_b, _dp(out))
    return out[:nd]
