"""Differentiation form: gradients of a CarpenterKennedy2N54 trajectory through the library's
hand-written adjoint (tp_adjoint_forward / tp_adjoint_backward of the C ABI).

`Trajectory` is the rrule of `solve`: the forward records checkpoints on the device, the
pullback maps cotangents of the final (v, u) to cotangents of the initial (v0, u0) and of the
parameters (Monaghan alpha, Molteni-Colagrossi delta, gravity magnitude).  `SolveCK2N54` wraps
the same pair as a torch.autograd.Function.  The loss helpers define the free-surface height
objective of the differentiated dam break: the mean final height of the particles that formed
the fluid's top layer at t = 0.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi

PARAMS = ("alpha", "delta", "gravity")


class Trajectory:
    """Forward solve with checkpoints plus its pullback (one Semidiscretization)."""

    def __init__(self, semi, v0, u0, *, dt: float, n_steps: int, checkpoint_every: int = 25):
        semi._ensure_handle()
        if semi._lib is None:
            raise RuntimeError("the CUDA library is not loaded")
        self.semi = semi
        self.dt = float(dt)
        self.n_steps = int(n_steps)
        self.checkpoint_every = int(checkpoint_every)
        self.v = v0.detach().clone().contiguous()
        self.u = u0.detach().clone().contiguous()
        semi._set_stream()
        semi._call("tp_adjoint_forward", self.v.data_ptr(), self.u.data_ptr(),
                   ctypes.c_double(self.dt), ctypes.c_int64(self.n_steps),
                   ctypes.c_int64(self.checkpoint_every))

    def pullback(self, v_bar, u_bar):
        """(v_bar, u_bar) of the final state -> (v0_bar, u0_bar, {param: gradient})."""
        vb = v_bar.detach().clone().to(self.v.dtype).contiguous()
        ub = u_bar.detach().clone().to(self.u.dtype).contiguous()
        out = (ctypes.c_double * 3)()
        self.semi._set_stream()
        self.semi._call("tp_adjoint_backward", vb.data_ptr(), ub.data_ptr(), out)
        return vb, ub, dict(zip(PARAMS, list(out)))


def top_layer_indices(tank) -> np.ndarray:
    """Fluid particles of the initial top layer (within half a spacing of the highest one)."""
    y = tank.fluid.coordinates[:, 1]
    return np.nonzero(y >= y.max() - 0.5 * tank.fluid.particle_spacing)[0]


def surface_height_loss(u, idx, ndims: int):
    """Mean height (coordinate 1) of the particles `idx` in the flat u (ndims, n) layout, and its
    gradient with respect to u as a flat array of u's shape."""
    import torch

    uu = u.view(-1, ndims)
    sel = torch.as_tensor(idx, device=u.device, dtype=torch.long)
    loss = uu[sel, 1].mean()
    grad = torch.zeros_like(uu)
    grad[sel, 1] = 1.0 / len(idx)
    return loss, grad.view(-1)


def _make_function():
    import torch

    class SolveCK2N54(torch.autograd.Function):
        """(v0, u0) -> (v_T, u_T) with the library adjoint as the backward.  The parameter
        gradients of the last backward are left in `ctx.params_bar` of the trajectory (the
        parameters live in the Semidiscretization, not in tensors)."""

        @staticmethod
        def forward(ctx, v0, u0, semi, dt, n_steps, checkpoint_every):
            traj = Trajectory(semi, v0, u0, dt=dt, n_steps=n_steps,
                              checkpoint_every=checkpoint_every)
            ctx.traj = traj
            return traj.v.clone(), traj.u.clone()

        @staticmethod
        def backward(ctx, v_bar, u_bar):
            vb, ub, params = ctx.traj.pullback(v_bar, u_bar)
            ctx.traj.params_bar = params
            return vb, ub, None, None, None, None

    return SolveCK2N54


_fn = None


def solve_ck2n54(v0, u0, semi, dt: float, n_steps: int, checkpoint_every: int = 25):
    """Differentiable solve (torch.autograd) through the library adjoint."""
    global _fn
    if _fn is None:
        _fn = _make_function()
    return _fn.apply(v0, u0, semi, dt, n_steps, checkpoint_every)


def check_library(lib) -> None:
    """Raises if the loaded library lacks the differentiation entry points."""
    for name in ("tp_adjoint_forward", "tp_adjoint_backward"):
        if not hasattr(lib, name):
            raise _abi.TpError(f"library lacks {name}")
