"""interpolate_points / interpolate_line / interpolate_plane_2d / interpolate_plane_3d
(src/general/interpolation.jl:56-322, 381-697, 787-824) and the pressure
sensors of the 2D dam-break validation (validation/dam_break_2d/sensors.jl:5-18), through the
library's tp_interpolate_points."""
from __future__ import annotations

import ctypes

import numpy as np


def interpolate_points(point_coords, semi, ref_system, v_ode, u_ode, *, smoothing_length=None,
                       cut_off_bnd=True, clip_negative_pressure=False,
                       include_wall_velocity=False) -> dict:
    """SPH interpolation of the fluid fields at `point_coords` ((ndims, n) array: the i-th
    column holds point i, as in the reference).  Returns a dict of numpy arrays with the
    reference's NamedTuple fields: computed_density, point_coords, neighbor_count, velocity
    ((ndims, n)), pressure, density."""
    import torch

    if ref_system is not semi.fluid:
        raise ValueError("ArgumentError: the reference system must be the fluid system")
    semi._ensure_handle()
    nd = semi.ndims
    pts = np.asarray(point_coords, dtype=np.float64)
    if pts.ndim == 1:
        pts = pts.reshape(nd, 1)
    if pts.shape[0] != nd:
        raise ValueError(f"ArgumentError: point_coords must have {nd} rows")
    n = pts.shape[1]
    h = semi.fluid.smoothing_length if smoothing_length is None else float(smoothing_length)
    dev = semi.device
    p_t = torch.as_tensor(np.ascontiguousarray(pts.T).reshape(-1), device=dev)
    cd = torch.empty(n, dtype=torch.float64, device=dev)
    vel = torch.empty(n * nd, dtype=torch.float64, device=dev)
    pr = torch.empty(n, dtype=torch.float64, device=dev)
    de = torch.empty(n, dtype=torch.float64, device=dev)
    cnt = torch.empty(n, dtype=torch.int32, device=dev)
    semi._set_stream()
    semi._call("tp_interpolate_points", v_ode.data_ptr(), u_ode.data_ptr(), p_t.data_ptr(),
               ctypes.c_int64(n), ctypes.c_double(h), int(cut_off_bnd),
               int(clip_negative_pressure), int(include_wall_velocity), cd.data_ptr(),
               vel.data_ptr(), pr.data_ptr(), de.data_ptr(), cnt.data_ptr())
    semi.sync()
    return dict(computed_density=cd.cpu().numpy(), point_coords=pts.copy(),
                neighbor_count=cnt.cpu().numpy(),
                velocity=vel.cpu().numpy().reshape(n, nd).T.copy(), pressure=pr.cpu().numpy(),
                density=de.cpu().numpy())


def line_points(start, end_, n_points: int, endpoint: bool = True) -> np.ndarray:
    """The (ndims, n) points of range(start, end_, length=n_points) (without the two end points
    when endpoint=false), interpolation.jl:393-403."""
    a = np.asarray(start, dtype=np.float64)
    b = np.asarray(end_, dtype=np.float64)
    t = np.arange(n_points, dtype=np.float64) / (n_points - 1)
    pts = (1.0 - t)[None, :] * a[:, None] + t[None, :] * b[:, None]
    if not endpoint:
        pts = pts[:, 1:-1]
    return pts


def interpolate_line(start, end_, n_points, semi, ref_system, v_ode, u_ode, *, endpoint=True,
                     include_wall_velocity=False, smoothing_length=None, cut_off_bnd=True,
                     clip_negative_pressure=False) -> dict:
    """interpolate_points along `n_points` equidistant points from `start` to `end_`."""
    return interpolate_points(line_points(start, end_, n_points, endpoint), semi, ref_system,
                              v_ode, u_ode, smoothing_length=smoothing_length,
                              cut_off_bnd=cut_off_bnd,
                              clip_negative_pressure=clip_negative_pressure,
                              include_wall_velocity=include_wall_velocity)


def _keep_points_with_neighbors(res: dict) -> dict:
    """Drop the points without fluid neighbours from every field (interpolation.jl:211-223)."""
    keep = np.nonzero(res["neighbor_count"] > 0)[0]
    return {k: (x[keep] if x.ndim == 1 else x[:, keep]) for k, x in res.items()}


def plane_points_2d(min_corner, max_corner, resolution) -> np.ndarray:
    """The (2, n) grid of interpolate_plane_2d (interpolation.jl:183-209): ceil((max - min) /
    resolution) + 1 points per axis, the first on `min_corner`, spaced by `resolution`, x
    fastest (rectangular_shape_coords with place_on_shell, rectangular_shape.jl:198-224)."""
    lo = np.asarray(min_corner, dtype=np.float64)
    hi = np.asarray(max_corner, dtype=np.float64)
    if lo.shape != (2,) or hi.shape != (2,):
        raise ValueError("ArgumentError: function is intended for 2D coordinates only")
    if np.any(lo > hi):
        raise ValueError("ArgumentError: `min_corner` should be smaller than `max_corner` in "
                         "every dimension")
    s = float(resolution)
    n = np.ceil((hi - lo) / s).astype(int) + 1
    iy, ix = np.meshgrid(np.arange(1, n[1] + 1), np.arange(1, n[0] + 1), indexing="ij")
    idx = np.stack([ix.ravel(), iy.ravel()])
    return (lo - 0.5 * s)[:, None] + s * (idx - 0.5)


def interpolate_plane_2d(min_corner, max_corner, resolution, semi, ref_system, v_ode, u_ode, *,
                         include_wall_velocity=False, smoothing_length=None, cut_off_bnd=True,
                         clip_negative_pressure=False) -> dict:
    """interpolate_points on the grid of plane_points_2d, points without fluid neighbours
    removed (interpolation.jl:73-87, 183-225)."""
    res = interpolate_points(plane_points_2d(min_corner, max_corner, resolution), semi,
                             ref_system, v_ode, u_ode, smoothing_length=smoothing_length,
                             cut_off_bnd=cut_off_bnd,
                             clip_negative_pressure=clip_negative_pressure,
                             include_wall_velocity=include_wall_velocity)
    return _keep_points_with_neighbors(res)


def face_points(point1, point2, point3, resolution) -> np.ndarray:
    """The (3, n) points of the parallelogram spanned by point2 - point1 and point3 - point1,
    ceil(|edge| / resolution) + 1 points per edge, the second edge fastest
    (sample_face_with_fixed_size, interpolation.jl:787-824)."""
    p1, p2, p3 = (np.asarray(p, dtype=np.float64) for p in (point1, point2, point3))
    if p1.shape != (3,) or p2.shape != (3,) or p3.shape != (3,):
        raise ValueError("ArgumentError: all points must be 3D coordinates")
    e1, e2 = p2 - p1, p3 - p1
    if abs(np.linalg.norm(np.cross(e1, e2))) <= np.finfo(np.float64).eps:
        raise ValueError("ArgumentError: the vectors `AB` and `AC` must not be collinear")
    n1 = int(np.ceil(np.linalg.norm(e1) / resolution))
    n2 = int(np.ceil(np.linalg.norm(e2) / resolution))
    i, j = np.meshgrid(np.arange(n1 + 1), np.arange(n2 + 1), indexing="ij")
    a = (i.ravel() / n1)[None, :]
    b = (j.ravel() / n2)[None, :]
    return (p1[:, None] + a * e1[:, None]) + b * e2[:, None]


def interpolate_plane_3d(point1, point2, point3, resolution, semi, ref_system, v_ode, u_ode, *,
                         include_wall_velocity=False, smoothing_length=None, cut_off_bnd=True,
                         clip_negative_pressure=False) -> dict:
    """interpolate_points on the points of face_points, points without fluid neighbours removed
    (interpolation.jl:295-322)."""
    if semi.ndims != 3:
        raise ValueError("ArgumentError: `interpolate_plane_3d` requires a 3D simulation")
    res = interpolate_points(face_points(point1, point2, point3, resolution), semi, ref_system,
                             v_ode, u_ode, smoothing_length=smoothing_length,
                             cut_off_bnd=cut_off_bnd,
                             clip_negative_pressure=clip_negative_pressure,
                             include_wall_velocity=include_wall_velocity)
    return _keep_points_with_neighbors(res)


def interpolated_pressure(coord_top, coord_bottom, v_ode, u_ode, semi) -> float:
    """The validation pressure sensor: mean clipped pressure over 10 points of the segment,
    interpolated with twice the initial smoothing length and no boundary cut-off; points
    without fluid count as zero (sensors.jl:5-18)."""
    r = interpolate_line(coord_top, coord_bottom, 10, semi, semi.fluid, v_ode, u_ode,
                         smoothing_length=2.0 * semi.fluid.smoothing_length,
                         clip_negative_pressure=True, cut_off_bnd=False)
    p = np.where(np.isnan(r["pressure"]), 0.0, r["pressure"])
    return float(p.sum() / 10)


def dam_break_sensor_segments(H: float, tank_length: float):
    """(top, bottom) of the pressure sensors P1-P4 on the right tank wall of the 2D dam break
    (validation/dam_break_2d/setup_marrone_2011.jl:47-73)."""
    size = 0.0084
    out = []
    for mm in (6.0, 30.0, 60.0, 160.0):
        top = (mm + 4.2) / 600 * H
        out.append(((tank_length, top), (tank_length, top - size)))
    return out
