"""Cameras and scenes shared by the tracer tests."""
import numpy as np

import dag_compression_fast_gb300 as D


def look_at(position, target, up_hint=(0.0, 1.0, 0.0)):
    """(right, up, forward) of a camera at `position` looking at `target`."""
    f = np.asarray(target, np.float64) - np.asarray(position, np.float64)
    f /= np.linalg.norm(f)
    r = np.cross(np.asarray(up_hint, np.float64), f)
    if np.linalg.norm(r) < 1e-9:
        r = np.cross((1.0, 0.0, 0.0), f)
    r /= np.linalg.norm(r)
    u = np.cross(f, r)
    return r, u, f


def camera(depth, position, target, width=64, height=48, fov=60.0, debug_level=D.TRACE_POSITION_COLORS):
    """Trace parameters for a camera in the unit box [0, 1]^3 of the volume."""
    r, u, f = look_at(position, target)
    return D.trace_camera(position, r, u, f, fov, width, height, (0, 0, 0), (1, 1, 1), depth, debug_level)


def axis_ray_params(depth, width=8, height=8):
    """Rays from outside the grid whose pixel (0, 0) runs exactly along +z
    (two zero direction components), the others slightly off axis."""
    side = float(1 << depth)
    p = D.TraceParams()
    p.debug_level = D.TRACE_POSITION_COLORS
    p.width, p.height = width, height
    c = side / 2 + 0.5
    p.camera[:] = (c, c, -side / 4)
    p.ray_min[:] = (c, c, 0.0)
    p.ray_ddx[:] = (0.75, 0.0, 0.0)
    p.ray_ddy[:] = (0.0, 0.75, 0.0)
    return p


def voxel_xyz(codes, depth):
    """Morton codes -> integer (x, y, z) (x = bit 2, y = bit 1, z = bit 0)."""
    codes = np.asarray(codes, np.uint64)
    xyz = np.zeros((codes.size, 3), np.int64)
    for b in range(depth):
        for a, sh in enumerate((2, 1, 0)):
            xyz[:, a] |= ((codes >> np.uint64(3 * b + sh)) & np.uint64(1)).astype(np.int64) << b
    return xyz
