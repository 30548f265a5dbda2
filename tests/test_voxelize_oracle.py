"""CPU checks of the voxelizer's GL-rule restatement (the checker of
dagc_voxelize's reference mode) on cases with known answers."""
import numpy as np

from oracle import oracle as O
from tests.trace_scenes import voxel_xyz


def quad(z, lo, hi):
    """Two triangles covering [lo, hi]^2 in the plane z (grid units)."""
    a, b, c, d = (lo, lo, z), (hi, lo, z), (hi, hi, z), (lo, hi, z)
    return np.array([[a, b, c], [a, c, d]], np.float64)


def test_axis_plane_quad_covers_its_columns():
    depth = 5
    codes = O.voxelize_gl(quad(10.3, 4.25, 12.75), (0, 0, 0, 32, 32, 32), depth)
    xyz = voxel_xyz(codes, depth)
    assert np.all(xyz[:, 2] == 10)  # every fragment in the plane's cell
    # Conservative coverage: columns 4..12 in x and y (touching counts).
    assert set(map(tuple, xyz[:, :2])) == {(x, y) for x in range(4, 13) for y in range(4, 13)}


def test_dominant_axis_and_swizzle():
    depth = 5
    box = (0, 0, 0, 32, 32, 32)
    # Facing +x: projected on the (z, y) view, depth = x.
    tri = np.array([[[7.5, 2.2, 2.2], [7.5, 9.8, 2.2], [7.5, 2.2, 9.8]]], np.float64)
    xyz = voxel_xyz(O.voxelize_gl(tri, box, depth), depth)
    assert np.all(xyz[:, 0] == 7) and len(xyz) > 10
    # Facing +y: depth = y.
    tri = np.array([[[2.2, 20.5, 2.2], [9.8, 20.5, 2.2], [2.2, 20.5, 9.8]]], np.float64)
    xyz = voxel_xyz(O.voxelize_gl(tri, box, depth), depth)
    assert np.all(xyz[:, 1] == 20) and len(xyz) > 10


def test_sloped_triangle_takes_the_smallest_depth_over_each_pixel():
    depth = 6
    # z = 0.5 x + 3: over pixel column x the plane spans z in [0.5x + 3,
    # 0.5x + 3.5]; the fragment sits at the lower end.
    tri = np.array([[[1.0, 1.0, 3.5], [41.0, 1.0, 23.5], [1.0, 41.0, 3.5]]], np.float64)
    xyz = voxel_xyz(O.voxelize_gl(tri, (0, 0, 0, 64, 64, 64), depth), depth)
    interior = (xyz[:, 0] >= 2) & (xyz[:, 1] >= 2) & (xyz[:, 0] + xyz[:, 1] <= 38)
    assert interior.sum() > 100
    x = xyz[interior, 0]
    assert np.all(xyz[interior, 2] == np.floor(0.5 * x + 3.0).astype(np.int64))


def test_degenerate_and_outside_triangles_emit_nothing():
    box = (0, 0, 0, 16, 16, 16)
    line = np.array([[[1, 1, 1], [5, 5, 5], [9, 9, 9]]], np.float64)
    point = np.array([[[3, 3, 3], [3, 3, 3], [3, 3, 3]]], np.float64)
    outside = np.array([[[20, 20, 1], [30, 20, 1], [20, 30, 1]]], np.float64)
    for t in (line, point, outside):
        assert O.voxelize_gl(t, box, 4).size == 0


def test_scene_box_maps_onto_the_grid():
    depth = 4
    tris = quad(10.3, 4.25, 12.75)
    a = O.voxelize_gl(tris, (0, 0, 0, 16, 16, 16), depth)
    b = O.voxelize_gl(tris / 2.0 - 2.0, (-2, -2, -2, 6, 6, 6), depth)  # same scene, scene units
    assert np.array_equal(a, b)
