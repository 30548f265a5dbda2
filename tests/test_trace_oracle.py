"""CPU checks of the tracer's restatement (the checker of dagc_trace): hits
are input voxels, and they are the first voxel along the ray by an exact
slab test over every voxel (brute force, double precision)."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import random_codes
from tests.trace_scenes import axis_ray_params, camera, voxel_xyz


def ray_dirs(p):
    """The rays the tracer sets up (src/DAGTracer.cu:310-318), float32 directions."""
    xs, ys = np.meshgrid(np.arange(p.width, dtype=np.float64), np.arange(p.height, dtype=np.float64))
    v = [np.asarray(p.ray_min[a]) + xs * p.ray_ddx[a] + ys * p.ray_ddy[a] - p.camera[a] for a in range(3)]
    s = 1.0 / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
    return [(s * v[a]).astype(np.float32).astype(np.float64) for a in range(3)]


def brute_spans(p, codes, depth):
    """Per ray and voxel, the parameter span [t0, t1] inside the voxel (t0 > t1: not crossed)."""
    xyz = voxel_xyz(codes, depth).astype(np.float64)
    o = np.array([np.float32(p.camera[a]) for a in range(3)], np.float64)
    d = ray_dirs(p)
    t0 = np.full((p.height, p.width, xyz.shape[0]), -np.inf)
    t1 = np.full((p.height, p.width, xyz.shape[0]), np.inf)
    with np.errstate(divide="ignore", invalid="ignore"):
        for a in range(3):
            da = d[a][..., None]
            lo = (xyz[None, None, :, a] - o[a]) / da
            hi = (xyz[None, None, :, a] + 1 - o[a]) / da
            inside = (o[a] >= xyz[None, None, :, a]) & (o[a] <= xyz[None, None, :, a] + 1)
            t0 = np.maximum(t0, np.where(da == 0, np.where(inside, -np.inf, np.inf), np.minimum(lo, hi)))
            t1 = np.minimum(t1, np.where(da == 0, np.where(inside, np.inf, -np.inf), np.maximum(lo, hi)))
    return np.maximum(t0, 0.0), t1


@pytest.mark.parametrize("seed,depth,n", [(1, 5, 400), (2, 6, 1500)])
def test_oracle_first_hit_matches_brute_force(seed, depth, n):
    codes = np.unique(random_codes(depth, n, seed, cluster=True))
    words = O.final_dag(O.create_dag(codes, depth))
    p = camera(depth, (1.6, 1.3, -0.7), (0.45, 0.5, 0.55), width=40, height=30)
    colors, hits, bad = O.trace(words, depth, p)
    assert bad == 0
    t0, t1 = brute_spans(p, codes, depth)
    crossed = t1 - t0 > 1e-3  # entered for more than a graze
    ent = np.where(t0 <= t1, t0, np.inf)
    best = np.where(crossed, t0, np.inf).min(axis=2)
    index = {int(c): i for i, c in enumerate(codes)}
    miss = hits == np.uint64(0xFFFFFFFFFFFFFFFF)
    assert (~miss).sum() > 50 and miss.sum() > 50
    for y in range(p.height):
        for x in range(p.width):
            if miss[y, x]:
                assert not crossed[y, x].any()  # a miss crosses no voxel
                continue
            i = index[int(hits[y, x])]  # the hit is an input voxel the ray touches...
            assert np.isfinite(ent[y, x, i])
            assert ent[y, x, i] <= best[y, x] + 1e-3  # ... and no voxel is entered before it


def test_axis_aligned_rays_run_with_infinite_inverse():
    depth = 5
    codes = np.unique(random_codes(depth, 3000, 7, cluster=False))
    words = O.final_dag(O.create_dag(codes, depth))
    p = axis_ray_params(depth)
    colors, hits, bad = O.trace(words, depth, p)
    assert bad == 0
    # Pixel (0, 0) runs along +z through column (16, 16): its hit is the
    # lowest-z input voxel of that column, if any.
    xyz = voxel_xyz(codes, depth)
    col = xyz[(xyz[:, 0] == 16) & (xyz[:, 1] == 16)]
    if col.size:
        z = col[:, 2].min()
        expect = [c for c, v in zip(codes, xyz) if v[0] == 16 and v[1] == 16 and v[2] == z][0]
        assert hits[0, 0] == expect
    else:
        assert hits[0, 0] == np.uint64(~np.uint64(0))


def test_position_colours_and_debug_colours():
    depth = 6
    codes = D.gen_sphere_shell(6, 3) if hasattr(D, "gen_sphere_shell") else random_codes(depth, 2000, 3)
    codes = np.unique(codes)
    words = O.final_dag(O.create_dag(codes, depth))
    p = camera(depth, (0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=24, height=24)
    colors, hits, bad = O.trace(words, depth, p)
    xyz = voxel_xyz(hits[hits != np.uint64(~np.uint64(0))], depth)
    c = colors[hits != np.uint64(~np.uint64(0))]
    assert np.array_equal(c & 0xFF, xyz[:, 0] & 0xFF)
    assert np.array_equal((c >> 8) & 0xFF, xyz[:, 1] & 0xFF)
    assert np.array_equal((c >> 16) & 0xFF, xyz[:, 2] & 0xFF)
    assert np.all(colors[hits == np.uint64(~np.uint64(0))] == 0)
    p.debug_level = 0
    dcol, dhits, _ = O.trace(words, depth, p)
    assert np.array_equal(dhits, hits)
    assert len(np.unique(dcol[hits != np.uint64(~np.uint64(0))])) > 1


def test_truncated_words_are_reported():
    depth = 5
    codes = np.unique(random_codes(depth, 500, 4))
    words = O.final_dag(O.create_dag(codes, depth))
    p = camera(depth, (0.5, 0.5, -1.5), (0.5, 0.5, 0.5), width=16, height=16)
    _, _, bad = O.trace(words[: words.size // 3], depth, p)
    assert bad > 0


def test_trace_camera_maps_box_to_grid():
    p = camera(8, (0.5, 0.5, -1.0), (0.5, 0.5, 0.5), width=10, height=10)
    assert np.allclose(list(p.camera), [128.0, 128.0, -256.0])
    assert p.width == 10 and p.height == 10
    with pytest.raises(D.DagcError):
        D.trace_camera((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), 60, 0, 10, (0, 0, 0), (1, 1, 1), 8)
