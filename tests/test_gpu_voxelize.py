"""GPU tests of dagc_voxelize: the reference (GL) rule array-equal to its CPU
restatement, the separating-axis rule equal to the host triangle-soup
generator voxel for voxel, and voxelize -> CreateDAG -> final DAG end to end."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from oracle.decode import decode_final

pytestmark = pytest.mark.gpu


def codes_of(t):
    return t.cpu().numpy().view(np.uint64)


@pytest.mark.parametrize("depth,n,size,box", [
    (8, 5000, 3.0, (0, 0, 0, 256, 256, 256)),            # small triangles, grid units
    (10, 2000, 60.0, (0, 0, 0, 1024, 1024, 1024)),       # large triangles
    (9, 3000, 0.2, (-1.5, 0.25, 3.0, 2.5, 4.75, 7.0)),   # scene units, non-cubic box
])
def test_gl_rule_matches_restatement(ctx, depth, n, size, box):
    rng = np.random.default_rng(depth)
    lo, hi = np.array(box[:3]), np.array(box[3:])
    tris = lo + (hi - lo) * rng.uniform(-0.05, 1.05, (n, 1, 3)) + np.concatenate(
        [np.zeros((n, 1, 3)), rng.normal(0, size, (n, 2, 3))], axis=1)
    gpu = codes_of(ctx.voxelize(tris, box, depth, D.VOXELIZE_GL))
    ref = O.voxelize_gl(tris, box, depth)
    assert gpu.size > n
    assert np.array_equal(gpu, ref)


def test_gl_rule_degenerate_and_axis_aligned(ctx):
    rng = np.random.default_rng(3)
    base = np.floor(rng.uniform(0, 60, (500, 1, 3))) + 0.5
    flat = base + np.stack([np.zeros((500, 3)), [4, 0, 0] * np.ones((500, 3)), [0, 5, 0] * np.ones((500, 3))], 1)
    line = base + np.stack([np.zeros((500, 3)), np.ones((500, 3)), 2 * np.ones((500, 3))], 1)
    tris = np.concatenate([flat, line])
    gpu = codes_of(ctx.voxelize(tris, (0, 0, 0, 64, 64, 64), 6, D.VOXELIZE_GL))
    assert np.array_equal(gpu, O.voxelize_gl(tris, (0, 0, 0, 64, 64, 64), 6))


@pytest.mark.parametrize("depth,n,seed", [(9, 20_000, 1), (11, 100_000, 2)])
def test_sat_rule_equals_soup_generator(ctx, depth, n, seed):
    tris = D.gen_soup_triangles(depth, seed, n)
    g = 1 << depth
    gpu = codes_of(ctx.voxelize(tris, (0, 0, 0, g, g, g), depth, D.VOXELIZE_SAT))
    host = D.gen_triangle_soup(depth, seed, n, threads=8)
    assert gpu.size == host.size
    assert np.array_equal(np.sort(gpu), np.sort(host))


def test_voxelize_then_compress_end_to_end(ctx):
    depth = 10
    tris = D.gen_soup_triangles(depth, 7, 30_000)
    frags = ctx.voxelize(tris, (0, 0, 0, 1024, 1024, 1024), depth, D.VOXELIZE_GL)
    dag = ctx.create_dag(frags, depth)  # straight from device memory
    words = ctx.create_final_dag(dag).to_numpy()
    codes = codes_of(frags)
    assert np.array_equal(decode_final(words, depth), np.unique(codes))
    assert np.array_equal(words, O.final_dag(O.create_dag(codes, depth)))


def test_capacity_too_small_reports_the_needed_count(ctx):
    tris = D.gen_soup_triangles(8, 3, 2000)
    full = codes_of(ctx.voxelize(tris, (0, 0, 0, 256, 256, 256), 8, D.VOXELIZE_SAT))
    with pytest.raises(D.DagcError) as e:
        ctx.voxelize(tris, (0, 0, 0, 256, 256, 256), 8, D.VOXELIZE_SAT, capacity=full.size - 1)
    assert e.value.status == D.ERR_TOO_LARGE
    exact = codes_of(ctx.voxelize(tris, (0, 0, 0, 256, 256, 256), 8, D.VOXELIZE_SAT, capacity=full.size))
    assert np.array_equal(exact, full)
    with pytest.raises(D.DagcError):
        ctx.voxelize(tris, (0, 0, 0, 256, 0, 256), 8)  # empty box
    assert codes_of(ctx.voxelize(np.zeros((0, 9)), (0, 0, 0, 1, 1, 1), 8)).size == 0
