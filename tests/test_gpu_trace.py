"""GPU tests of dagc_trace: colours and hit voxels bit-exact with the tracer's
CPU restatement, on final DAGs built by the GPU path; malformed input is
rejected without reading outside the word array."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import random_codes
from tests.trace_scenes import axis_ray_params, camera

pytestmark = pytest.mark.gpu

MISS = np.uint64(0xFFFFFFFFFFFFFFFF)

SCENES = {
    "sphere_d7": lambda: (D.gen_sphere_shell(7, 0xDA6C0DE), 7),
    "terrain_d9": lambda: (D.gen_terrain(9, 3), 9),
    "sparse_d10": lambda: (random_codes(10, 20_000, 5, cluster=False), 10),
    "soup_d9": lambda: (D.gen_triangle_soup(9, 5, 2000, threads=4), 9),
}
CAMERAS = [
    ((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), 64, 48),     # outside, looking at the centre
    ((1.7, 1.4, 1.9), (0.4, 0.45, 0.5), 57, 33),     # outside, odd image size
    ((0.52, 0.61, 0.47), (0.9, 0.2, 0.1), 40, 40),   # inside the volume
]


@pytest.mark.parametrize("scene", sorted(SCENES))
@pytest.mark.parametrize("cam", range(len(CAMERAS)))
def test_trace_bit_exact_with_oracle(ctx, scene, cam):
    codes, depth = SCENES[scene]()
    words = ctx.create_final_dag(ctx.create_dag(codes, depth))
    host_words = words.to_numpy()
    pos, target, w, h = CAMERAS[cam]
    for debug in (D.TRACE_POSITION_COLORS, 0, 2):
        p = camera(depth, pos, target, width=w, height=h, debug_level=debug)
        colors, hits = ctx.trace(words, depth, p)
        ref_c, ref_h, bad = O.trace(host_words, depth, p)
        assert bad == 0
        assert np.array_equal(hits, ref_h)
        assert np.array_equal(colors, ref_c)
    hit = hits[hits != MISS]
    assert np.isin(hit, np.unique(codes)).all()  # every hit is an input voxel


def test_trace_axis_aligned_rays(ctx):
    codes = random_codes(6, 20_000, 8, cluster=False)
    words = ctx.create_final_dag(ctx.create_dag(codes, 6))
    p = axis_ray_params(6, width=16, height=16)
    colors, hits = ctx.trace(words, 6, p)
    ref_c, ref_h, _ = O.trace(words.to_numpy(), 6, p)
    assert np.array_equal(hits, ref_h) and np.array_equal(colors, ref_c)


def test_trace_full_terrain_frame(ctx):
    """A 1280x720 frame of the 2048^3 terrain."""
    codes = D.gen_terrain(11, 0xDA6C0DE + 2)
    words = ctx.create_final_dag(ctx.create_dag(codes, 11))
    p = camera(11, (0.1, 0.5, -0.4), (0.6, 0.2, 0.7), width=1280, height=720)
    colors, hits = ctx.trace(words, 11, p)
    ref_c, ref_h, _ = O.trace(words.to_numpy(), 11, p, threads=16)
    assert np.array_equal(hits, ref_h) and np.array_equal(colors, ref_c)
    assert (hits != MISS).mean() > 0.1


def test_trace_rejects_malformed_words(ctx):
    codes = random_codes(8, 5000, 9)
    words = ctx.create_final_dag(ctx.create_dag(codes, 8)).to_numpy()
    p = camera(8, (0.5, 0.5, -1.2), (0.5, 0.5, 0.5), width=32, height=32)
    with pytest.raises(D.DagcError) as e:
        ctx.trace(words[: words.size // 4], 8, p)  # pointers run past the end
    assert e.value.status == D.ERR_BAD_INPUT
    rng = np.random.default_rng(1)
    junk = rng.integers(0, words.size, words.size, dtype=np.uint32)  # pointers inside, nonsense content
    try:
        ctx.trace(junk, 8, p)
    except D.DagcError as err:
        assert err.status == D.ERR_BAD_INPUT
    with pytest.raises(D.DagcError):
        ctx.trace(words, 2, p)
