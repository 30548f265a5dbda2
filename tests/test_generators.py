"""CPU tests of the seeded synthetic fragment generators."""
import numpy as np

import dag_compression_fast_gb300 as D
from oracle.decode import decode_final  # noqa: F401  (imported to check the module loads)


def test_sphere_shell_config_small():
    a = D.gen_sphere_shell(7, 0xDA6C0DE)
    b = D.gen_sphere_shell(7, 0xDA6C0DE)
    assert np.array_equal(a, b)
    u = np.unique(a)
    assert 38_000 < u.size < 43_000          # ~40k shell voxels in a 128^3 grid
    assert 2.2 < a.size / u.size < 2.8       # each voxel emitted U{1..4} times
    assert a.max() < 1 << 21
    assert not np.array_equal(a, np.sort(a))  # shuffled


def test_terrain_small_depth():
    a = D.gen_terrain(8, 5)
    u = np.unique(a)
    assert u.size == 3 * 256 * 256             # three voxels per column
    assert a.max() < 1 << 24


def test_terrain_column_fraction():
    a = np.unique(D.gen_terrain(8, 5, 0.25))
    assert 0.2 * 3 * 65536 < a.size < 0.3 * 3 * 65536


def test_triangle_soup_thread_independent():
    a = D.gen_triangle_soup(10, 3, 2000, threads=1)
    b = D.gen_triangle_soup(10, 3, 2000, threads=3)
    assert np.array_equal(a, b)
    assert a.size > 2000 and a.max() < 1 << 30


def test_batched_chunks():
    codes, counts, morton = D.gen_batched(chunk_depth=8, grid_xz=2, chunk_row=1, seed=1,
                                          min_fragments=1e3, max_fragments=1e5, threads=2)
    assert counts.size == 4 and morton.size == 4
    assert counts.sum() == codes.size
    assert np.all(np.diff(morton.astype(np.int64)) > 0)
    assert codes.max() < 1 << 24
