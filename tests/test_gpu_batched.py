"""GPU tests of the batched form: many chunks in one call must equal the
per-chunk CreateDAG + MergeDAGs of the same chunks, bit for bit, and the
oracle's CreateDAG of the whole volume."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import random_codes
from tests.test_gpu_parity import assert_dag_equal

pytestmark = pytest.mark.gpu




def global_codes(local_chunks, morton, chunk_depth):
    parts = [(np.uint64(m) << np.uint64(3 * chunk_depth)) | c for c, m in zip(local_chunks, morton) if c.size]
    return np.concatenate(parts) if parts else np.zeros(0, np.uint64)


def per_chunk_merge(ctx, local_chunks, morton, chunk_depth, top_levels):
    slots = 8 ** top_levels
    by_slot = {int(m): c for c, m in zip(local_chunks, morton)}
    dags = [ctx.create_dag(by_slot.get(i, np.zeros(0, np.uint64)), chunk_depth) for i in range(slots)]
    return ctx.merge_dags(dags)


def make_chunks(chunk_depth, top_levels, k, seed):
    rng = np.random.default_rng(seed)
    morton = np.sort(rng.choice(8 ** top_levels, size=k, replace=False)).astype(np.uint64)
    chunks = []
    for i in range(k):
        n = int(rng.integers(0, 6000)) if i % 5 else 0  # some chunks empty, sizes uneven
        chunks.append(random_codes(chunk_depth, n, seed * 100 + i, cluster=bool(i % 2)))
    return chunks, morton


@pytest.mark.parametrize("chunk_depth,top_levels,k,seed", [(5, 2, 20, 1), (6, 1, 8, 2), (4, 3, 100, 3), (7, 1, 1, 4),
                                                          (8, 1, 6, 5)])
@pytest.mark.parametrize("path", [1, 0])
def test_batched_equals_per_chunk_merge_and_whole_volume(chunk_depth, top_levels, k, seed, path):
    """Both batched paths (1: persistent per-chunk leaves, 0: composite keys)
    equal the per-chunk CreateDAG + MergeDAGs and the oracle's whole volume."""
    chunks, morton = make_chunks(chunk_depth, top_levels, k, seed)
    counts = np.array([c.size for c in chunks], np.uint64)
    frag = np.concatenate(chunks) if counts.sum() else np.zeros(0, np.uint64)
    whole = O.create_dag(global_codes(chunks, morton, chunk_depth), chunk_depth + top_levels)
    with D.Context(0) as c:
        c.set_option(D.OPT_BATCH_PATH, path)
        batched = c.create_dag_batched(frag, counts, morton, chunk_depth, top_levels).to_host()
        merged = per_chunk_merge(c, chunks, morton, chunk_depth, top_levels).to_host()
    assert_dag_equal(batched, whole)
    assert_dag_equal(merged, whole)


@pytest.mark.parametrize("path", [1, 0])
def test_batched_large_uneven_chunks_depth_10(path):
    """Chunks of 1024^3 (the batched workload's chunk size) with uneven counts,
    several of them over many 8192-fragment tiles and 2048 bins, some empty:
    bit-exact against the oracle, called three times (graph replay)."""
    cd, top = 10, 1
    morton = np.arange(8, dtype=np.uint64)
    sizes = [0, 3, 9000, 250_000, 70_000, 0, 600_000, 17]
    chunks = [random_codes(cd, n, 100 + i, cluster=bool(i % 2)) for i, n in enumerate(sizes)]
    counts = np.array([c.size for c in chunks], np.uint64)
    frag = np.concatenate(chunks)
    whole = O.create_dag(global_codes(chunks, morton, cd), cd + top, threads=8)
    with D.Context(0) as c:
        c.set_option(D.OPT_BATCH_PATH, path)
        for _ in range(3):
            assert_dag_equal(c.create_dag_batched(frag, counts, morton, cd, top).to_host(), whole)


def test_batched_chunk_path_other_sizes_same_shape():
    """Same buffer, fragment count, chunk count and depths, but other chunk
    sizes: the recorded call sequence must follow the new sizes."""
    import torch
    cd, top = 10, 1
    rng = np.random.default_rng(13)
    total = 200_000
    frag = rng.integers(0, 1 << (3 * cd), total, dtype=np.uint64)
    d_frag = torch.from_numpy(frag.view(np.int64)).cuda()
    morton = np.arange(8, dtype=np.uint64)
    splits = [np.array([0, 10, 20, 30, 40, 50, 60, total - 210], np.uint64),
              np.array([total - 7 * 9000, 9000, 9000, 9000, 9000, 9000, 9000, 9000], np.uint64)]
    expect = []
    for counts in splits:
        parts = np.split(frag, np.cumsum(counts)[:-1].astype(np.int64))
        expect.append(O.create_dag(global_codes(parts, morton, cd), cd + top, threads=8))
    with D.Context(0) as c:
        for _ in range(3):
            for counts, ref in zip(splits, expect):
                assert_dag_equal(c.create_dag_batched(d_frag, counts, morton, cd, top).to_host(), ref)


@pytest.mark.parametrize("mode", [0, 2])
def test_batched_grouping_forms(mode):
    chunks, morton = make_chunks(5, 2, 20, 6)
    counts = np.array([c.size for c in chunks], np.uint64)
    frag = np.concatenate(chunks)
    whole = O.create_dag(global_codes(chunks, morton, 5), 7)
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, mode)
        assert_dag_equal(c.create_dag_batched(frag, counts, morton, 5, 2).to_host(), whole)


def test_batched_generator_terrain_chunks(ctx):
    """A reduced config-4 layout: 4x4 terrain chunks of 256^3 with sponges."""
    codes, counts, morton = D.gen_batched(chunk_depth=8, grid_xz=4, chunk_row=1, seed=11,
                                          min_fragments=1e3, max_fragments=3e5, threads=8)
    chunks = np.split(codes, np.cumsum(counts)[:-1].astype(np.int64))
    batched = ctx.create_dag_batched(codes, counts, morton, 8, 2)
    whole = O.create_dag(global_codes(chunks, morton, 8), 10, threads=8)
    assert_dag_equal(batched.to_host(), whole)
    words = ctx.create_final_dag(batched).to_numpy()
    assert np.array_equal(words, O.final_dag(whole))


@pytest.mark.parametrize("path", [1, 0])
@pytest.mark.parametrize("cd", [5, 9])
def test_batched_rejects_out_of_range_local_code(path, cd):
    chunks = [np.array([1, 2, 3], np.uint64), np.array([1 << (3 * cd)], np.uint64)]  # = 8^cd
    with D.Context(0) as c:
        c.set_option(D.OPT_BATCH_PATH, path)
        with pytest.raises(D.DagcError) as e:
            c.create_dag_batched(np.concatenate(chunks), [3, 1], [0, 5], cd, 1)
        assert e.value.status == D.ERR_BAD_INPUT


def test_batched_rejects_unordered_chunks(ctx):
    with pytest.raises(D.DagcError) as e:
        ctx.create_dag_batched(np.array([1, 2], np.uint64), [1, 1], [5, 3], 5, 1)
    assert e.value.status == D.ERR_INVALID_ARGUMENT


def test_batched_graph_key_includes_chunk_split(ctx):
    """Two batched calls on one fragment buffer with the same fragment count,
    chunk count and total depth but a different chunk/top split: a call shape
    is recorded as a CUDA graph on its second call and replayed after that, so
    each split is called three times in turn; every result must equal the
    oracle's for its own split."""
    import torch
    k = 8
    rng = np.random.default_rng(21)
    local = rng.integers(0, 8 ** 5, 4000, dtype=np.uint64)  # valid for chunk depth 5 and 6
    counts = np.full(k, local.size // k, np.uint64)
    d_frag = torch.from_numpy(local.view(np.int64)).cuda()
    chunks = np.split(local, k)
    splits = [(5, 2, np.arange(0, 64, 8, dtype=np.uint64)), (6, 1, np.arange(8, dtype=np.uint64))]
    expect = {cd: O.create_dag(global_codes(chunks, morton, cd), cd + top) for cd, top, morton in splits}
    for _ in range(3):
        for cd, top, morton in splits:
            got = ctx.create_dag_batched(d_frag, counts, morton, cd, top).to_host()
            assert_dag_equal(got, expect[cd])
