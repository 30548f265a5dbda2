"""GPU parity tests: the CUDA path (through the dagc C ABI) against the CPU
oracle, bit-exact, on seeded inputs, edge cases and full-size workloads."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from oracle.decode import decode_final
from tests.inputs import chunks_of, random_codes

pytestmark = pytest.mark.gpu


def assert_dag_equal(gpu: D.HostDag, ref: O.Dag):
    assert gpu.num_levels == ref.num_levels
    assert gpu.level_sizes() == ref.level_sizes()
    assert np.array_equal(gpu.leaves, ref.leaves)
    for l in range(ref.num_levels):
        assert np.array_equal(gpu.hashes[l], ref.hashes[l]), f"hashes of level {l}"
        assert np.array_equal(gpu.masks[l], ref.masks[l]), f"masks of level {l}"
        assert np.array_equal(gpu.children[l], ref.children[l]), f"children of level {l}"


def clustered_codes(depth, n, seed):
    return random_codes(depth, n, seed, cluster=True)


# ------------------------------------------------------------------ sort ----
@pytest.mark.parametrize("n", [1, 2, 100, 4095, 4096, 4097, 65_537, 1_000_003])
@pytest.mark.parametrize("lo,hi", [(0, 64), (6, 33), (0, 3), (61, 64)])
def test_sort_keys_matches_stable_numpy(ctx, n, lo, hi):
    rng = np.random.default_rng(n * 131 + lo)
    k = rng.integers(0, 2**64 - 1, n, dtype=np.uint64)
    if n > 10:
        k[: n // 3] = k[0]  # long runs of one key
    out = ctx.sort_keys(k, lo, hi).cpu().numpy().view(np.uint64)
    mask = np.uint64((1 << (hi - lo)) - 1) if hi - lo < 64 else np.uint64(2**64 - 1)
    expect = k[np.argsort((k >> np.uint64(lo)) & mask, kind="stable")]
    assert np.array_equal(out, expect)


def test_sort_keys_past_2_30_keys(ctx):
    """1.2e9 keys, more than 2^30: the digit passes' look-back prefixes pass
    2^30 (a count + 1 in 31 bits); the result equals torch's stable sort on
    the same bits."""
    import torch
    n = 1_200_000_000
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    k = torch.randint(0, 2**62, (n,), dtype=torch.int64, device="cuda", generator=g)
    out = ctx.sort_keys(k, 0, 32)
    order = torch.sort(k & 0xFFFFFFFF, stable=True).indices
    assert torch.equal(out, k[order])


def test_key_count_limit(ctx):
    """At most 2^31 - 2 keys (fragments) per call, checked before any
    pointer: one more is TOO_LARGE, the limit itself passes the size check."""
    L = D.lib()
    assert L.dagc_sort_keys(ctx.handle, None, None, 2**31 - 1, 0, 64, None) == D.ERR_TOO_LARGE
    assert L.dagc_sort_keys(ctx.handle, None, None, 2**31 - 2, 0, 64, None) == D.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("n", [1, 5000, 300_001])
def test_sort_pairs_iota_is_stable_permutation(ctx, n):
    rng = np.random.default_rng(n)
    k = rng.integers(0, 1000, n, dtype=np.uint64)  # many ties
    keys, vals = ctx.sort_pairs(k)
    keys = keys.cpu().numpy().view(np.uint64)
    vals = vals.cpu().numpy().view(np.uint32)
    order = np.argsort(k, kind="stable")
    assert np.array_equal(keys, k[order])
    assert np.array_equal(vals, order.astype(np.uint32))


# ------------------------------------------------------------ CreateDAG ----
CASES = {
    "sphere_d7": lambda: (D.gen_sphere_shell(7, 0xDA6C0DE), 7),
    "terrain_d8": lambda: (D.gen_terrain(8, 3), 8),
    "random_dense_d5": lambda: (random_codes(5, 50_000, 1), 5),
    "clustered_d10": lambda: (clustered_codes(10, 200_000, 2), 10),
    "tiny_d3": lambda: (np.array([69, 0, 69, 5], np.uint64), 3),
    "depth2": lambda: (np.array([0, 63, 7, 7], np.uint64), 2),
    "single": lambda: (np.array([12345], np.uint64), 9),
    "all_duplicates": lambda: (np.full(100_000, 777, np.uint64), 6),
    "sparse_d21": lambda: (np.random.default_rng(4).integers(0, 2**63, 20_000, dtype=np.uint64), 21),
    "soup_d10": lambda: (D.gen_triangle_soup(10, 5, 3000, threads=4), 10),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_create_dag_bit_exact(ctx, case):
    codes, depth = CASES[case]()
    ref = O.create_dag(codes, depth)
    dag = ctx.create_dag(codes, depth)
    assert_dag_equal(dag.to_host(), ref)
    words = ctx.create_final_dag(dag)
    w = words.to_numpy()
    assert np.array_equal(w, O.final_dag(ref))
    assert np.array_equal(decode_final(w, depth), np.unique(codes))


@pytest.mark.parametrize("case", ["sphere_d7", "clustered_d10", "all_duplicates", "sparse_d21", "depth2"])
def test_radix_form_bit_exact(case):
    """The radix-sort form of the level dedup (option off) gives the same DAG."""
    codes, depth = CASES[case]()
    with D.Context(0) as c:
        c.set_option(D.OPT_DEDUP, 0)
        dag = c.create_dag(codes, depth)
        assert_dag_equal(dag.to_host(), O.create_dag(codes, depth))
        assert c.dedup_fallbacks() == 0


@pytest.mark.parametrize("mode", [0, 2])
@pytest.mark.parametrize("case", ["sphere_d7", "terrain_d8", "clustered_d10", "all_duplicates", "sparse_d21",
                                  "depth2", "tiny_d3", "soup_d10"])
def test_grouping_forms_bit_exact(mode, case):
    """Fragments grouped by the radix sort (0) or by the hash table (2, forced
    even where the sketch would not choose it) give the same DAG."""
    codes, depth = CASES[case]()
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, mode)
        dag = c.create_dag(codes, depth)
        assert_dag_equal(dag.to_host(), O.create_dag(codes, depth))
        w = c.create_final_dag(dag).to_numpy()
        assert np.array_equal(decode_final(w, depth), np.unique(codes))


def test_forced_grouping_with_overfull_tables_reruns():
    """Grouping forced on an input whose partitions hold more distinct bricks
    than their tables (10M random bricks over 2048 tables of 4096 slots): the
    full tables are detected, the call reruns on the sort path and the DAG is
    exact."""
    rng = np.random.default_rng(21)
    depth = 12
    codes = rng.integers(0, 1 << (3 * depth), 10_000_000, dtype=np.uint64)
    ref = O.create_dag(codes, depth, threads=8)
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, 2)
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert c.dedup_fallbacks() >= 1


def test_grouping_spills_a_brick_larger_than_its_slab():
    """One brick holds most fragments (duplicates of a few codes): its
    partition's slab overflows into the shared overflow area, and the DAG is
    exact."""
    rng = np.random.default_rng(22)
    depth = 9
    bulk = rng.integers(0, 1 << (3 * depth), 300_000, dtype=np.uint64)
    heavy = np.repeat(np.array([12345 << 6 | k for k in range(0, 64, 3)], np.uint64), 40_000)
    codes = np.concatenate([bulk, heavy])
    rng.shuffle(codes)
    ref = O.create_dag(codes, depth)
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, 2)
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert c.dedup_fallbacks() == 0


def test_grouping_rejects_out_of_range_codes():
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, 2)
        with pytest.raises(D.DagcError) as e:
            c.create_dag(np.array([1, 2, 1 << 30], np.uint64), 9)  # 2^30 >= 8^9
        assert e.value.status == D.ERR_BAD_INPUT


def test_dedup_rerun_when_unique_list_is_full():
    """A level with more distinct hashes than the hash-set form holds is rerun
    in the radix form: same result, one rerun counted."""
    codes, depth = CASES["sparse_d21"]()  # ~20k distinct nodes on most levels
    ref = O.create_dag(codes, depth)
    with D.Context(0) as c:
        c.set_option(D.OPT_DEDUP_UNIQUE_LIMIT, 100)
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert c.dedup_fallbacks() == 1
        # The aborted levels left the table empty: the next call, with room
        # again, runs the hash-set form and agrees.
        c.set_option(D.OPT_DEDUP_UNIQUE_LIMIT, 1 << 30)
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert c.dedup_fallbacks() == 1


def test_dedup_form_is_the_one_that_runs():
    """Three launches per deduplicated node level instead of a radix sort's
    ten or more: the launch counter tells the two forms apart."""
    codes, depth = CASES["clustered_d10"]()
    launches = {}
    for form in (0, 1):
        with D.Context(0) as c:
            c.set_option(D.OPT_GRAPHS, 0)
            c.set_option(D.OPT_DEDUP, form)
            before = c.kernel_launches()
            c.create_dag(codes, depth)
            launches[form] = c.kernel_launches() - before
    assert launches[1] < launches[0]


def test_dedup_over_a_million_distinct_leaves():
    """Over a million distinct leaf masks: the grid-wide sort of the unique
    list orders them without a rerun in the radix form."""
    rng = np.random.default_rng(12)
    depth = 11
    bricks = rng.choice(8 ** (depth - 2), size=1_500_000, replace=False).astype(np.uint64)
    low = rng.integers(0, 64, size=(bricks.size, 5)).astype(np.uint64)
    codes = np.concatenate([(bricks << np.uint64(6)) | low[:, k] for k in range(5)])
    ref = O.create_dag(codes, depth, threads=8)
    assert ref.leaves.size > 1_050_000
    with D.Context(0) as c:
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert c.dedup_fallbacks() == 0


def test_dedup_many_buckets_and_skewed_leaves():
    """Leaf masks confined to their low 16 bits (a skewed key distribution) and
    levels with hundreds of thousands of distinct hashes (hundreds of buckets)."""
    rng = np.random.default_rng(9)
    depth = 9
    bricks = rng.choice(8 ** (depth - 2), size=400_000, replace=False).astype(np.uint64)
    low = rng.integers(0, 16, size=(bricks.size, 3)).astype(np.uint64)
    codes = np.concatenate([(bricks << np.uint64(6)) | low[:, k] for k in range(3)])
    ref = O.create_dag(codes, depth)
    with D.Context(0) as c:
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert c.dedup_fallbacks() == 0


@pytest.mark.parametrize("distinct", [1, 12_287, 12_288, 12_289, 40_000])
def test_distinct_leaf_masks_around_the_one_cta_sort(distinct):
    """Exactly `distinct` distinct leaf masks (each brick's mask a different
    value, some bricks sharing one): up to 12,288 of them are sorted by one
    CTA in shared memory, more by the grid-wide sort; both equal the oracle."""
    rng = np.random.default_rng(distinct)
    depth = 9
    bricks = rng.choice(8 ** (depth - 2), size=distinct + 3000, replace=False).astype(np.uint64)
    masks = rng.choice(2**40, size=distinct, replace=False).astype(np.uint64) + np.uint64(1)
    brick_mask = np.concatenate([masks, masks[rng.integers(0, distinct, size=3000)]])
    codes = []
    for k in range(40):
        sel = (brick_mask >> np.uint64(k)) & np.uint64(1) == 1
        codes.append((bricks[sel] << np.uint64(6)) | np.uint64(k))
    codes = np.concatenate(codes)
    rng.shuffle(codes)
    ref = O.create_dag(codes, depth, threads=8)
    assert ref.leaves.size == distinct
    with D.Context(0) as c:
        assert_dag_equal(c.create_dag(codes, depth).to_host(), ref)
        assert np.array_equal(c.compress(codes, depth).to_numpy(), O.final_dag(ref))
        assert c.dedup_fallbacks() == 0


def test_counts_reported(ctx):
    codes, depth = CASES["sphere_d7"]()
    ctx.create_dag(codes, depth).free()
    c = ctx.last_counts()
    ref = O.create_dag(codes, depth)
    assert c[0] == codes.size
    assert c[2] == ref.leaves.size


def test_empty_input(ctx):
    dag = ctx.create_dag(np.zeros(0, np.uint64), 7)
    assert dag.level_sizes() == [0] * 5 and dag.num_leaves == 0
    assert ctx.create_final_dag(dag).n == 0


def test_out_of_range_code_is_bad_input(ctx):
    codes = random_codes(7, 10_000, 3)
    codes[1234] = np.uint64(1 << 21)
    with pytest.raises(D.DagcError) as e:
        ctx.create_dag(codes, 7)
    assert e.value.status == D.ERR_BAD_INPUT
    # The context stays usable after a rejected input.
    ok = random_codes(7, 1000, 4)
    assert_dag_equal(ctx.create_dag(ok, 7).to_host(), O.create_dag(ok, 7))


def test_bad_depth_rejected(ctx):
    with pytest.raises(D.DagcError) as e:
        ctx.create_dag(np.array([1], np.uint64), 22)
    assert e.value.status == D.ERR_INVALID_ARGUMENT


def test_arena_reuse_large_then_small(ctx):
    big = clustered_codes(11, 1_500_000, 8)
    small = random_codes(6, 500, 9)
    for codes, depth in ((big, 11), (small, 6), (big, 11)):
        assert_dag_equal(ctx.create_dag(codes, depth).to_host(), O.create_dag(codes, depth, threads=8))


def test_compress_host_and_fused(ctx):
    codes, depth = CASES["terrain_d8"]()
    ref_words = O.final_dag(O.create_dag(codes, depth))
    assert np.array_equal(ctx.compress_host(codes, depth), ref_words)
    assert np.array_equal(ctx.compress(codes, depth).to_numpy(), ref_words)


@pytest.mark.parametrize("dedup", [1, 0])
@pytest.mark.parametrize("case", sorted(CASES))
def test_compress_from_call_pools_bit_exact(case, dedup):
    """dagc_compress lays the words out straight from the call's level pools
    (no DAG copied out of the call's scratch): every input case, both dedup
    forms, direct launches and the recorded graph, equal the oracle's words
    and CreateDAG + CreateFinalDAG."""
    codes, depth = CASES[case]()
    ref = O.final_dag(O.create_dag(codes, depth, threads=8))
    with D.Context(0) as c:
        c.set_option(D.OPT_DEDUP, dedup)
        for _ in range(3):  # first call, recording call, replay
            assert np.array_equal(c.compress(codes, depth).to_numpy(), ref)
        assert np.array_equal(c.create_final_dag(c.create_dag(codes, depth)).to_numpy(), ref)


def test_graph_replay_matches_direct_launches(ctx):
    """Repeated calls on one device buffer replay a recorded CUDA graph; the
    result must equal the directly launched pipeline and the oracle."""
    import torch
    codes = random_codes(10, 400_000, 21, cluster=True)
    t = torch.from_numpy(codes.view(np.int64)).cuda()
    ref = O.create_dag(codes, 10)
    for _ in range(4):  # first call launches directly, the second records, the rest replay
        assert_dag_equal(ctx.create_dag(t, 10).to_host(), ref)
    ctx.set_option(D.OPT_GRAPHS, 0)
    try:
        assert_dag_equal(ctx.create_dag(t, 10).to_host(), ref)
    finally:
        ctx.set_option(D.OPT_GRAPHS, 1)
    for _ in range(2):  # recorded again
        assert_dag_equal(ctx.create_dag(t, 10).to_host(), ref)
    # A different input in the same buffer: the replay must see the new data.
    codes2 = random_codes(10, 400_000, 22, cluster=True)
    t.copy_(torch.from_numpy(codes2.view(np.int64)))
    assert_dag_equal(ctx.create_dag(t, 10).to_host(), O.create_dag(codes2, 10))


def test_input_left_unchanged(ctx):
    import torch
    codes = random_codes(8, 100_000, 12)
    t = torch.from_numpy(codes.view(np.int64)).cuda()
    ctx.create_dag(t, 8).free()
    assert np.array_equal(t.cpu().numpy().view(np.uint64), codes)


# -------------------------------------------------------------- MergeDAGs ----
@pytest.mark.parametrize("depth,levels_up,seed", [(7, 1, 1), (9, 2, 2), (8, 1, 3)])
def test_merge_bit_exact(ctx, depth, levels_up, seed):
    codes = clustered_codes(depth, 100_000, seed)
    codes = codes[(codes >> np.uint64(3 * (depth - 1))) != np.uint64(5)]  # one empty octant
    chunks, sub = chunks_of(codes, depth, levels_up)
    ref_parts = [O.create_dag(c, sub) for c in chunks]
    ref = O.merge_dags(ref_parts)
    gpu = ctx.merge_dags([ctx.create_dag(c, sub) for c in chunks])
    assert_dag_equal(gpu.to_host(), ref)
    # ... and equals compressing the whole volume at once.
    assert O.dags_equal(ref, O.create_dag(codes, depth))
    assert np.array_equal(ctx.create_final_dag(gpu).to_numpy(), O.final_dag(ref))


def test_merge_all_empty(ctx):
    gpu = ctx.merge_dags([ctx.create_dag(np.zeros(0, np.uint64), 5) for _ in range(8)])
    assert gpu.level_sizes() == [0] * 4 and gpu.num_leaves == 0


def test_merge_collision_detected_on_device(ctx):
    # Two uploaded DAGs whose level-0 nodes share a hash but differ in content:
    # the merge's full compare must report a collision instead of picking one.
    def one(mask, child, h):
        return D.HostDag(masks=[np.array([mask], np.uint8)],
                         children=[np.array([[child if (mask >> c) & 1 else 0xFFFFFFFF for c in range(8)]],
                                            np.uint32)],
                         hashes=[np.array([h], np.uint64)],
                         leaves=np.array([1], np.uint64))
    empty = D.HostDag(masks=[np.zeros(0, np.uint8)], children=[np.zeros((0, 8), np.uint32)],
                      hashes=[np.zeros(0, np.uint64)], leaves=np.zeros(0, np.uint64))
    parts = [ctx.upload_dag(one(1, 0, 42)), ctx.upload_dag(one(2, 0, 42))]
    parts += [ctx.upload_dag(empty) for _ in range(6)]
    with pytest.raises(D.DagcError) as e:
        ctx.merge_dags(parts)
    assert e.value.status == D.ERR_HASH_COLLISION


def test_upload_rejects_malformed(ctx):
    bad = D.HostDag(masks=[np.array([1], np.uint8)],
                    children=[np.array([[5] + [0xFFFFFFFF] * 7], np.uint32)],  # child 5 of 1 leaf
                    hashes=[np.array([7], np.uint64)], leaves=np.array([1], np.uint64))
    with pytest.raises(D.DagcError) as e:
        ctx.upload_dag(bad)
    assert e.value.status == D.ERR_BAD_INPUT


# -------------------------------------------------------- full-size cases ----
def test_terrain_2048_full_size_bit_exact(ctx):
    """Procedural terrain, 2048^3 (depth 11), ~31M fragments: exact against the
    multi-threaded oracle, and decoded back to the input voxel set."""
    codes = D.gen_terrain(11, 0xDA6C0DE + 1)
    assert codes.size > 30_000_000
    ref = O.create_dag(codes, 11, threads=16)
    dag = ctx.create_dag(codes, 11)
    assert_dag_equal(dag.to_host(), ref)
    w = ctx.create_final_dag(dag).to_numpy()
    assert np.array_equal(w, O.final_dag(ref))
    assert np.array_equal(decode_final(w, 11), np.unique(codes))


@pytest.fixture(scope="module")
def soup_8192():
    """The triangle-soup workload at full size: 2M triangles in an 8192^3 grid
    (depth 13), ~65M shuffled fragments, and the multi-threaded oracle's DAG."""
    codes = D.gen_triangle_soup(13, 0xDA6C0DE + 3, 2_000_000)
    assert codes.size > 60_000_000
    ref = O.create_dag(codes, 13, threads=16)
    return codes, ref, O.final_dag(ref)


@pytest.mark.parametrize("group", [1, 2, 0])
def test_soup_8192_full_size_bit_exact(soup_8192, group):
    """Triangle soup, 8192^3, ~65M fragments (low redundancy: the device's
    own choice is the sort path), bit-exact against the oracle on the
    device-chosen path (1), with fragment grouping forced (2) and with the
    sort path forced (0); decoded back to the input voxel set."""
    codes, ref, ref_words = soup_8192
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, group)
        dag = c.create_dag(codes, 13)
        assert_dag_equal(dag.to_host(), ref)
        w = c.create_final_dag(dag).to_numpy()
        # The one-call form (words straight from the call's level pools).
        wc = c.compress(codes, 13).to_numpy()
    assert np.array_equal(w, ref_words)
    assert np.array_equal(wc, ref_words)
    if group == 1:
        assert np.array_equal(decode_final(w, 13), np.unique(codes))
