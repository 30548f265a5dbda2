"""CPU tests of the oracle: pinned to the reference's own hash code, checked
for the reference's structural invariants, and cross-checked between its
serial and multi-threaded modes, its merge and its final layout."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle.decode import decode_final
from tests.inputs import chunks_of, random_codes

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden():
    with open(os.path.join(GOLDEN, "hash_kats.json")) as f:
        return json.load(f)


# ------------------------------------------------------------------ hash ----
def test_hash_matches_reference_known_answers():
    g = golden()
    assert len(g["node_hash_kats"]) >= 50
    for kat in g["node_hash_kats"]:
        h = [int(x, 16) for x in kat["children"]]
        assert O.hash_children(h) == int(kat["node_hash"], 16)


def test_hash_known_answers_of_reference_utils():
    # Values computed from the reference's src/Utils.h (MurmurHash128xN, Size 4).
    assert O.hash_children([0] * 8) == 0x8B0AE71F762F012B
    assert O.hash_children([1, 0, 0, 0, 0, 0, 0, 0]) == 0xB9F19737C11352F1
    assert O.hash_children([0] * 7 + [2**64 - 1]) == 0x28A5EBE05A3D201D
    assert O.hash_children(list(range(1, 9))) == 0x6092AF62B5FF4D2A
    assert O.hash_children([2**64 - 1] * 8) == 0x807E8B314ACA2600


def test_hash_against_live_reference_build():
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference checkout not present on this machine")
    rng = np.random.default_rng(7)
    for _ in range(200):
        a = rng.integers(0, 2**64 - 1, 8, dtype=np.uint64)
        a[rng.random(8) < 0.3] = 0
        raw = int(R.ref_murmur128x4_lo(a.ctypes.data))
        assert O.hash_children(a) == (raw if raw else 1)


def test_child_offset_table_matches_reference():
    g = golden()
    for mask in range(256):
        for c in range(8):
            expect = bin(mask & ((1 << c) - 1)).count("1") + 1
            assert g["child_offset"][mask][c] == expect


# ------------------------------------------------------------ CreateDAG ----
def test_single_voxel_hand_derived():
    # One voxel at code 0, depth 3: one leaf with bit 0; one root with child 0.
    d = O.create_dag(np.array([0, 0, 0], np.uint64), 3)
    assert d.level_sizes() == [1]
    assert list(d.leaves) == [1]
    assert d.masks[0][0] == 1
    assert list(d.children[0][0]) == [0] + [0xFFFFFFFF] * 7
    assert int(d.hashes[0][0]) == 0xB9F19737C11352F1  # hash of (leaf 1, 0, ..., 0)
    w = O.final_dag(d)
    assert list(w) == [1, 2, 1, 0]


def test_two_leaves_hand_derived():
    # Depth 3 (8^3 grid): voxel code 0 (brick 0) and code 64+5 (brick 1, bit 5).
    d = O.create_dag(np.array([69, 0, 69], np.uint64), 3)
    assert list(d.leaves) == [1, 1 << 5]
    assert d.masks[0][0] == 0b11
    assert list(d.children[0][0][:2]) == [0, 1]
    w = O.final_dag(d)
    # root: mask, ptr to leaf 0 at word 3, ptr to leaf 1 at word 5
    assert list(w) == [3, 3, 5, 1, 0, 32, 0]


def test_identical_bricks_share_a_leaf():
    # Two bricks with the same 4x4x4 pattern deduplicate to one leaf.
    codes = np.array([0, 1, 64 * 3 + 0, 64 * 3 + 1], np.uint64)
    d = O.create_dag(codes, 3)
    assert list(d.leaves) == [0b11]
    assert list(d.children[0][0][[0, 3]]) == [0, 0]


def test_empty_input():
    d = O.create_dag(np.zeros(0, np.uint64), 7)
    assert d.level_sizes() == [0] * 5 and d.leaves.size == 0
    assert O.final_dag(d).size == 0


def test_bad_input_rejected():
    with pytest.raises(O.OracleError) as e:
        O.create_dag(np.array([1 << 21], np.uint64), 7)
    assert e.value.status == O.ERR_BAD_INPUT


def check_invariants(d, depth):
    """The reference's own checks: level 0 has one node, child index empty
    iff mask bit clear (src/DAGCompression.cu:860, :959-965), ascending
    unique hashes, indices in range."""
    assert d.num_levels == depth - 2
    if depth > 2:
        assert d.level_sizes()[0] == 1
    for l in range(d.num_levels):
        h = d.hashes[l]
        assert np.all(h[1:] > h[:-1])
        nxt = d.level_sizes()[l + 1] if l + 1 < d.num_levels else d.leaves.size
        for c in range(8):
            has = ((d.masks[l] >> c) & 1).astype(bool)
            ch = d.children[l][:, c]
            assert np.all((ch != 0xFFFFFFFF) == has)
            assert np.all(ch[has] < nxt)
    assert np.all(d.leaves[1:] > d.leaves[:-1])


@pytest.mark.parametrize("depth,n,seed,cluster", [(3, 50, 1, False), (5, 3000, 2, False),
                                                  (7, 20000, 3, True), (9, 50000, 4, True)])
def test_create_invariants_and_roundtrip(depth, n, seed, cluster):
    codes = random_codes(depth, n, seed, cluster)
    d = O.create_dag(codes, depth)
    check_invariants(d, depth)
    w = O.final_dag(d)
    assert np.array_equal(decode_final(w, depth), np.unique(codes))


def test_serial_and_threaded_agree():
    codes = random_codes(10, 300_000, 11, cluster=True)
    a = O.create_dag(codes, 10, threads=1)
    b = O.create_dag(codes, 10, threads=4)
    assert O.dags_equal(a, b)


def test_radix_sort_matches_numpy():
    rng = np.random.default_rng(5)
    k = rng.integers(0, 2**64 - 1, 200_000, dtype=np.uint64)
    assert np.array_equal(O.radix_sort_keys(k, 0, 64, 4), np.sort(k))


# -------------------------------------------------------------- MergeDAGs ----
@pytest.mark.parametrize("depth,levels_up,seed", [(6, 1, 1), (7, 2, 2), (8, 1, 3)])
def test_merge_equals_whole_volume(depth, levels_up, seed):
    codes = random_codes(depth, 30_000, seed, cluster=True)
    whole = O.create_dag(codes, depth)
    chunks, sub = chunks_of(codes, depth, levels_up)
    parts = [O.create_dag(c, sub) for c in chunks]
    merged = O.merge_dags(parts)
    assert O.dags_equal(merged, whole)
    assert np.array_equal(O.final_dag(merged), O.final_dag(whole))


def test_merge_with_empty_chunks():
    codes = random_codes(6, 2_000, 9, cluster=True)
    codes = codes[(codes >> np.uint64(15)) % np.uint64(3) == 0]  # leave some chunks empty
    whole = O.create_dag(codes, 6)
    chunks, sub = chunks_of(codes, 6, 1)
    assert any(c.size == 0 for c in chunks)
    merged = O.merge_dags([O.create_dag(c, sub) for c in chunks])
    assert O.dags_equal(merged, whole)


def test_merge_requires_power_of_eight():
    parts = [O.create_dag(np.array([1], np.uint64), 4) for _ in range(4)]
    with pytest.raises(O.OracleError):
        O.merge_dags(parts)


def test_decoder_on_full_depth_sparse_codes():
    rng = np.random.default_rng(3)
    codes = rng.integers(0, 2**63, 500, dtype=np.uint64)  # depth 21: 63 bits
    d = O.create_dag(codes, 21)
    check_invariants(d, 21)
    assert np.array_equal(decode_final(O.final_dag(d), 21), np.unique(codes))
