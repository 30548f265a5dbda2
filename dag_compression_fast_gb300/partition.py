"""Chunk-partitioned compression across ranks (one process per GPU).

The volume's chunks are independent: each rank compresses its own chunks and
the ranks then exchange one set of records per level. Records are
content-addressed, so they mean the same on every rank: a node is
(hash, child mask, the 8 child hashes) instead of indices into one rank's
arrays, a leaf is its 64-bit mask. The union of all ranks' records per level,
sorted by hash, with children turned back into indices, is exactly the DAG
that one device would build from all chunks (the reference's MergeDAGs,
src/DAGCompression.cu:1446-1548, computes the same union pairwise).

The exchange is one all-gather per call (torch.distributed: NCCL across GPUs,
gloo on CPUs in the tests). The compressor of each rank's chunks is pluggable:
the dagc batched path on a GPU, or any callable returning a host DAG.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

EMPTY = np.uint32(0xFFFFFFFF)


def assign_chunks(chunk_morton: Sequence[int], world: int):
    """Contiguous runs of the Morton-ordered chunks, one per rank (locality)."""
    order = np.argsort(np.asarray(chunk_morton, dtype=np.uint64), kind="stable")
    return [order[r * len(order) // world:(r + 1) * len(order) // world] for r in range(world)]


def chunk_roots(dag, top_levels: int) -> dict:
    """{chunk slot (Morton index): root hash} of the chunks a DAG holds, found
    by walking its top_levels levels from the root (child slot = Morton digit)."""
    if dag.num_levels == 0 or dag.hashes[0].size == 0:
        return {}
    frontier = [(0, 0)]
    for l in range(top_levels):
        nxt = []
        for idx, prefix in frontier:
            ch = dag.children[l][idx]
            for c in range(8):
                if ch[c] != EMPTY:
                    nxt.append((int(ch[c]), prefix * 8 + c))
        frontier = nxt
    below = dag.hashes[top_levels] if top_levels < dag.num_levels else dag.leaves
    return {slot: int(below[idx]) for idx, slot in frontier}


def to_records(dag, first_level: int = 0) -> dict:
    """Content-addressed records of a host DAG's levels first_level.. (root
    first) and its leaves."""
    rec = {"leaves": np.asarray(dag.leaves, np.uint64), "levels": []}
    below = rec["leaves"]  # hashes of the level below: leaf masks for the last level
    for l in reversed(range(first_level, dag.num_levels)):
        ch = np.asarray(dag.children[l], np.uint32).reshape(-1, 8)
        child_hash = np.zeros(ch.shape, np.uint64)
        has = ch != EMPTY
        child_hash[has] = below[ch[has]]
        rec["levels"].insert(0, (np.asarray(dag.hashes[l], np.uint64), np.asarray(dag.masks[l], np.uint8),
                                 child_hash))
        below = np.asarray(dag.hashes[l], np.uint64)
    return rec


def union_records(records: list, num_levels: int):
    """Per-level union by hash of several ranks' records -> host DAG arrays.

    Equal hashes must carry equal content (the full-compare collision check);
    a mismatch raises ValueError."""
    from dag_compression_fast_gb300 import HostDag
    leaves = np.unique(np.concatenate([r["leaves"] for r in records])) if records else np.zeros(0, np.uint64)
    out = HostDag(leaves=leaves)
    below = leaves
    levels = []
    for l in reversed(range(num_levels)):
        hs = np.concatenate([r["levels"][l][0] for r in records])
        ms = np.concatenate([r["levels"][l][1] for r in records])
        cs = np.concatenate([r["levels"][l][2] for r in records]).reshape(-1, 8)
        order = np.argsort(hs, kind="stable")
        hs, ms, cs = hs[order], ms[order], cs[order]
        first = np.ones(hs.size, bool)
        first[1:] = hs[1:] != hs[:-1]
        # Collision check: every member of a run equals the run's first member.
        run = np.cumsum(first) - 1
        rep = np.flatnonzero(first)[run]
        if not (np.array_equal(ms, ms[rep]) and np.array_equal(cs, cs[rep])):
            raise ValueError(f"hash collision in level {l}")
        uh, um, uc = hs[first], ms[first], cs[first]
        children = np.full(uc.shape, EMPTY, np.uint32)
        has = uc != 0
        idx = np.searchsorted(below, uc[has])
        if idx.size and (np.any(idx >= below.size) or np.any(below[np.minimum(idx, below.size - 1)] != uc[has])):
            raise ValueError(f"level {l} references a child missing from the union")
        children[has] = idx.astype(np.uint32)
        levels.insert(0, (uh, um, children))
        below = uh
    for uh, um, children in levels:
        out.hashes.append(uh)
        out.masks.append(um)
        out.children.append(children)
    return out


def build_top_levels(dag, root_hashes: Sequence[int], top_levels: int, hash_children: Callable):
    """Adds the levels above the chunks: groups of 8 consecutive chunk slots
    (Morton order) become one node each, like the reference's root build
    (src/DAGCompression.cu:1504-1533), deduplicated by hash; repeated until one
    root remains. root_hashes[i] is chunk slot i's root hash or 0 if empty."""
    hashes = list(root_hashes)
    below = dag.hashes[0] if dag.num_levels else dag.leaves
    new_levels = []
    for _ in range(top_levels):
        nodes = {}
        next_hashes = []
        for g in range(len(hashes) // 8):
            hs = [int(h) for h in hashes[8 * g:8 * g + 8]]
            mask = sum(1 << c for c in range(8) if hs[c])
            if not mask:
                next_hashes.append(0)
                continue
            ch = [int(np.searchsorted(below, np.uint64(h))) if h else int(EMPTY) for h in hs]
            h = int(hash_children(hs))
            if h in nodes and nodes[h] != (mask, tuple(ch)):
                raise ValueError("hash collision in a top level")
            nodes[h] = (mask, tuple(ch))
            next_hashes.append(h)
        keys = np.array(sorted(nodes), np.uint64)
        masks = np.array([nodes[int(k)][0] for k in keys], np.uint8)
        children = np.array([nodes[int(k)][1] for k in keys], np.uint32).reshape(-1, 8)
        new_levels.insert(0, (keys, masks, children))
        below = keys
        hashes = next_hashes
    for keys, masks, children in new_levels[::-1]:
        dag.hashes.insert(0, keys)
        dag.masks.insert(0, masks)
        dag.children.insert(0, children)
    return dag


def partitioned_create(chunks: Sequence[np.ndarray], chunk_morton: Sequence[int], chunk_depth: int,
                       top_levels: int, compress_local: Callable, hash_children: Callable = None, group=None):
    """Every rank compresses its share of the chunks with compress_local
    (chunks, morton, chunk_depth, top_levels) -> host DAG of depth
    chunk_depth + top_levels holding just those chunks (for instance the dagc
    batched path), then the ranks exchange the records of the chunk-internal
    levels and the chunk root hashes in one all-gather. The union of the
    records plus the levels above the chunks, rebuilt from all root hashes, is
    the DAG of every chunk; each rank returns it."""
    import torch.distributed as dist
    if hash_children is None:
        from dag_compression_fast_gb300 import hash_children
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = assign_chunks(chunk_morton, world)[rank]
    local = compress_local([chunks[i] for i in mine], [chunk_morton[i] for i in mine], chunk_depth, top_levels)
    payload = (to_records(local, top_levels), chunk_roots(local, top_levels))
    gathered = [None] * world
    if world > 1:
        dist.all_gather_object(gathered, payload, group=group)
    else:
        gathered = [payload]
    return merge_payloads(gathered, chunk_depth, top_levels, hash_children)


def merge_payloads(payloads: list, chunk_depth: int, top_levels: int, hash_children: Callable):
    """Union of every rank's (records, roots) into the DAG of all chunks."""
    dag = union_records([p[0] for p in payloads], chunk_depth - 2)
    roots = {}
    for _, r in payloads:
        roots.update(r)
    root_hashes = [roots.get(slot, 0) for slot in range(8 ** top_levels)]
    if not roots:
        from dag_compression_fast_gb300 import HostDag
        empty = HostDag()
        for _ in range(chunk_depth + top_levels - 2):
            empty.masks.append(np.zeros(0, np.uint8))
            empty.children.append(np.zeros((0, 8), np.uint32))
            empty.hashes.append(np.zeros(0, np.uint64))
        return empty
    return build_top_levels(dag, root_hashes, top_levels, hash_children)
