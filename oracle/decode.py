"""Decoder of the final uint32 DAG layout back to voxel Morton codes.

TEST INFRASTRUCTURE ONLY. It walks the layout the way the reference's tracer
reads it (FDAG::get_node / get_child_index / get_leaf,
src/DAGTracer.cu:157-175): node = child-mask word followed by one absolute
child pointer per set bit in ascending slot order; leaf = two words, low 32
bits first; root at word 0. The voxel set it returns must equal the set of
distinct input fragments, independently of the canonical node order.
"""
from __future__ import annotations

import numpy as np

_POPC8 = np.array([bin(i).count("1") for i in range(256)], np.uint32)


def decode_final(words: np.ndarray, depth: int) -> np.ndarray:
    """Sorted unique uint64 codes of every voxel stored in the DAG."""
    words = np.asarray(words, np.uint32)
    if words.size == 0:
        return np.zeros(0, np.uint64)
    num_levels = depth - 2
    idx = np.zeros(1, np.int64)
    prefix = np.zeros(1, np.uint64)
    for _ in range(num_levels):
        masks = words[idx] & 0xFF
        new_idx, new_prefix = [], []
        for c in range(8):
            has = ((masks >> c) & 1).astype(bool)
            if not has.any():
                continue
            k = _POPC8[masks[has] & ((1 << c) - 1)] + 1
            new_idx.append(words[idx[has] + k].astype(np.int64))
            new_prefix.append((prefix[has] << np.uint64(3)) | np.uint64(c))
        idx = np.concatenate(new_idx)
        prefix = np.concatenate(new_prefix)
    leaf = words[idx].astype(np.uint64) | (words[idx + 1].astype(np.uint64) << np.uint64(32))
    out = []
    for b in range(64):
        has = ((leaf >> np.uint64(b)) & np.uint64(1)).astype(bool)
        if has.any():
            out.append((prefix[has] << np.uint64(6)) | np.uint64(b))
    codes = np.concatenate(out) if out else np.zeros(0, np.uint64)
    return np.unique(codes)
