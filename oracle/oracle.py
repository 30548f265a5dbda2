"""ctypes wrapper of the CPU oracle (oracle/dag_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``. The product (the dagc library and
its Python mirror) never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdag_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref_hash.so")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_BAD_INPUT = 3
ERR_HASH_COLLISION = 4
ERR_TOO_LARGE = 7

_lib = None


def build() -> None:
    """Compile the oracle (and the reference hash shim where the reference exists)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        L.oracle_hash_children.argtypes = [vp]
        L.oracle_hash_children.restype = u64
        L.oracle_create.argtypes = [vp, u64, i32, i32, ctypes.POINTER(i32)]
        L.oracle_create.restype = vp
        L.oracle_empty.argtypes = [i32]
        L.oracle_empty.restype = vp
        L.oracle_from_arrays.argtypes = [i32, vp, vp, vp, vp, vp, u64]
        L.oracle_from_arrays.restype = vp
        L.oracle_merge.argtypes = [vp, u64, ctypes.POINTER(i32)]
        L.oracle_merge.restype = vp
        L.oracle_free.argtypes = [vp]
        L.oracle_num_levels.argtypes = [vp]
        L.oracle_num_levels.restype = i32
        L.oracle_level_size.argtypes = [vp, i32]
        L.oracle_level_size.restype = u64
        L.oracle_num_leaves.argtypes = [vp]
        L.oracle_num_leaves.restype = u64
        L.oracle_level_copy.argtypes = [vp, i32, vp, vp, vp]
        L.oracle_leaves_copy.argtypes = [vp, vp]
        L.oracle_final.argtypes = [vp, vp, u64, ctypes.POINTER(u64)]
        L.oracle_final.restype = i32
        L.oracle_radix_sort_keys.argtypes = [vp, u64, i32, i32, i32]
        L.oracle_trace.argtypes = [vp, u64, i32, vp, vp, vp, i32]
        L.oracle_voxelize_gl.argtypes = [vp, u64, vp, i32, vp, u64]
        L.oracle_voxelize_gl.restype = u64
        L.oracle_trace.restype = u64
        _lib = L
    return _lib


def ref_lib():
    """The reference's own src/Utils.h compiled on the host, or None when absent."""
    if not os.path.exists(REF_PATH):
        return None
    L = ctypes.CDLL(REF_PATH)
    L.ref_murmur128x4_lo.argtypes = [ctypes.c_void_p]
    L.ref_murmur128x4_lo.restype = ctypes.c_uint64
    L.ref_murmur64.argtypes = [ctypes.c_uint64]
    L.ref_murmur64.restype = ctypes.c_uint64
    L.ref_child_offset.argtypes = [ctypes.c_uint, ctypes.c_uint]
    L.ref_child_offset.restype = ctypes.c_uint
    L.ref_total_size.argtypes = [ctypes.c_uint]
    L.ref_total_size.restype = ctypes.c_uint
    return L


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a.size else None


@dataclass
class Dag:
    """Host copy of an FCpuDag: per level (root first) masks/children/hashes + leaves."""

    masks: list = field(default_factory=list)
    children: list = field(default_factory=list)  # each (n, 8) uint32
    hashes: list = field(default_factory=list)
    leaves: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))

    @property
    def num_levels(self) -> int:
        return len(self.masks)

    def level_sizes(self):
        return [int(h.size) for h in self.hashes]


def _to_dag(handle) -> Dag:
    L = lib()
    d = Dag()
    for l in range(L.oracle_num_levels(handle)):
        n = L.oracle_level_size(handle, l)
        m = np.zeros(n, np.uint8)
        c = np.zeros((n, 8), np.uint32)
        h = np.zeros(n, np.uint64)
        L.oracle_level_copy(handle, l, _ptr(m), _ptr(c), _ptr(h))
        d.masks.append(m)
        d.children.append(c)
        d.hashes.append(h)
    nl = L.oracle_num_leaves(handle)
    d.leaves = np.zeros(nl, np.uint64)
    L.oracle_leaves_copy(handle, _ptr(d.leaves))
    return d


def _from_dag(d: Dag):
    L = lib()
    sizes = d.level_sizes()
    offs = np.zeros(len(sizes) + 1, np.uint64)
    offs[1:] = np.cumsum(sizes, dtype=np.uint64)
    masks = np.concatenate(d.masks).astype(np.uint8) if sizes else np.zeros(0, np.uint8)
    ch = (np.concatenate(d.children).astype(np.uint32).reshape(-1)
          if sizes else np.zeros(0, np.uint32))
    hs = np.concatenate(d.hashes).astype(np.uint64) if sizes else np.zeros(0, np.uint64)
    leaves = np.ascontiguousarray(d.leaves, np.uint64)
    return L.oracle_from_arrays(len(sizes), _ptr(offs), _ptr(masks), _ptr(ch), _ptr(hs),
                                _ptr(leaves), leaves.size)


class OracleError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"oracle {what} failed with status {status}")
        self.status = status


def hash_children(h8) -> int:
    a = np.ascontiguousarray(np.asarray(h8, dtype=np.uint64))
    assert a.size == 8
    return int(lib().oracle_hash_children(_ptr(a)))


def create_dag(codes: np.ndarray, depth: int, threads: int = 1) -> Dag:
    """DAGCompression::CreateDAG restated on the CPU."""
    codes = np.ascontiguousarray(codes, dtype=np.uint64)
    st = ctypes.c_int(0)
    h = lib().oracle_create(_ptr(codes), codes.size, depth, threads, ctypes.byref(st))
    if not h:
        raise OracleError(st.value, "create")
    try:
        return _to_dag(h)
    finally:
        lib().oracle_free(h)


def merge_dags(dags) -> Dag:
    """DAGCompression::MergeDAGs restated on the CPU (8^k inputs, Morton order)."""
    L = lib()
    handles = [_from_dag(d) for d in dags]
    try:
        arr = (ctypes.c_void_p * len(handles))(*handles)
        st = ctypes.c_int(0)
        h = L.oracle_merge(arr, len(handles), ctypes.byref(st))
        if not h:
            raise OracleError(st.value, "merge")
        try:
            return _to_dag(h)
        finally:
            L.oracle_free(h)
    finally:
        for x in handles:
            L.oracle_free(x)


def trace(words: np.ndarray, depth: int, params, threads: int = 4):
    """The reference's trace_paths (src/DAGTracer.cu:297-427) restated on the
    CPU: (colours uint32[h, w], hits uint64[h, w], pixels that read outside the
    word array). `params` is a dagc_trace_params (ctypes structure)."""
    w = np.ascontiguousarray(words, np.uint32)
    colors = np.zeros((params.height, params.width), np.uint32)
    hits = np.zeros((params.height, params.width), np.uint64)
    bad = lib().oracle_trace(w.ctypes.data, w.size, depth, ctypes.addressof(params), colors.ctypes.data,
                             hits.ctypes.data, threads)
    return colors, hits, int(bad)


def voxelize_gl(vertices: np.ndarray, aabb, depth: int) -> np.ndarray:
    """The reference's GL voxelization (Shaders/*.glsl, src/Voxelizer.cpp)
    restated on the CPU: Morton codes in triangle order."""
    v = np.ascontiguousarray(vertices, np.float64).reshape(-1, 9)
    box = np.ascontiguousarray(aabb, np.float64)
    n = lib().oracle_voxelize_gl(v.ctypes.data, v.shape[0], box.ctypes.data, depth, None, 0)
    out = np.zeros(n, np.uint64)
    if n:
        lib().oracle_voxelize_gl(v.ctypes.data, v.shape[0], box.ctypes.data, depth, out.ctypes.data, n)
    return out


def final_dag(d: Dag) -> np.ndarray:
    """DAGCompression::CreateFinalDAG restated on the CPU: the uint32 word array."""
    L = lib()
    h = _from_dag(d)
    try:
        n = ctypes.c_uint64(0)
        st = L.oracle_final(h, None, 0, ctypes.byref(n))
        if st:
            raise OracleError(st, "final")
        out = np.zeros(n.value, np.uint32)
        st = L.oracle_final(h, _ptr(out), out.size, ctypes.byref(n))
        if st:
            raise OracleError(st, "final")
        return out
    finally:
        L.oracle_free(h)


def radix_sort_keys(keys: np.ndarray, lo_bit: int, hi_bit: int, threads: int) -> np.ndarray:
    k = np.array(keys, dtype=np.uint64, copy=True)
    lib().oracle_radix_sort_keys(_ptr(k), k.size, lo_bit, hi_bit, threads)
    return k


def dags_equal(a: Dag, b: Dag) -> bool:
    if a.num_levels != b.num_levels:
        return False
    for l in range(a.num_levels):
        if not (np.array_equal(a.masks[l], b.masks[l]) and
                np.array_equal(a.children[l], b.children[l]) and
                np.array_equal(a.hashes[l], b.hashes[l])):
            return False
    return np.array_equal(a.leaves, b.leaves)
