"""dag_compression_fast_gb300: GB300-native sparse voxel DAG compression.

Python mirror of the reference's DAGCompression namespace
(src/DAGCompression.h:42-49 of Phyronnaz/DAG_Compression_Fast) over the dagc
C ABI (include/dagc.h):

    CreateDAG(Fragments, Depth)  -> Context.create_dag(fragments, depth)
    MergeDAGs(CpuDags)           -> Context.merge_dags(dags)
    CreateFinalDAG(CpuDag)       -> Context.create_final_dag(dag)
    FreeAll()                    -> Context.free_all()

Where the reference aborts (CUDA error, failed check) this module raises
DagcError carrying the library status. All compression runs in the native
library; if it has not been built this module refuses to import.
"""
from __future__ import annotations

import ctypes
import os
import weakref
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "_lib")
LIBDAGC_PATH = os.path.join(LIB_DIR, "libdagc.so")
LIBGEN_PATH = os.path.join(LIB_DIR, "libdagc_gen.so")

OPT_SORT_SHAPE_KEYS = 1
OPT_SORT_SHAPE_PAIRS = 2
OPT_GRAPHS = 3
OPT_DEDUP = 4
OPT_DEDUP_UNIQUE_LIMIT = 5
OPT_GROUP = 6
OPT_PDL = 7
OPT_SORT_RADIX_BITS = 8
OPT_TEST_SPIN_LIMIT = 9
OPT_TEST_STALL_LOOKBACK = 10
OPT_TEST_FAIL_ALLOCS = 11
OPT_BATCH_PATH = 12
VOXELIZE_GL = 0
VOXELIZE_SAT = 1
NUM_KEY_SHAPES = 9
NUM_PAIR_SHAPES = 10
NUM_SORT_SHAPES = NUM_PAIR_SHAPES
RADIX_BITS = (8, 9, 10, 11)

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_OUT_OF_MEMORY = 2
ERR_BAD_INPUT = 3
ERR_HASH_COLLISION = 4
ERR_DEVICE_TIMEOUT = 5
ERR_CUDA = 6
ERR_TOO_LARGE = 7

# Every symbol of include/dagc.h, in declaration order.
DAGC_SYMBOLS = [
    "dagc_context_create", "dagc_context_destroy", "dagc_last_error", "dagc_status_string",
    "dagc_version", "dagc_hash_children", "dagc_create", "dagc_create_batched", "dagc_dag_num_levels", "dagc_dag_level_size",
    "dagc_dag_num_leaves", "dagc_dag_level_device", "dagc_dag_leaves_device",
    "dagc_dag_download_level", "dagc_dag_download_leaves", "dagc_dag_upload", "dagc_dag_copy",
    "dagc_dag_free", "dagc_create_footprint",
    "dagc_merge", "dagc_final", "dagc_free_words", "dagc_words_download", "dagc_free_all",
    "dagc_compress_host",
    "dagc_compress", "dagc_file_write", "dagc_file_read", "dagc_memory_stats", "dagc_memory_events", "dagc_memory_report",
    "dagc_last_counts", "dagc_set_option", "dagc_dedup_fallbacks", "dagc_trace", "dagc_trace_camera", "dagc_voxelize", "dagc_profile_enable", "dagc_profile_reset",
    "dagc_profile_read", "dagc_kernel_launches", "dagc_sort_keys", "dagc_sort_pairs",
    "dagc_tune_sort", "dagc_tune_save", "dagc_tune_load", "dagc_tune_clear", "dagc_sort_plan",
    "dagc_sort_keys_noalloc", "dagc_server_create", "dagc_server_submit", "dagc_server_submit_into", "dagc_server_wait",
    "dagc_server_stats", "dagc_server_shared_dag", "dagc_server_folds", "dagc_server_timeline", "dagc_server_set_option",
    "dagc_server_destroy", "dagc_union", "dagc_dag_lift",
]

STAGES = ["fragment_hist", "fragment_pass", "leaf_build", "leaf_dedup", "levels", "materialise",
          "final", "merge", "group", "group_sketch", "group_aggregate", "group_scatter", "chunk_leaves"]
GEN_SYMBOLS = ["dagc_gen_free", "dagc_gen_sphere_shell", "dagc_gen_terrain",
               "dagc_gen_triangle_soup", "dagc_gen_soup_triangles", "dagc_gen_batched"]


class DagcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"dagc status {status}: {message}")
        self.status = status
        self.message = message


def _load(path: str) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build the native library first "
            "(python -m dag_compression_fast_gb300.build)")
    return ctypes.CDLL(path)


_lib = None
_gen = None


def lib() -> ctypes.CDLL:
    """The dagc CUDA library (loaded on first use)."""
    global _lib
    if _lib is None:
        L = _load(LIBDAGC_PATH)
        vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        pvp = ctypes.POINTER(ctypes.c_void_p)
        pu64 = ctypes.POINTER(u64)
        L.dagc_context_create.argtypes = [i32, pvp]
        L.dagc_context_destroy.argtypes = [vp]
        L.dagc_context_destroy.restype = None
        L.dagc_last_error.argtypes = [vp]
        L.dagc_last_error.restype = ctypes.c_char_p
        L.dagc_status_string.argtypes = [i32]
        L.dagc_status_string.restype = ctypes.c_char_p
        L.dagc_hash_children.argtypes = [vp]
        L.dagc_hash_children.restype = u64
        L.dagc_create.argtypes = [vp, vp, u64, i32, vp, pvp]
        L.dagc_create_batched.argtypes = [vp, vp, vp, vp, u64, i32, i32, vp, pvp]
        L.dagc_dag_num_levels.argtypes = [vp, ctypes.POINTER(i32)]
        L.dagc_dag_level_size.argtypes = [vp, i32, pu64]
        L.dagc_dag_num_leaves.argtypes = [vp, pu64]
        L.dagc_dag_level_device.argtypes = [vp, i32, pvp, pvp, pvp]
        L.dagc_dag_leaves_device.argtypes = [vp, pvp]
        L.dagc_dag_download_level.argtypes = [vp, i32, vp, vp, vp]
        L.dagc_dag_download_leaves.argtypes = [vp, vp]
        L.dagc_dag_upload.argtypes = [vp, i32, vp, vp, vp, vp, vp, u64, vp, pvp]
        L.dagc_dag_copy.argtypes = [vp, vp, vp, pvp]
        L.dagc_create_footprint.argtypes = [u64, i32]
        L.dagc_create_footprint.restype = u64
        L.dagc_server_create.argtypes = [i32, i32, u64, pvp]
        L.dagc_server_submit.argtypes = [vp, vp, u64, i32, ctypes.c_int64, pu64]
        L.dagc_server_submit_into.argtypes = [vp, vp, u64, i32, ctypes.c_int64, vp, u64, pu64]
        L.dagc_server_wait.argtypes = [vp, u64, vp, u64, pu64, ctypes.POINTER(ctypes.c_double)]
        L.dagc_server_stats.argtypes = [vp, pu64, pu64, pu64, pu64]
        L.dagc_server_shared_dag.argtypes = [vp, i32, pvp, pvp]
        L.dagc_server_folds.argtypes = [vp, pu64]
        L.dagc_server_set_option.argtypes = [vp, i32, i32]
        L.dagc_server_timeline.argtypes = [vp, u64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.dagc_union.argtypes = [vp, vp, u64, vp, pvp, vp]
        L.dagc_dag_lift.argtypes = [vp, vp, vp, u64, vp, pvp]
        L.dagc_server_destroy.argtypes = [vp]
        L.dagc_server_destroy.restype = None
        L.dagc_dag_free.argtypes = [vp]
        L.dagc_dag_free.restype = None
        L.dagc_merge.argtypes = [vp, vp, u64, vp, pvp]
        L.dagc_final.argtypes = [vp, vp, vp, pvp, pu64]
        L.dagc_free_words.argtypes = [vp, vp, vp]
        L.dagc_words_download.argtypes = [vp, vp, u64, vp]
        L.dagc_free_all.argtypes = [vp]
        L.dagc_compress_host.argtypes = [vp, vp, u64, i32, vp, vp, u64, pu64]
        L.dagc_compress.argtypes = [vp, vp, u64, i32, vp, pvp, pu64]
        L.dagc_last_counts.argtypes = [vp, pu64, i32]
        L.dagc_dedup_fallbacks.argtypes = [vp, pu64]
        L.dagc_trace.argtypes = [vp, vp, u64, i32, vp, vp, vp, vp]
        L.dagc_voxelize.argtypes = [vp, vp, u64, vp, i32, i32, vp, u64, pu64, vp]
        L.dagc_trace_camera.argtypes = [vp, vp, vp, vp, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32, vp, vp,
                                        i32, ctypes.c_uint32, vp]
        L.dagc_file_write.argtypes = [ctypes.c_char_p, vp, ctypes.c_uint32, vp, u64]
        L.dagc_file_read.argtypes = [ctypes.c_char_p, vp, ctypes.POINTER(ctypes.c_uint32), vp, u64, pu64]
        L.dagc_memory_stats.argtypes = [vp, pu64, pu64, pu64, pu64]
        L.dagc_memory_events.argtypes = [vp, pu64, pu64]
        L.dagc_memory_report.argtypes = [vp, vp, u64, pu64]
        L.dagc_set_option.argtypes = [vp, i32, i32]
        L.dagc_profile_enable.argtypes = [vp, i32]
        L.dagc_profile_reset.argtypes = [vp]
        L.dagc_profile_read.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_double), pu64, pu64]
        L.dagc_kernel_launches.argtypes = [vp, pu64]
        L.dagc_sort_keys.argtypes = [vp, vp, vp, u64, i32, i32, vp]
        L.dagc_sort_pairs.argtypes = [vp, vp, vp, vp, vp, u64, i32, i32, vp]
        L.dagc_sort_keys_noalloc.argtypes = [vp, vp, u64, i32, i32, vp]
        pi32 = ctypes.POINTER(i32)
        pdbl = ctypes.POINTER(ctypes.c_double)
        L.dagc_tune_sort.argtypes = [vp, u64, i32, i32, i32, i32, pi32, pi32, pdbl, pdbl]
        L.dagc_tune_save.argtypes = [vp, ctypes.c_char_p]
        L.dagc_tune_load.argtypes = [vp, ctypes.c_char_p]
        L.dagc_tune_clear.argtypes = [vp]
        L.dagc_sort_plan.argtypes = [vp, u64, i32, i32, i32, pi32, pi32]
        _lib = L
    return _lib


def gen_lib() -> ctypes.CDLL:
    """The host-only synthetic fragment generators."""
    global _gen
    if _gen is None:
        G = _load(LIBGEN_PATH)
        vp, u64, i32, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_double
        G.dagc_gen_free.argtypes = [vp]
        G.dagc_gen_free.restype = None
        G.dagc_gen_sphere_shell.argtypes = [i32, u64, dbl, vp, vp]
        G.dagc_gen_terrain.argtypes = [i32, u64, dbl, vp, vp]
        G.dagc_gen_triangle_soup.argtypes = [i32, u64, u64, i32, vp, vp]
        G.dagc_gen_soup_triangles.argtypes = [i32, u64, u64, vp]
        G.dagc_gen_batched.argtypes = [i32, i32, i32, u64, dbl, dbl, i32, vp, vp, vp, vp, vp]
        _gen = G
    return _gen


def _np_ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a.size else None


def _stream_handle(stream):
    """cudaStream_t as an integer: None -> the current torch stream."""
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


@dataclass
class HostDag:
    """Host copy of an FCpuDag (src/DAGCompression.h:12-40): per level (root
    first) child masks, children (n, 8) and ascending hashes, plus leaves."""

    masks: list = field(default_factory=list)
    children: list = field(default_factory=list)
    hashes: list = field(default_factory=list)
    leaves: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint64))

    @property
    def num_levels(self) -> int:
        return len(self.masks)

    def level_sizes(self):
        return [int(h.size) for h in self.hashes]


class Dag:
    """A device-resident DAG (the FCpuDag equivalent kept in HBM)."""

    def __init__(self, ctx: "Context", handle: int):
        self.ctx = ctx
        self.handle = handle
        live = getattr(ctx, "_live", None)
        if live is not None:
            live.add(self)

    def _live(self):
        if not self.handle:
            raise DagcError(ERR_INVALID_ARGUMENT, "DAG was consumed or freed")
        return self.handle

    @property
    def num_levels(self) -> int:
        n = ctypes.c_int(0)
        self.ctx._check(lib().dagc_dag_num_levels(self._live(), ctypes.byref(n)))
        return n.value

    def level_sizes(self):
        out = []
        for l in range(self.num_levels):
            n = ctypes.c_uint64(0)
            self.ctx._check(lib().dagc_dag_level_size(self._live(), l, ctypes.byref(n)))
            out.append(n.value)
        return out

    @property
    def num_leaves(self) -> int:
        n = ctypes.c_uint64(0)
        self.ctx._check(lib().dagc_dag_num_leaves(self._live(), ctypes.byref(n)))
        return n.value

    def to_host(self) -> HostDag:
        """FGpuLevel::ToCPU for every level plus the leaves."""
        d = HostDag()
        for l, n in enumerate(self.level_sizes()):
            m = np.zeros(n, np.uint8)
            c = np.zeros((n, 8), np.uint32)
            h = np.zeros(n, np.uint64)
            self.ctx._check(lib().dagc_dag_download_level(self._live(), l, _np_ptr(m), _np_ptr(c), _np_ptr(h)))
            d.masks.append(m)
            d.children.append(c)
            d.hashes.append(h)
        d.leaves = np.zeros(self.num_leaves, np.uint64)
        self.ctx._check(lib().dagc_dag_download_leaves(self._live(), _np_ptr(d.leaves)))
        return d

    def free(self):
        if self.handle:
            lib().dagc_dag_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Words:
    """The final uint32 DAG (device memory owned by the caller)."""

    def __init__(self, ctx: "Context", ptr: int, n: int):
        self.ctx = ctx
        self.ptr = ptr
        self.n = n
        ctx._live.add(self)

    def to_numpy(self) -> np.ndarray:
        out = np.zeros(self.n, np.uint32)
        if self.n:
            self.ctx._check(lib().dagc_words_download(self.ctx.handle, self.ptr, self.n, _np_ptr(out)))
        return out

    def free(self):
        if self.ptr:
            lib().dagc_free_words(self.ctx.handle, self.ptr, None)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class TraceParams(ctypes.Structure):
    """dagc_trace_params: the reference's FDAGTracer::TracePathsParams
    (src/DAGTracer.h:15-25) in voxel units of the 2^depth grid."""
    _fields_ = [("debug_level", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("pad", ctypes.c_uint32), ("camera", ctypes.c_double * 3), ("ray_min", ctypes.c_double * 3),
                ("ray_ddx", ctypes.c_double * 3), ("ray_ddy", ctypes.c_double * 3)]


TRACE_POSITION_COLORS = 0xFFFFFFFF


def trace_camera(position, right, up, forward, fov_degrees: float, width: int, height: int, aabb_min, aabb_max,
                 depth: int, debug_level: int = TRACE_POSITION_COLORS) -> TraceParams:
    """FDAGTracer::GetTraceParams (src/DAGTracer.h:26-79): a camera in scene
    units mapped onto the 2^depth voxel grid of the box [aabb_min, aabb_max]."""
    vecs = [np.ascontiguousarray(v, np.float64) for v in (position, right, up, forward, aabb_min, aabb_max)]
    p = TraceParams()
    st = lib().dagc_trace_camera(*[v.ctypes.data for v in vecs[:4]], float(fov_degrees), width, height,
                                 vecs[4].ctypes.data, vecs[5].ctypes.data, depth, debug_level, ctypes.byref(p))
    if st:
        raise DagcError(st, "bad camera")
    return p


def _device_u64(fragments, device: int):
    """(pointer, count, keepalive) for a uint64 fragment array on the device."""
    import torch
    if isinstance(fragments, torch.Tensor):
        t = fragments
        if t.dtype not in (torch.int64, torch.uint64):
            raise DagcError(ERR_INVALID_ARGUMENT, "fragments must be 64-bit")
        if not t.is_cuda:
            t = t.to(f"cuda:{device}")
        t = t.contiguous()
        return t.data_ptr(), t.numel(), t
    a = np.ascontiguousarray(fragments, dtype=np.uint64)
    t = torch.from_numpy(a.view(np.int64)).to(f"cuda:{device}")
    return t.data_ptr(), t.numel(), t


class Context:
    """One dagc context (device scratch arena + DAG memory pool)."""

    def __init__(self, device: int = 0):
        self.device = device
        h = ctypes.c_void_p()
        st = lib().dagc_context_create(device, ctypes.byref(h))
        if st:
            raise DagcError(st, "dagc_context_create failed")
        self.handle = h.value
        self._live = weakref.WeakSet()  # DAGs and word arrays to release before the context

    def close(self):
        if getattr(self, "handle", None):
            for obj in list(self._live):
                obj.free()
            lib().dagc_context_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st: int):
        if st:
            msg = lib().dagc_last_error(self.handle).decode(errors="replace")
            raise DagcError(st, msg)

    # ------------------------------------------------------------ API ----
    def create_dag(self, fragments, depth: int, stream=None) -> Dag:
        """DAGCompression::CreateDAG: fragments (device tensor or host array of
        uint64 Morton codes) -> device-resident DAG with depth-2 levels."""
        ptr, n, keep = _device_u64(fragments, self.device)
        out = ctypes.c_void_p()
        st = lib().dagc_create(self.handle, ptr, n, depth, _stream_handle(stream), ctypes.byref(out))
        del keep
        self._check(st)
        return Dag(self, out.value)

    def create_dag_batched(self, fragments, chunk_counts, chunk_morton, chunk_depth: int, top_levels: int,
                           stream=None) -> Dag:
        """Batched CreateDAG + MergeDAGs: chunk-local fragments of k chunks back to
        back (chunk_counts[i] each), chunks in ascending Morton order
        chunk_morton[i] of a 2^top_levels-per-side chunk grid."""
        ptr, n, keep = _device_u64(fragments, self.device)
        counts = np.ascontiguousarray(chunk_counts, np.uint64)
        offsets = np.zeros(counts.size + 1, np.uint64)
        offsets[1:] = np.cumsum(counts, dtype=np.uint64)
        morton = np.ascontiguousarray(chunk_morton, np.uint64)
        if int(offsets[-1]) != n:
            raise DagcError(ERR_INVALID_ARGUMENT, "chunk counts do not add up to the fragment count")
        out = ctypes.c_void_p()
        st = lib().dagc_create_batched(self.handle, ptr, _np_ptr(offsets), _np_ptr(morton), counts.size,
                                       chunk_depth, top_levels, _stream_handle(stream), ctypes.byref(out))
        del keep
        self._check(st)
        return Dag(self, out.value)

    def merge_dags(self, dags, stream=None) -> Dag:
        """DAGCompression::MergeDAGs: 8^m sub-DAGs in Morton order -> one DAG
        with m more levels. Consumes the inputs."""
        arr = (ctypes.c_void_p * len(dags))(*[d._live() for d in dags])
        out = ctypes.c_void_p()
        st = lib().dagc_merge(self.handle, arr, len(dags), _stream_handle(stream), ctypes.byref(out))
        self._check(st)
        for i, d in enumerate(dags):
            d.handle = arr[i]  # consumed inputs come back as NULL
        return Dag(self, out.value)

    def create_final_dag(self, dag: Dag, stream=None) -> Words:
        """DAGCompression::CreateFinalDAG: consumes the DAG, returns the uint32 words."""
        ptr = ctypes.c_void_p()
        n = ctypes.c_uint64(0)
        st = lib().dagc_final(self.handle, dag._live(), _stream_handle(stream), ctypes.byref(ptr), ctypes.byref(n))
        self._check(st)
        dag.handle = None
        return Words(self, ptr.value or 0, n.value)

    def compress(self, fragments, depth: int, stream=None) -> Words:
        """CreateDAG + CreateFinalDAG in one call."""
        ptr, n, keep = _device_u64(fragments, self.device)
        wp = ctypes.c_void_p()
        nw = ctypes.c_uint64(0)
        st = lib().dagc_compress(self.handle, ptr, n, depth, _stream_handle(stream), ctypes.byref(wp), ctypes.byref(nw))
        del keep
        self._check(st)
        return Words(self, wp.value or 0, nw.value)

    def compress_host(self, fragments: np.ndarray, depth: int, stream=None) -> np.ndarray:
        """Host fragments -> host words through dagc_compress_host."""
        a = np.ascontiguousarray(fragments, dtype=np.uint64)
        nw = ctypes.c_uint64(0)
        sh = _stream_handle(stream)
        self._check(lib().dagc_compress_host(self.handle, _np_ptr(a), a.size, depth, sh, None, 0, ctypes.byref(nw)))
        out = np.zeros(nw.value, np.uint32)
        self._check(lib().dagc_compress_host(self.handle, _np_ptr(a), a.size, depth, sh, _np_ptr(out), out.size,
                                             ctypes.byref(nw)))
        return out

    def upload_dag(self, host: HostDag, stream=None) -> Dag:
        """FGpuLevel::FromCPU for every level: a host DAG -> device DAG."""
        nl = host.num_levels
        sizes = np.array(host.level_sizes(), np.uint64)
        ms = [np.ascontiguousarray(m, np.uint8) for m in host.masks]
        cs = [np.ascontiguousarray(c, np.uint32) for c in host.children]
        hs = [np.ascontiguousarray(h, np.uint64) for h in host.hashes]
        mp = (ctypes.c_void_p * max(nl, 1))(*[m.ctypes.data for m in ms])
        cp = (ctypes.c_void_p * max(nl, 1))(*[c.ctypes.data for c in cs])
        hp = (ctypes.c_void_p * max(nl, 1))(*[h.ctypes.data for h in hs])
        leaves = np.ascontiguousarray(host.leaves, np.uint64)
        out = ctypes.c_void_p()
        st = lib().dagc_dag_upload(self.handle, nl, _np_ptr(sizes), mp, cp, hp, _np_ptr(leaves), leaves.size,
                                   _stream_handle(stream), ctypes.byref(out))
        self._check(st)
        return Dag(self, out.value)

    def union_dags(self, dags, stream=None):
        """Per-level union of DAGs of equal depth (dagc_union): (DAG, root hashes)."""
        arr = (ctypes.c_void_p * len(dags))(*[d._live() for d in dags])
        roots = np.zeros(len(dags), np.uint64)
        out = ctypes.c_void_p()
        self._check(lib().dagc_union(self.handle, arr, len(dags), _stream_handle(stream), ctypes.byref(out),
                                     roots.ctypes.data))
        return Dag(self, out.value), roots

    def lift_dag(self, body: "Dag", slot_root_hashes, stream=None) -> Dag:
        """The DAG over 8^m chunk slots whose roots are in `body` (dagc_dag_lift)."""
        h = np.ascontiguousarray(slot_root_hashes, np.uint64)
        out = ctypes.c_void_p()
        self._check(lib().dagc_dag_lift(self.handle, body._live(), h.ctypes.data, h.size, _stream_handle(stream),
                                        ctypes.byref(out)))
        return Dag(self, out.value)

    def free_all(self):
        """DAGCompression::FreeAll."""
        self._check(lib().dagc_free_all(self.handle))

    def set_option(self, option: int, value: int):
        """dagc_set_option: OPT_SORT_SHAPE_KEYS / OPT_SORT_SHAPE_PAIRS."""
        self._check(lib().dagc_set_option(self.handle, option, value))

    def profile(self, enable: bool = True):
        """Turns per-stage CUDA-event timing on or off (see include/dagc.h)."""
        self._check(lib().dagc_profile_enable(self.handle, int(enable)))

    def profile_reset(self):
        self._check(lib().dagc_profile_reset(self.handle))

    def profile_read(self):
        """{stage: (device_ms, launches, algorithmic_bytes)} accumulated so far."""
        out = {}
        for i, name in enumerate(STAGES):
            ms, la, by = ctypes.c_double(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
            self._check(lib().dagc_profile_read(self.handle, i, ctypes.byref(ms), ctypes.byref(la), ctypes.byref(by)))
            out[name] = (ms.value, la.value, by.value)
        return out

    def kernel_launches(self) -> int:
        n = ctypes.c_uint64(0)
        self._check(lib().dagc_kernel_launches(self.handle, ctypes.byref(n)))
        return n.value

    def memory_stats(self):
        """Device memory of this context (dagc_memory_stats)."""
        v = [ctypes.c_uint64(0) for _ in range(4)]
        self._check(lib().dagc_memory_stats(self.handle, *[ctypes.byref(x) for x in v]))
        return dict(zip(["in_use", "peak", "cached", "arena"], [x.value for x in v]))

    def memory_report(self) -> str:
        """The context's device memory by allocation name (dagc_memory_report)."""
        need = ctypes.c_uint64(0)
        self._check(lib().dagc_memory_report(self.handle, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self._check(lib().dagc_memory_report(self.handle, buf, need.value, ctypes.byref(need)))
        return buf.value.decode()

    def memory_events(self):
        """Failed device allocations (injected or real) and allocations that
        succeeded on their retry (dagc_memory_events)."""
        f, r = ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._check(lib().dagc_memory_events(self.handle, ctypes.byref(f), ctypes.byref(r)))
        return {"alloc_failures": f.value, "retries_ok": r.value}

    def trace(self, words, depth: int, params: TraceParams, hits: bool = True, stream=None):
        """Headless FDAGTracer::ResolvePaths: traces the final DAG (a Words
        object, or a uint32 array / tensor of its words) and returns
        (colours uint32[h, w], hits uint64[h, w] or None) on the host."""
        import torch
        if isinstance(words, Words):
            ptr, n, keep = words.ptr, words.n, None
        else:
            t = words if isinstance(words, torch.Tensor) else torch.from_numpy(
                np.ascontiguousarray(words, np.uint32).view(np.int32))
            keep = t.to(f"cuda:{self.device}").contiguous()
            ptr, n = keep.data_ptr(), keep.numel()
        dev = f"cuda:{self.device}"
        colors = torch.empty((params.height, params.width), dtype=torch.int32, device=dev)
        hit_t = torch.empty((params.height, params.width), dtype=torch.int64, device=dev) if hits else None
        st = lib().dagc_trace(self.handle, ptr, n, depth, ctypes.byref(params), colors.data_ptr(),
                              hit_t.data_ptr() if hits else None, _stream_handle(stream))
        del keep
        self._check(st)
        c = colors.cpu().numpy().view(np.uint32)
        h = hit_t.cpu().numpy().view(np.uint64) if hits else None
        return c, h

    def voxelize(self, vertices, aabb, depth: int, mode: int = 0, capacity: int = None, stream=None):
        """FVoxelizer::GenerateFragments on the GPU: triangles (n x 9 or n x 3 x 3
        doubles, scene units; host array or device tensor) in the box aabb =
        (min xyz, max xyz) -> device tensor of Morton codes (int64 view of the
        uint64 codes), in a fixed order. mode: VOXELIZE_GL (the reference's
        rule) or VOXELIZE_SAT. Without a capacity, a counting call sizes the buffer."""
        import torch
        dev = f"cuda:{self.device}"
        if isinstance(vertices, torch.Tensor):
            v = vertices.to(device=dev, dtype=torch.float64).contiguous()
        else:
            v = torch.from_numpy(np.ascontiguousarray(vertices, np.float64)).to(dev)
        n_tri = v.numel() // 9
        box = np.ascontiguousarray(aabb, np.float64)
        n = ctypes.c_uint64(0)
        if capacity is None:
            st = lib().dagc_voxelize(self.handle, v.data_ptr(), n_tri, box.ctypes.data, depth, mode, None, 0,
                                     ctypes.byref(n), _stream_handle(stream))
            if st not in (OK, ERR_TOO_LARGE):
                self._check(st)
            capacity = n.value
        out = torch.empty(max(capacity, 1), dtype=torch.int64, device=dev)
        st = lib().dagc_voxelize(self.handle, v.data_ptr(), n_tri, box.ctypes.data, depth, mode, out.data_ptr(),
                                 capacity, ctypes.byref(n), _stream_handle(stream))
        self._check(st)
        return out[: n.value]

    def dedup_fallbacks(self) -> int:
        """Calls rerun in the radix form because the hash-set dedup could not hold them."""
        v = ctypes.c_uint64(0)
        self._check(lib().dagc_dedup_fallbacks(self.handle, ctypes.byref(v)))
        return v.value

    def last_counts(self):
        buf = (ctypes.c_uint64 * 64)()
        k = lib().dagc_last_counts(self.handle, buf, 64)
        return [int(buf[i]) for i in range(k)]

    def sort_keys(self, keys, lo_bit: int = 0, hi_bit: int = 64, stream=None):
        import torch
        ptr, n, t = _device_u64(keys, self.device)
        out = torch.empty_like(t)
        self._check(lib().dagc_sort_keys(self.handle, ptr, out.data_ptr(), n, lo_bit, hi_bit, _stream_handle(stream)))
        return out

    # ------------------------------------------------------- autotuner ----
    def tune_sort(self, n: int, lo_bit: int, hi_bit: int, with_values: bool = False, reps: int = 5):
        """Times every valid digit-pass plan of one sort class on the device
        and keeps the fastest in the context's tuning table (dagc_tune_sort).
        Returns {"shape", "radix_bits", "ms", "default_ms"}."""
        sh, rb = ctypes.c_int(0), ctypes.c_int(0)
        ms, dms = ctypes.c_double(0), ctypes.c_double(0)
        self._check(lib().dagc_tune_sort(self.handle, n, lo_bit, hi_bit, int(with_values), reps, ctypes.byref(sh),
                                         ctypes.byref(rb), ctypes.byref(ms), ctypes.byref(dms)))
        return {"shape": sh.value, "radix_bits": rb.value, "ms": ms.value, "default_ms": dms.value}

    def sort_plan(self, n: int, lo_bit: int, hi_bit: int, with_values: bool = False):
        """(shape, radix_bits) a sort of this class would take."""
        sh, rb = ctypes.c_int(0), ctypes.c_int(0)
        self._check(lib().dagc_sort_plan(self.handle, n, lo_bit, hi_bit, int(with_values), ctypes.byref(sh),
                                         ctypes.byref(rb)))
        return sh.value, rb.value

    def tune_save(self, path: str):
        self._check(lib().dagc_tune_save(self.handle, os.fsencode(path)))

    def tune_load(self, path: str):
        self._check(lib().dagc_tune_load(self.handle, os.fsencode(path)))

    def tune_clear(self):
        self._check(lib().dagc_tune_clear(self.handle))

    def sort_pairs(self, keys, values=None, lo_bit: int = 0, hi_bit: int = 64, stream=None):
        import torch
        ptr, n, t = _device_u64(keys, self.device)
        kout = torch.empty_like(t)
        vout = torch.empty(n, dtype=torch.int32, device=t.device)
        vin = None
        if values is not None:
            values = values.to(t.device).contiguous()
            vin = values.data_ptr()
        self._check(lib().dagc_sort_pairs(self.handle, ptr, kout.data_ptr(), vin, vout.data_ptr(), n, lo_bit, hi_bit,
                                          _stream_handle(stream)))
        return kout, vout


class _BorrowedContext:
    """A context owned by the library (the server's merge context)."""

    def __init__(self, handle, device):
        self.handle = handle
        self.device = device

    def _check(self, st: int):
        if st:
            raise DagcError(st, lib().dagc_last_error(self.handle).decode(errors="replace"))


class Server:
    """The serving loop (dagc_server_*): jobs admitted by device-memory
    footprint into `slots` concurrent worker slots."""

    def __init__(self, device: int = 0, slots: int = 4, hbm_budget_bytes: int = 64 << 30):
        h = ctypes.c_void_p()
        st = lib().dagc_server_create(device, slots, hbm_budget_bytes, ctypes.byref(h))
        if st:
            raise DagcError(st, "dagc_server_create failed")
        self.handle = h.value
        self.device = device
        self._inputs = {}
        self._outputs = {}
        self._shared = []  # DAGs on the server's merge context: freed before it

    def submit(self, fragments: np.ndarray, depth: int, chunk_morton: int = -1) -> int:
        a = np.ascontiguousarray(fragments, dtype=np.uint64)
        t = ctypes.c_uint64(0)
        st = lib().dagc_server_submit(self.handle, _np_ptr(a), a.size, depth, chunk_morton, ctypes.byref(t))
        if st:
            raise DagcError(st, "dagc_server_submit failed")
        self._inputs[t.value] = a  # keep alive until the job is collected
        return t.value

    def submit_into(self, fragments: np.ndarray, depth: int, out: np.ndarray, chunk_morton: int = -1) -> int:
        """submit() with the words written straight into `out` (uint32, ideally
        page-locked memory); wait() then returns a view of it."""
        a = np.ascontiguousarray(fragments, dtype=np.uint64)
        if out.dtype != np.uint32 or not out.flags.c_contiguous:
            raise DagcError(ERR_INVALID_ARGUMENT, "out must be a contiguous uint32 array")
        t = ctypes.c_uint64(0)
        st = lib().dagc_server_submit_into(self.handle, _np_ptr(a), a.size, depth, chunk_morton, _np_ptr(out),
                                           out.size, ctypes.byref(t))
        if st:
            raise DagcError(st, "dagc_server_submit_into failed")
        self._inputs[t.value] = a
        self._outputs[t.value] = out
        return t.value

    def wait(self, ticket: int):
        """(words, latency_ms) of a finished job."""
        n = ctypes.c_uint64(0)
        lat = ctypes.c_double(0)
        st = lib().dagc_server_wait(self.handle, ticket, None, 0, ctypes.byref(n), ctypes.byref(lat))
        if st:
            self._inputs.pop(ticket, None)
            self._outputs.pop(ticket, None)
            raise DagcError(st, "job failed")
        out = self._outputs.pop(ticket, None)
        if out is not None and n.value <= out.size:
            self._inputs.pop(ticket, None)
            return out[: n.value], lat.value
        out = np.zeros(n.value, np.uint32)
        st = lib().dagc_server_wait(self.handle, ticket, _np_ptr(out), out.size, ctypes.byref(n), ctypes.byref(lat))
        self._inputs.pop(ticket, None)
        if st:
            raise DagcError(st, "job failed")
        return out, lat.value

    def stats(self):
        c, f, m, p = (ctypes.c_uint64(0) for _ in range(4))
        lib().dagc_server_stats(self.handle, ctypes.byref(c), ctypes.byref(f), ctypes.byref(m), ctypes.byref(p))
        return {"completed": c.value, "fragments": f.value, "max_concurrent": m.value, "peak_footprint": p.value}

    def set_option(self, option: int, value: int):
        """dagc_set_option on every worker slot's context."""
        st = lib().dagc_server_set_option(self.handle, option, value)
        if st:
            raise DagcError(st, "dagc_server_set_option failed")

    def folds(self) -> int:
        """Unions of finished chunks into the resident shared DAG so far."""
        v = ctypes.c_uint64(0)
        lib().dagc_server_folds(self.handle, ctypes.byref(v))
        return v.value

    def timeline(self, ticket: int):
        """(gpu_start_ms, gpu_end_ms) of a finished job's device work."""
        a, b = ctypes.c_double(0), ctypes.c_double(0)
        st = lib().dagc_server_timeline(self.handle, ticket, ctypes.byref(a), ctypes.byref(b))
        if st:
            raise DagcError(st, "no timeline for this ticket")
        return a.value, b.value

    def shared_dag(self, top_levels: int) -> Dag:
        """Merges every chunk job so far into one device DAG."""
        ctx = ctypes.c_void_p()
        out = ctypes.c_void_p()
        st = lib().dagc_server_shared_dag(self.handle, top_levels, ctypes.byref(ctx), ctypes.byref(out))
        if st:
            raise DagcError(st, "dagc_server_shared_dag failed")
        d = Dag(_BorrowedContext(ctx.value, self.device), out.value)
        self._shared.append(d)
        return d

    def close(self):
        if getattr(self, "handle", None):
            for d in self._shared:
                d.free()
            self._shared = []
            lib().dagc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_dag_file(path: str, words: np.ndarray, depth: int, aabb=(0, 0, 0, 1, 1, 1)) -> None:
    """Writes a final DAG as a .dag.bin file (the reference's format)."""
    w = np.ascontiguousarray(words, np.uint32)
    box = np.ascontiguousarray(np.asarray(aabb, np.float64))
    st = lib().dagc_file_write(os.fsencode(path), box.ctypes.data, depth, _np_ptr(w), w.size)
    if st:
        raise DagcError(st, f"cannot write {path}")


def read_dag_file(path: str):
    """(words, depth, aabb) of a .dag.bin file."""
    box = np.zeros(6, np.float64)
    d = ctypes.c_uint32(0)
    n = ctypes.c_uint64(0)
    st = lib().dagc_file_read(os.fsencode(path), box.ctypes.data, ctypes.byref(d), None, 0, ctypes.byref(n))
    if st:
        raise DagcError(st, f"cannot read {path}")
    w = np.zeros(n.value, np.uint32)
    st = lib().dagc_file_read(os.fsencode(path), None, None, _np_ptr(w), w.size, ctypes.byref(n))
    if st:
        raise DagcError(st, f"cannot read {path}")
    return w, d.value, tuple(box)


def hash_children(h8) -> int:
    """The node hash of 8 child hashes (dagc_hash_children)."""
    a = np.ascontiguousarray(np.asarray(h8, dtype=np.uint64))
    if a.size != 8:
        raise DagcError(ERR_INVALID_ARGUMENT, "need 8 child hashes")
    return int(lib().dagc_hash_children(a.ctypes.data))


def create_footprint(n: int, depth: int) -> int:
    """Device scratch bytes of one CreateDAG call (dagc_create_footprint)."""
    return int(lib().dagc_create_footprint(n, depth))


# ---------------------------------------------------------------- inputs ----
def _gen_call(fn, *args) -> np.ndarray:
    out = ctypes.POINTER(ctypes.c_uint64)()
    n = ctypes.c_uint64(0)
    st = fn(*args, ctypes.byref(out), ctypes.byref(n))
    if st:
        raise DagcError(ERR_INVALID_ARGUMENT, f"generator failed ({st})")
    try:
        return np.ctypeslib.as_array(out, (n.value,)).copy() if n.value else np.zeros(0, np.uint64)
    finally:
        gen_lib().dagc_gen_free(out)


def gen_sphere_shell(depth: int = 7, seed: int = 0xDA6C0DE, target_fragments: float = 0.0) -> np.ndarray:
    return _gen_call(gen_lib().dagc_gen_sphere_shell, depth, seed, float(target_fragments))


def gen_terrain(depth: int = 11, seed: int = 0xDA6C0DE + 1, column_fraction: float = 1.0) -> np.ndarray:
    return _gen_call(gen_lib().dagc_gen_terrain, depth, seed, float(column_fraction))


def gen_soup_triangles(depth: int = 13, seed: int = 0xDA6C0DE + 2, num_triangles: int = 2_000_000) -> np.ndarray:
    """The triangles of gen_triangle_soup (same arguments), grid units, shape (n, 3, 3)."""
    out = np.zeros((num_triangles, 3, 3), np.float64)
    if gen_lib().dagc_gen_soup_triangles(depth, seed, num_triangles, out.ctypes.data if num_triangles else None):
        raise ValueError("bad generator arguments")
    return out


def gen_triangle_soup(depth: int = 13, seed: int = 0xDA6C0DE + 2, num_triangles: int = 2_000_000,
                      threads: int = 0) -> np.ndarray:
    threads = threads or (os.cpu_count() or 1)
    return _gen_call(gen_lib().dagc_gen_triangle_soup, depth, seed, num_triangles, threads)


def gen_batched(chunk_depth: int = 10, grid_xz: int = 16, chunk_row: int = 7, seed: int = 0xDA6C0DE + 3,
                min_fragments: float = 1e4, max_fragments: float = 8e6, threads: int = 0):
    """(codes, counts, chunk_morton): chunk-local codes concatenated in chunk Morton order."""
    threads = threads or (os.cpu_count() or 1)
    G = gen_lib()
    P = ctypes.POINTER(ctypes.c_uint64)
    codes, counts, morton = P(), P(), P()
    total, k = ctypes.c_uint64(0), ctypes.c_uint64(0)
    st = G.dagc_gen_batched(chunk_depth, grid_xz, chunk_row, seed, float(min_fragments), float(max_fragments),
                            threads, ctypes.byref(codes), ctypes.byref(total), ctypes.byref(counts),
                            ctypes.byref(morton), ctypes.byref(k))
    if st:
        raise DagcError(ERR_INVALID_ARGUMENT, f"batched generator failed ({st})")
    try:
        c = np.ctypeslib.as_array(codes, (total.value,)).copy() if total.value else np.zeros(0, np.uint64)
        n = np.ctypeslib.as_array(counts, (k.value,)).copy()
        m = np.ctypeslib.as_array(morton, (k.value,)).copy()
        return c, n, m
    finally:
        G.dagc_gen_free(codes)
        G.dagc_gen_free(counts)
        G.dagc_gen_free(morton)
