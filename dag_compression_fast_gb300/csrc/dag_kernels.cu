// DAG construction kernels for sm_103a: fused fragment-unique + leaf build,
// level extract + node hash, hash-run unique with a full-compare collision
// check, and the final word layout. Each is a persistent kernel over
// 2048-item tiles taken in order from an atomic counter, with a single-value
// decoupled look-back (bounded waits) for its compaction offsets, so counts
// never leave the device.
//
// Reference steps replaced (src/DAGCompression.cu):
//   SelectUnique :396-422 + leaf ReduceByKey :424-463 at :1035-1068 -> leaf_build
//   ExtractLevel :916-974 + ComputeHashes :827-833 / HashChildren :765-774 -> extract_level
//   SortLevel's flags/scan/scatters :886-913 -> unique_runs
//   ComputeChildPositions :834-844 + WriteTo :845-861 + leaf copy :1597 -> final_*

#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

#include <algorithm>

namespace dagc {
namespace {

constexpr int kT = kScanThreads;  // 256
constexpr int kI = kScanItems;    // 8 items per thread (blocked)
constexpr int kTile = kScanTile;  // 2048
// Padded shared index for blocked access of 64-bit items: one pad word per 8.
__device__ __forceinline__ int pad8(int i) { return i + (i >> 3); }
constexpr int kPadded = kTile + kTile / 8;

__device__ __forceinline__ uint64_t load_count(const uint64_t* d_n, uint64_t n) { return d_n ? *d_n : n; }

// Takes the next tile id for the CTA (thread 0 fetches, all threads read).
__device__ __forceinline__ uint32_t next_tile(uint32_t* counter, uint32_t* s_slot) {
    if (threadIdx.x == 0) *s_slot = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t t = *s_slot;
    return t;
}

// ---------------------------------------------------------------------------
// Fused unique + leaf build.
// ---------------------------------------------------------------------------
// Tiles of kLeafTile sorted keys; thread t holds keys [16t, 16t + 16) of the
// tile in registers (one 128-byte line, eight 16-byte loads), so shared memory
// carries only one word per thread. 512 threads per tile, two CTAs per SM:
// every tile waits once for its predecessors' run counts (the look-back), so
// larger tiles wait less per key.
constexpr int kLeafItems = 16;
constexpr int kLeafThreads = 512;
static_assert(kLeafTile == kLeafThreads * kLeafItems, "leaf tile = 512 threads x 16 keys");

struct LeafSmem {
    uint64_t lead[kLeafThreads];   // OR of the thread's keys before its first run head (all keys if none)
    uint8_t has_head[kLeafThreads];
    uint32_t scan[34];
    uint32_t slot;
    uint64_t p_base;
};

// Batched input: (segment << seg_shift) | local -> (seg_code[segment] << seg_shift) | local.
__device__ __forceinline__ uint64_t global_code(const LeafBuildArgs& a, uint64_t key) {
    if (!a.seg_code) return key;
    const uint64_t local = key & ((1ull << a.seg_shift) - 1);
    return (__ldg(a.seg_code + (key >> a.seg_shift)) << a.seg_shift) | local;
}

// Fused unique + leaf build. A run is a maximal range of keys with equal
// key >> 6 (composite keys of the batched form have the same runs as their
// global codes, since seg_shift >= 6); each tile emits the runs that START in
// it as (parent, mask) pairs. A run is written by the thread holding its
// head, which ORs in the leading keys of the following threads (shared
// memory) up to the next head. Keys before the tile's first head continue a
// run of an earlier tile: their OR goes to lead_or[tile] and leaf_fixup folds
// it in after this kernel.
__global__ void __launch_bounds__(kLeafThreads, 2) leaf_build(LeafBuildArgs a) {
    pdl_prologue();
    __shared__ LeafSmem S;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (a.gate && *a.gate != a.gate_run) return;
    const uint64_t n = load_count(a.d_n, a.n_bound);
    const uint32_t ntiles = leaf_tiles(n);
    if (blockIdx.x >= ntiles) return;  // grids are sized by an upper bound on n
    while (true) {
        const uint32_t tile = next_tile(a.tile_counter, &S.slot);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kLeafTile;
        const uint64_t i0 = base + (uint64_t)tid * kLeafItems;
        // Valid keys of this thread: the first nv.
        const uint32_t nv = i0 >= n ? 0u : (uint32_t)(n - i0 < (uint64_t)kLeafItems ? n - i0 : kLeafItems);
        uint64_t k[kLeafItems];
        if (nv == kLeafItems) {
            const ulonglong2* src = reinterpret_cast<const ulonglong2*>(a.sorted + i0);
#pragma unroll
            for (int j = 0; j < kLeafItems / 2; ++j) {
                const ulonglong2 v = __ldg(src + j);
                k[2 * j] = v.x;
                k[2 * j + 1] = v.y;
            }
        } else {
#pragma unroll
            for (int j = 0; j < kLeafItems; ++j) k[j] = (uint32_t)j < nv ? __ldg(a.sorted + i0 + j) : 0;
        }
        // Previous key's parent: the previous thread's last key (lane 0 reads it).
        uint64_t prev = __shfl_up_sync(0xFFFFFFFFu, k[kLeafItems - 1], 1);
        if (lane == 0 && i0 > 0 && nv > 0) prev = __ldg(a.sorted + i0 - 1);
        const bool has_prev = i0 > 0;
        uint32_t heads = 0;
        uint64_t lead = 0;
        {
            uint64_t pv = prev >> 6;
#pragma unroll
            for (int j = 0; j < kLeafItems; ++j) {
                if ((uint32_t)j < nv) {
                    const uint64_t par = k[j] >> 6;
                    if ((j == 0 && !has_prev) || par != pv) heads |= 1u << j;
                    if (!heads) lead |= 1ull << (k[j] & 63);
                    pv = par;
                }
            }
        }
        S.lead[tid] = lead;
        S.has_head[tid] = heads != 0;
        uint32_t total_heads;
        const uint32_t excl = block_exclusive_sum<uint32_t>((uint32_t)__popc(heads), S.scan, &total_heads);
        if (warp == 0) {
            const uint64_t pb = sv_lookback(a.status, tile, total_heads, a.err);
            if (lane == 0) S.p_base = pb;
        }
        __syncthreads();
        const uint64_t p_base = S.p_base;
        bool overflow = false;
        if (heads) {
            // Runs starting here: each ends at the next head of this thread or
            // continues through the following threads' leading keys.
            uint64_t r = p_base + excl;
            uint64_t acc = 0, parent = 0;
            bool open = false;
#pragma unroll
            for (int j = 0; j < kLeafItems; ++j) {
                if ((uint32_t)j < nv) {
                    if ((heads >> j) & 1u) {
                        if (open) {
                            if (r < a.out_capacity) { a.parents[r] = parent; a.leaves[r] = acc; } else overflow = true;
                            ++r;
                        }
                        open = true;
                        acc = 0;
                        parent = global_code(a, k[j]) >> 6;
                    }
                    acc |= open ? 1ull << (k[j] & 63) : 0ull;
                }
            }
            for (uint32_t t = tid + 1; t < (uint32_t)kLeafThreads; ++t) {
                acc |= S.lead[t];
                if (S.has_head[t]) break;
            }
            if (r < a.out_capacity) { a.parents[r] = parent; a.leaves[r] = acc; } else overflow = true;
        }
        if (overflow) atomicOr(a.err, kErrCapacity);
        if (tid == 0) {
            // Keys continuing the previous run: folded in by leaf_fixup. Tile 0
            // starts with a head, so it never has any.
            uint64_t lo = 0;
            for (uint32_t t = 0; t < (uint32_t)kLeafThreads; ++t) {
                lo |= S.lead[t];
                if (S.has_head[t]) break;
            }
            a.lead_or[tile] = lo;
            a.lead_run[tile] = p_base - 1;
            if (base + kLeafTile >= n) {
                const uint64_t cnt = p_base + total_heads;
                *a.d_out_n = cnt < a.out_capacity ? cnt : a.out_capacity;
            }
        }
        __syncthreads();
    }
}

// ORs every tile's leading keys into the run they continue (written by an
// earlier tile of leaf_build, one launch before, with a plain store).
__global__ void leaf_fixup(LeafBuildArgs a) {
    pdl_prologue();
    if (a.gate && *a.gate != a.gate_run) return;
    const uint64_t n = load_count(a.d_n, a.n_bound);
    const uint32_t ntiles = leaf_tiles(n);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
        if (t == 0) continue;
        const uint64_t m = a.lead_or[t];
        const uint64_t r = a.lead_run[t];
        if (m && r < a.out_capacity) atomicOr((unsigned long long*)&a.leaves[r], (unsigned long long)m);
    }
}

// ---------------------------------------------------------------------------
// Extract one level + node hash. Child codes are unique and sorted, so a
// parent owns at most 8 consecutive children. Each step is one round trip
// for the whole tile rather than a chain per thread: the tile's child codes
// and ids, then all their hashes (gathered at once into shared memory); the
// nodes' first children are compacted in shared memory and the CTA's threads
// take the nodes in turn, so a sparse level (one child per node) costs what a
// dense one does.
// ---------------------------------------------------------------------------
struct ExtractSmem {
    uint64_t codes[kPadded];   // the tile's child codes (blocked reads padded)
    uint64_t hash[kTile];      // the tile's child hashes
    uint32_t map[kTile];       // the tile's child ids
    uint16_t head[kTile + 1];  // first child of each node in the tile, in order; then tile_n
    uint32_t scan[34];
    uint32_t slot;
    uint64_t p_base;
};

// Three CTAs per SM (80 registers, ~47 KB of shared memory each): one more
// tile's round trips in flight per SM than the two that 109 registers allowed.
__global__ void __launch_bounds__(kT, 3) extract_level(ExtractArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ExtractSmem& S = *reinterpret_cast<ExtractSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t n = load_count(a.d_n, a.n_bound);
    const uint32_t ntiles = scan_tiles(n);
    // Fused insert (node levels of the hash-set form): table and buckets sized
    // by the child count n, which bounds the node count.
    const DedupArgs& dd = a.dedup;
    bool fuse = a.fuse_insert != 0 && n <= kFuseInsertMax;
    uint64_t tslots = 0;
    int shift = 64;
    uint32_t nb = 0;
    if (fuse) {
        tslots = table_size_for(n, false);
        nb = topbit_buckets(n, &shift);
        if (tslots > dd.table_cap || n > dd.item_cap || (uint64_t)nb * kDedupTopBitCap > dd.bucket_area) {
            if (blockIdx.x == 0 && threadIdx.x == 0) { atomicOr(a.err, kErrFallback); dd.state->nbuckets = 0; }
            fuse = false;
        } else if (blockIdx.x == 0 && threadIdx.x == 0) {
            dd.state->nbuckets = nb;
            dd.state->inserted = 1u;
        }
    }
    const bool read_first = n > kDedupClaimFirstMax;
    uint32_t* aux = reinterpret_cast<uint32_t*>(dd.table_aux);  // slot s: [4s] representative, [4s+1] unique id
    bool bad = false, full = false, overflow = false;
    if (blockIdx.x >= ntiles) return;  // grids are sized by an upper bound on n
    while (true) {
        const uint32_t tile = next_tile(a.tile_counter, &S.slot);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kTile;
        const uint32_t tile_n = (uint32_t)(n - base < (uint64_t)kTile ? n - base : (uint64_t)kTile);
        {
            uint32_t m[kI];
#pragma unroll
            for (int k = 0; k < kI; ++k) {
                const int i = tid + k * kT;
                if (i < (int)tile_n) {
                    S.codes[pad8(i)] = a.child_codes[base + i];
                    m[k] = a.child_map[base + i];
                    S.map[i] = m[k];
                }
            }
#pragma unroll
            for (int k = 0; k < kI; ++k) {
                const int i = tid + k * kT;
                if (i < (int)tile_n) S.hash[i] = __ldg(a.child_hashes + m[k]);
            }
        }
        __syncthreads();
        const int i0 = tid * kI;
        uint32_t head_bits = 0, heads = 0;
        {
            bool hp;
            uint64_t pv;
            if (i0 == 0) { hp = base > 0; pv = hp ? (a.child_codes[base - 1] >> 3) : 0; }
            else { hp = true; pv = i0 - 1 < (int)tile_n ? (S.codes[pad8(i0 - 1)] >> 3) : 0; }
#pragma unroll
            for (int j = 0; j < kI; ++j) {
                const int i = i0 + j;
                if (i < (int)tile_n) {
                    const uint64_t par = S.codes[pad8(i)] >> 3;
                    if (!hp || par != pv) { head_bits |= 1u << j; ++heads; }
                    pv = par;
                    hp = true;
                }
            }
        }
        uint32_t total_heads;
        const uint32_t excl = block_exclusive_sum<uint32_t>(heads, S.scan, &total_heads);
        {
            uint32_t r = excl;
#pragma unroll
            for (int j = 0; j < kI; ++j)
                if (head_bits & (1u << j)) S.head[r++] = (uint16_t)(i0 + j);
            if (tid == 0) S.head[total_heads] = (uint16_t)tile_n;
        }
        if (warp == 0) {
            const uint64_t pb = sv_lookback(a.status, tile, total_heads, a.err);
            if (lane == 0) S.p_base = pb;
        }
        __syncthreads();
        const uint64_t p_base = S.p_base;
        for (uint32_t h = tid; h < total_heads; h += kT) {
            const uint64_t p = p_base + h;
            if (p >= a.out_capacity) { overflow = true; break; }
            const int i = S.head[h], e = S.head[h + 1];
            const uint64_t par = S.codes[pad8(i)] >> 3;
            uint32_t ch[8];
            uint64_t hc[8];
#pragma unroll
            for (int c = 0; c < 8; ++c) { ch[c] = kEmptyChild; hc[c] = 0; }
            uint32_t mask = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                uint64_t code, hk;
                uint32_t id;
                if (i + k < e) {
                    code = S.codes[pad8(i + k)];
                    id = S.map[i + k];
                    hk = S.hash[i + k];
                } else if (e == (int)tile_n && base + i + k < n) {
                    // The tile's last node may go on into the next tile.
                    code = a.child_codes[base + i + k];
                    if ((code >> 3) != par) break;
                    id = a.child_map[base + i + k];
                    hk = __ldg(a.child_hashes + id);
                } else {
                    break;
                }
                const uint32_t slot = (uint32_t)(code & 7);
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (slot == (uint32_t)c) { ch[c] = id; hc[c] = hk; }
                mask |= 1u << slot;
            }
            const uint64_t hv = hash_children(hc);
            a.node_codes[p] = par;
            a.node_masks[p] = (uint8_t)mask;
            uint4* dst = reinterpret_cast<uint4*>(a.node_children + p * 8);
            dst[0] = make_uint4(ch[0], ch[1], ch[2], ch[3]);
            dst[1] = make_uint4(ch[4], ch[5], ch[6], ch[7]);
            a.node_hashes[p] = hv;
            if (fuse) {
                // The node's hash into the dedup table; the first inserter of
                // a hash is its representative and appends it to its bucket.
                uint64_t sl = home_slot(hv, tslots);
                bool won = false, placed = false;
                if (hv == 0) {
                    bad = true;  // 0 marks an empty slot
                } else {
                    for (uint64_t probe = 0; probe < tslots; ++probe) {
                        uint64_t cur = read_first ? ld_relaxed(dd.table_key + 2 * sl) : 0ull;
                        if (cur == 0)
                            cur = atomicCAS((unsigned long long*)(dd.table_key + 2 * sl), 0ull, (unsigned long long)hv);
                        if (cur == 0 || cur == hv) { won = cur == 0; placed = true; break; }
                        sl = next_slot(sl, tslots);
                    }
                }
                if (!placed && hv != 0) full = true;
                dd.item_slot[p] = placed ? (uint32_t)sl : 0xFFFFFFFFu;
                if (won) {
                    aux[4 * sl] = (uint32_t)p;
                    const uint32_t b = shift >= 64 ? 0u : (uint32_t)(hv >> shift);
                    const uint32_t bs = atomicAdd(dd.bucket_count + b, 1u);
                    if (bs < kDedupTopBitCap) {
                        const uint64_t be = (uint64_t)b * kDedupTopBitCap + bs;
                        dd.bucket[be] = make_uint4((uint32_t)hv, (uint32_t)(hv >> 32), (uint32_t)sl, (uint32_t)p);
                    } else {
                        full = true;
                    }
                }
            }
        }
        if (tid == 0 && base + tile_n == n) {
            const uint64_t cnt = p_base + total_heads;
            *a.d_out_n = cnt < a.out_capacity ? cnt : a.out_capacity;
        }
        __syncthreads();
    }
    if (overflow) atomicOr(a.err, kErrCapacity);
    if (bad) atomicOr(a.err, kErrBadInput);
    if (full) atomicOr(a.err, kErrFallback);
}

// ---------------------------------------------------------------------------
// Unique over runs of equal keys (after the hash sort), with the collision
// check: every run member must carry the same mask and children as its
// predecessor in the run.
// ---------------------------------------------------------------------------
struct UniqueSmem {
    uint64_t keys[kPadded];
    uint32_t perm[kTile];
    uint32_t scan[34];
    uint32_t slot;
    uint64_t p_base;
};

__global__ void __launch_bounds__(kT) unique_runs(UniqueArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    UniqueSmem& S = *reinterpret_cast<UniqueSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t n = load_count(a.d_n, a.n_bound);
    const uint32_t ntiles = scan_tiles(n);
    if (blockIdx.x >= ntiles) return;  // grids are sized by an upper bound on n
    while (true) {
        const uint32_t tile = next_tile(a.tile_counter, &S.slot);
        if (tile >= ntiles) break;
        const uint64_t base = (uint64_t)tile * kTile;
        const uint32_t tile_n = (uint32_t)(n - base < (uint64_t)kTile ? n - base : (uint64_t)kTile);
        for (int i = tid; i < (int)tile_n; i += kT) {
            S.keys[pad8(i)] = a.keys[base + i];
            S.perm[i] = a.perm[base + i];
        }
        __syncthreads();
        const int i0 = tid * kI;
        uint32_t head_bits = 0, heads = 0;
        bool collision = false;
        {
            bool hp;
            uint64_t pv;
            uint32_t pperm = 0;
            if (i0 == 0) {
                hp = base > 0;
                pv = hp ? a.keys[base - 1] : 0;
                pperm = hp ? a.perm[base - 1] : 0;
            } else {
                hp = true;
                pv = i0 - 1 < (int)tile_n ? S.keys[pad8(i0 - 1)] : 0;
                pperm = i0 - 1 < (int)tile_n ? S.perm[i0 - 1] : 0;
            }
            for (int j = 0; j < kI; ++j) {
                const int i = i0 + j;
                if (i >= (int)tile_n) break;
                const uint64_t k = S.keys[pad8(i)];
                const uint32_t pm = S.perm[i];
                if (!hp || k != pv) {
                    head_bits |= 1u << j;
                    ++heads;
                } else if (a.children) {
                    const uint4* x = reinterpret_cast<const uint4*>(a.children + (uint64_t)pm * 8);
                    const uint4* y = reinterpret_cast<const uint4*>(a.children + (uint64_t)pperm * 8);
                    const uint4 x0 = x[0], x1 = x[1], y0 = y[0], y1 = y[1];
                    const bool same = a.masks[pm] == a.masks[pperm] && x0.x == y0.x && x0.y == y0.y &&
                                      x0.z == y0.z && x0.w == y0.w && x1.x == y1.x && x1.y == y1.y &&
                                      x1.z == y1.z && x1.w == y1.w;
                    collision |= !same;
                }
                pv = k;
                pperm = pm;
                hp = true;
            }
        }
        if (__any_sync(0xFFFFFFFFu, collision) && lane == 0) atomicOr(a.err, kErrCollision);
        uint32_t total_heads;
        const uint32_t excl = block_exclusive_sum<uint32_t>(heads, S.scan, &total_heads);
        if (warp == 0) {
            const uint64_t pb = sv_lookback(a.status, tile, total_heads, a.err);
            if (lane == 0) S.p_base = pb;
        }
        __syncthreads();
        // uid of the run an item belongs to; items before the tile's first
        // head continue the previous tile's last run (uid p_base - 1).
        int64_t uid = (int64_t)S.p_base + excl - 1;
        bool overflow = false;
        for (int j = 0; j < kI; ++j) {
            const int i = i0 + j;
            if (i >= (int)tile_n) break;
            const uint32_t pm = S.perm[i];
            if (head_bits & (1u << j)) {
                ++uid;
                if ((uint64_t)uid < a.out_capacity) {
                    a.out_keys[uid] = S.keys[pad8(i)];
                    if (a.out_masks) a.out_masks[uid] = a.masks[pm];
                    if (a.out_children) {
                        const uint4* src = reinterpret_cast<const uint4*>(a.children + (uint64_t)pm * 8);
                        uint4* dst = reinterpret_cast<uint4*>(a.out_children + (uint64_t)uid * 8);
                        dst[0] = src[0];
                        dst[1] = src[1];
                    }
                } else {
                    overflow = true;
                }
            }
            a.map[pm] = (uint64_t)uid < a.out_capacity ? (uint32_t)uid : (uint32_t)(a.out_capacity - 1);
        }
        if (overflow) atomicOr(a.err, kErrCapacity);
        if (tid == 0 && base + tile_n == n) {
            const uint64_t cnt = S.p_base + total_heads;
            *a.d_out_n = cnt < a.out_capacity ? cnt : a.out_capacity;
        }
        __syncthreads();
    }
}


// ---------------------------------------------------------------------------
// Tail: all levels with at most kTailCap nodes, in one CTA.
// ---------------------------------------------------------------------------
struct TailSmem {
    uint64_t code[2][kTailCap];   // node codes of the level being built / its children
    uint64_t key[kTailCap];       // node hashes, by node
    uint32_t idx[kTailCap];       // sorted position -> node (by hash, then node)
    uint32_t map[2][kTailCap];    // node -> unique id, per level (ping-pong)
    uint64_t uhash[kTailCap];     // the level's unique hashes: the next level's child hashes
    uint32_t first[kTailCap];     // node -> index of its first child (its children follow it)
    uint8_t mask[kTailCap];
    uint32_t scan[34];
    uint32_t flags;
};
static_assert(sizeof(TailSmem) <= 227 * 1024, "tail state fits one CTA's shared memory");
// The sort's buckets: at most 2^kTailBucketLog, one per thread for the scan;
// node ids in bucket order + count, start and fill cursor per bucket, in the
// room of uhash.
constexpr int kTailBucketLog = 10;
constexpr uint32_t kTailBuckets = 1u << kTailBucketLog;
static_assert(kTailBuckets <= (uint32_t)kTailThreads && (4u << kTailBucketLog) >= (uint32_t)kTailCap, "tail buckets");
static_assert((kTailCap + 3 * kTailBuckets) * 4 <= sizeof(uint64_t) * kTailCap, "tail buckets fit uhash");

__global__ void __launch_bounds__(kTailThreads) tail_levels(TailArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TailSmem& S = *reinterpret_cast<TailSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x;
    if (tid == 0) S.flags = 0;
    const uint64_t* cc = a.child_codes;
    const uint32_t* cm = a.child_map;
    const uint64_t* ch = a.child_hashes;
    uint64_t nc = *a.d_child_n;
    if (nc <= (uint64_t)kTailCap) {
        // The first level's children (codes, ids, and the hashes their ids
        // index, all below nc) into shared memory, every load in flight at
        // once; each level then reads only shared memory.
        constexpr int kPer = kTailCap / kTailThreads;
        uint64_t c[kPer], h[kPer];
        uint32_t m[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const uint32_t i = tid + k * kTailThreads;
            if (i < nc) { c[k] = cc[i]; m[k] = cm[i]; h[k] = ch[i]; }
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const uint32_t i = tid + k * kTailThreads;
            if (i < nc) { S.code[1][i] = c[k]; S.map[1][i] = m[k]; S.uhash[i] = h[k]; }
        }
        cc = S.code[1];
        cm = S.map[1];
        ch = S.uhash;
    }
    int ping = 0;
    __syncthreads();
    for (int l = a.first_level; l >= 0; --l) {
        const TailLevelOut& out = a.lv[l];
        const uint64_t cap = out.capacity < (uint64_t)kTailCap ? out.capacity : (uint64_t)kTailCap;
        uint64_t* node_code = S.code[ping];
        uint32_t* node_map = S.map[ping];
        // Extract: one node per distinct child code >> 3; its first child
        // (the head of the run) is recorded in node order.
        uint64_t nn = 0;
        for (uint64_t c0 = 0; c0 < nc; c0 += kTailThreads) {
            const uint64_t i = c0 + tid;
            bool head = false;
            uint64_t par = 0;
            if (i < nc) {
                par = cc[i] >> 3;
                head = i == 0 || (cc[i - 1] >> 3) != par;
            }
            uint32_t total;
            const uint32_t excl = block_exclusive_sum<uint32_t>(head ? 1u : 0u, S.scan, &total);
            if (head) {
                const uint64_t p = nn + excl;
                if (p < cap) {
                    node_code[p] = par;
                    S.first[p] = (uint32_t)i;
                } else {
                    atomicOr(&S.flags, kErrCapacity);
                }
            }
            nn += total;
            __syncthreads();
        }
        const uint32_t n = (uint32_t)(nn < cap ? nn : cap);
        // Hash: one node per thread (dense warps); a node's children run from
        // its first child to the next node's.
        for (uint32_t p = tid; p < n; p += kTailThreads) {
            const uint32_t f = S.first[p];
            const uint64_t e = p + 1 < n ? (uint64_t)S.first[p + 1] : nc;
            const uint32_t cnt = (uint32_t)(e - f < 8 ? e - f : 8);
            uint64_t code[8], h[8];
            uint32_t id[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                code[k] = 0;
                id[k] = 0;
                h[k] = 0;
                if ((uint32_t)k < cnt) { code[k] = cc[f + k]; id[k] = cm[f + k]; }
            }
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                if ((uint32_t)k >= cnt) continue;
                const uint32_t slot = (uint32_t)(code[k] & 7);
                const uint64_t hk = ch[id[k]];
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (slot == (uint32_t)c) h[c] = hk;
                m |= 1u << slot;
            }
            S.key[p] = hash_children(h);
            S.mask[p] = (uint8_t)m;
        }
        __syncthreads();
        // Sort of the nodes by (hash, node): counting sort on the hash's top
        // bits (the hashes are uniform: ~4 nodes per bucket), then each node's
        // rank among its bucket's. The order goes to idx (sorted position ->
        // node); the hashes stay by node. The buckets use uhash's room, free
        // from the hashing to the unique pass.
        {
            uint32_t* border = reinterpret_cast<uint32_t*>(S.uhash);
            uint32_t* bcnt = border + kTailCap;
            uint32_t* bstart = bcnt + kTailBuckets;
            uint32_t* bfill = bstart + kTailBuckets;
            int lb = 0;
            while (lb < kTailBucketLog && (4u << lb) < n) ++lb;
            const uint32_t nb = 1u << lb;
            for (uint32_t b = tid; b < nb; b += kTailThreads) bcnt[b] = 0;
            __syncthreads();
            for (uint32_t p = tid; p < n; p += kTailThreads)
                atomicAdd(&bcnt[lb ? (uint32_t)(S.key[p] >> (64 - lb)) : 0u], 1u);
            __syncthreads();
            uint32_t total;
            const uint32_t ex = block_exclusive_sum<uint32_t>(tid < nb ? bcnt[tid] : 0u, S.scan, &total);
            if (tid < nb) {
                bstart[tid] = ex;
                bfill[tid] = ex;
            }
            __syncthreads();
            for (uint32_t p = tid; p < n; p += kTailThreads) {
                const uint32_t b = lb ? (uint32_t)(S.key[p] >> (64 - lb)) : 0u;
                border[atomicAdd(&bfill[b], 1u)] = p;
            }
            __syncthreads();
            for (uint32_t p = tid; p < n; p += kTailThreads) {
                const uint64_t k = S.key[p];
                const uint32_t b = lb ? (uint32_t)(k >> (64 - lb)) : 0u;
                const uint32_t s0 = bstart[b], s1 = s0 + bcnt[b];
                uint32_t rank = 0;
                for (uint32_t j = s0; j < s1; ++j) {
                    const uint32_t q = border[j];
                    const uint64_t kq = S.key[q];
                    rank += kq < k || (kq == k && q < p);
                }
                S.idx[s0 + rank] = p;
            }
            __syncthreads();
        }
        // Unique with the full compare; node -> unique id into node_map. A
        // node's children are the popc(mask) children from its first one on,
        // in slot order.
        uint64_t uid_base = 0;
        for (uint32_t c0 = 0; c0 < n; c0 += kTailThreads) {
            const uint32_t i = c0 + tid;
            bool head = false;
            if (i < n) {
                const uint32_t x = S.idx[i];
                head = i == 0 || S.key[x] != S.key[S.idx[i - 1]];
                if (!head) {
                    const uint32_t y = S.idx[i - 1];
                    bool same = S.mask[x] == S.mask[y];
                    const uint32_t fx = S.first[x], fy = S.first[y], cnt = __popc((uint32_t)S.mask[x]);
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if ((uint32_t)k < cnt) same &= cm[fx + k] == cm[fy + k];
                    if (!same) atomicOr(&S.flags, kErrCollision);
                }
            }
            uint32_t total;
            const uint32_t excl = block_exclusive_sum<uint32_t>(head ? 1u : 0u, S.scan, &total);
            if (i < n) {
                // Items before the chunk's first head continue the previous run.
                const uint64_t uid = uid_base + excl + (head ? 1 : 0) - 1;
                const uint32_t x = S.idx[i];
                node_map[x] = (uint32_t)uid;
                if (head && uid < out.capacity) {
                    out.hashes[uid] = S.key[x];
                    S.uhash[uid] = S.key[x];
                    const uint32_t m = S.mask[x], f = S.first[x], cnt = __popc(m);
                    out.masks[uid] = (uint8_t)m;
                    uint32_t chd[8];
#pragma unroll
                    for (int c = 0; c < 8; ++c) chd[c] = kEmptyChild;
                    uint64_t code[8];
                    uint32_t id[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        code[k] = 0;
                        id[k] = 0;
                        if ((uint32_t)k < cnt) { code[k] = cc[f + k]; id[k] = cm[f + k]; }
                    }
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        if ((uint32_t)k >= cnt) continue;
                        const uint32_t slot = (uint32_t)(code[k] & 7);
#pragma unroll
                        for (int c = 0; c < 8; ++c)
                            if (slot == (uint32_t)c) chd[c] = id[k];
                    }
                    uint4* dst = reinterpret_cast<uint4*>(out.children + uid * 8);
                    dst[0] = make_uint4(chd[0], chd[1], chd[2], chd[3]);
                    dst[1] = make_uint4(chd[4], chd[5], chd[6], chd[7]);
                }
            }
            uid_base += total;
            __syncthreads();
        }
        if (tid == 0) {
            *out.d_nodes = n;
            *out.d_unique = uid_base;
        }
        // The next level's children are this level's nodes.
        cc = node_code;
        cm = node_map;
        ch = S.uhash;
        nc = n;
        ping ^= 1;
        __syncthreads();
    }
    if (tid == 0 && S.flags) atomicOr(a.err, S.flags);
}

// ---------------------------------------------------------------------------
// Final layout.
// ---------------------------------------------------------------------------
struct FinalScanSmem {
    uint32_t scan[34];
    uint32_t slot;
    uint64_t p_base;
};

// The level table of FinalArgs in shared memory (indexed at run time).
struct FinalLevels {
    const uint8_t* masks[kFinalMaxLevels];
    const uint32_t* children[kFinalMaxLevels];
    uint64_t off[kFinalMaxLevels + 1];
};
__device__ __forceinline__ void load_levels(const FinalArgs& a, FinalLevels& L) {
    const int t = threadIdx.x;
    if (t < a.num_levels) { L.masks[t] = a.lv_masks[t]; L.children[t] = a.lv_children[t]; }
    if (t <= a.num_levels) L.off[t] = a.lv_off[t];
    __syncthreads();
}
// Level of node i, searching up from level l (nodes are visited in order).
__device__ __forceinline__ int level_of(const FinalLevels& L, int num_levels, uint64_t i, int l) {
    while (l + 1 < num_levels && i >= L.off[l + 1]) ++l;
    return l;
}

// word_pos[i] = sum over nodes j < i of (popc(mask_j) + 1); word_pos[n] = total.
__global__ void __launch_bounds__(kT) final_positions(FinalArgs a) {
    pdl_prologue();
    __shared__ FinalScanSmem S;
    __shared__ FinalLevels LV;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t n = a.num_nodes;
    const uint32_t ntiles = scan_tiles(n);
    if (blockIdx.x >= ntiles) return;  // grids are sized by an upper bound on n
    load_levels(a, LV);
    while (true) {
        const uint32_t tile = next_tile(a.tile_counter, &S.slot);
        if (tile >= ntiles) break;
        const uint64_t i0 = (uint64_t)tile * kTile + (uint64_t)tid * kI;
        uint32_t w[kI];
        uint32_t sum = 0;
        int l = level_of(LV, a.num_levels, i0, 0);
#pragma unroll
        for (int j = 0; j < kI; ++j) {
            w[j] = 0;
            if (i0 + j < n) {
                l = level_of(LV, a.num_levels, i0 + j, l);
                w[j] = (uint32_t)__popc(LV.masks[l][i0 + j - LV.off[l]]) + 1u;
            }
            sum += w[j];
        }
        uint32_t total;
        const uint32_t excl = block_exclusive_sum<uint32_t>(sum, S.scan, &total);
        if (warp == 0) {
            const uint64_t pb = sv_lookback(a.status, tile, total, a.err);
            if (lane == 0) S.p_base = pb;
        }
        __syncthreads();
        uint64_t pos = S.p_base + excl;
#pragma unroll
        for (int j = 0; j < kI; ++j) {
            if (i0 + j < n) a.word_pos[i0 + j] = (uint32_t)pos;
            pos += w[j];
        }
        if (tid == 0 && (uint64_t)(tile + 1) * kTile >= n) {
            a.word_pos[n] = (uint32_t)(S.p_base + total);
            *a.d_total = S.p_base + total;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kT) final_write(FinalArgs a) {
    pdl_prologue();
    __shared__ FinalLevels LV;
    load_levels(a, LV);
    const uint64_t* s_off = LV.off;
    const uint64_t n = a.num_nodes;
    const uint64_t leaf_start = a.word_pos[n];
    const uint64_t gstride = (uint64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n + a.num_leaves; i += gstride) {
        if (i >= n) {
            const uint64_t j = i - n;
            const uint64_t leaf = a.leaves[j];
            a.words[leaf_start + 2 * j] = (uint32_t)leaf;
            a.words[leaf_start + 2 * j + 1] = (uint32_t)(leaf >> 32);
            continue;
        }
        const int l = level_of(LV, a.num_levels, i, 0);
        const bool last = l + 1 == a.num_levels;
        const uint64_t li = i - s_off[l];
        const uint32_t mask = LV.masks[l][li];
        const uint64_t pos = a.word_pos[i];
        a.words[pos] = mask;
        const uint4* src = reinterpret_cast<const uint4*>(LV.children[l] + li * 8);
        const uint4 c0 = src[0], c1 = src[1];
        const uint32_t ch[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
        uint32_t k = 1;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const bool has = (mask >> c) & 1u;
            // WriteTo's structural check (src/DAGCompression.cu:860) plus a
            // range check, so a malformed DAG can never index out of bounds.
            const uint64_t limit = last ? a.num_leaves : s_off[l + 2] - s_off[l + 1];
            const bool ok = has == (ch[c] != kEmptyChild) && (!has || ch[c] < limit);
            bad |= !ok;
            if (!has || !ok) continue;
            const uint64_t ptr = last ? leaf_start + 2ull * ch[c] : a.word_pos[s_off[l + 1] + ch[c]];
            a.words[pos + k++] = (uint32_t)ptr;
        }
    }
    if (bad) atomicOr(a.err, kErrBadInput);
}

// ---------------------------------------------------------------------------
// Small helpers.
// ---------------------------------------------------------------------------
__global__ void remap_children(const uint32_t* __restrict__ in, const uint32_t* __restrict__ map,
                               uint32_t* __restrict__ out, uint64_t n_words) {
    pdl_prologue();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t c = in[i];
        out[i] = c == kEmptyChild ? kEmptyChild : map[c];
    }
}

// Up to kCopyUnroll units per thread: every load is issued before any store.
constexpr int kCopyUnroll = 8;
template <typename T>
__device__ __forceinline__ void copy_units(const CopySeg& c, uint64_t t0, uint64_t stride) {
    const T* src = static_cast<const T*>(c.src);
    T* dst = static_cast<T*>(c.dst);
    const uint64_t n = c.bytes / sizeof(T);
    for (uint64_t i0 = t0; i0 < n; i0 += stride * kCopyUnroll) {
        T v[kCopyUnroll];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u)
            if (i0 + u * stride < n) v[u] = src[i0 + u * stride];
#pragma unroll
        for (int u = 0; u < kCopyUnroll; ++u)
            if (i0 + u * stride < n) dst[i0 + u * stride] = v[u];
    }
}

// CTA b copies piece b - first_cta[k] of segment k, where first_cta[k] <= b <
// first_cta[k + 1]; a piece is up to kCopyPiece bytes.
__global__ void __launch_bounds__(256) copy_segments(CopyTable t) {
    pdl_prologue();
    if (blockIdx.x == 0 && (int)threadIdx.x < t.lit_count) t.lit_dst[threadIdx.x] = t.lit[threadIdx.x];
    int k = 0;
    while (k + 1 < t.count && t.first_cta[k + 1] <= blockIdx.x) ++k;
    if (k >= t.count || blockIdx.x >= t.first_cta[t.count]) return;
    CopySeg c = t.seg[k];
    const uint64_t off = (uint64_t)(blockIdx.x - t.first_cta[k]) * kCopyPiece;
    const uint64_t len = c.bytes - off < kCopyPiece ? c.bytes - off : kCopyPiece;
    c.src = static_cast<const char*>(c.src) + off;
    c.dst = static_cast<char*>(c.dst) + off;
    c.bytes = len;
    const uint64_t align = (uint64_t)(uintptr_t)c.src | (uint64_t)(uintptr_t)c.dst | c.bytes;
    if ((align & 15) == 0) copy_units<uint4>(c, threadIdx.x, blockDim.x);
    else if ((align & 7) == 0) copy_units<uint64_t>(c, threadIdx.x, blockDim.x);
    else if ((align & 3) == 0) copy_units<uint32_t>(c, threadIdx.x, blockDim.x);
    else copy_units<uint8_t>(c, threadIdx.x, blockDim.x);
}

__global__ void iota_offset(uint32_t* out, uint64_t n, uint32_t offset) {
    pdl_prologue();
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = offset + (uint32_t)i;
}

int g_blocks_small = 152 * 8;

// Asks for a shared-memory carveout that holds `ctas` CTAs of `smem` bytes
// (the driver's default may pick a smaller one and cap the occupancy).
void prefer_shared(const void* fn, size_t smem, int ctas) {
    int dev = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (per_sm <= 0) return;
    const size_t want = (size_t)ctas * (smem + 1024);  // 1 KB reserved per CTA
    const int pct = (int)std::min<size_t>(100, (want * 100 + per_sm - 1) / per_sm);
    cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
}

}  // namespace

void kernels_configure() {
    cudaFuncSetAttribute(leaf_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(LeafSmem));
    cudaFuncSetAttribute(extract_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ExtractSmem));
    prefer_shared(reinterpret_cast<const void*>(extract_level), sizeof(ExtractSmem), 3);
    cudaFuncSetAttribute(unique_runs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(UniqueSmem));
    cudaFuncSetAttribute(tail_levels, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TailSmem));
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    g_blocks_small = sms * 8;
}

int occupancy_kernel(int which) {
    int occ = 0;
    switch (which) {
        case kKernelLeafBuild:
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, leaf_build, kLeafThreads, 0);
            break;
        case kKernelExtract:
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, extract_level, kT, sizeof(ExtractSmem));
            break;
        case kKernelUnique:
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, unique_runs, kT, sizeof(UniqueSmem));
            break;
        case kKernelFinalWrite:
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, final_write, kT, 0);
            break;
        default:
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, final_positions, kT, 0);
            break;
    }
    return occ;
}

void launch_leaf_build(const LeafBuildArgs& a, cudaStream_t s) {
    launch_pdl(leaf_build, dim3(a.grid), dim3(kLeafThreads), 0, s, a);
    const uint64_t tiles = leaf_tiles(a.n_bound);
    const int grid = (int)std::min<uint64_t>((tiles + 255) / 256, (uint64_t)g_blocks_small);
    launch_pdl(leaf_fixup, dim3(grid > 0 ? grid : 1), dim3(256), 0, s, a);
}
void launch_extract(const ExtractArgs& a, cudaStream_t s) {
    launch_pdl(extract_level, dim3(a.grid), dim3(kT), sizeof(ExtractSmem), s, a);
}
void launch_unique(const UniqueArgs& a, cudaStream_t s) {
    launch_pdl(unique_runs, dim3(a.grid), dim3(kT), sizeof(UniqueSmem), s, a);
}
void launch_tail(const TailArgs& a, cudaStream_t s) {
    launch_pdl(tail_levels, dim3(1), dim3(kTailThreads), sizeof(TailSmem), s, a);
}
void launch_final_positions(const FinalArgs& a, cudaStream_t s) {
    launch_pdl(final_positions, dim3(a.grid_scan), dim3(kT), 0, s, a);
}
void launch_final_write(const FinalArgs& a, cudaStream_t s) {
    launch_pdl(final_write, dim3(a.grid_write), dim3(kT), 0, s, a);
}
void launch_remap_children(const uint32_t* in, const uint32_t* map, uint32_t* out, uint64_t n_nodes,
                           cudaStream_t s) {
    if (n_nodes == 0) return;
    const uint64_t words = n_nodes * 8;
    const int grid = (int)std::min<uint64_t>((words + 255) / 256, (uint64_t)g_blocks_small);
    launch_pdl(remap_children, dim3(grid), dim3(256), 0, s, in, map, out, words);
}
void launch_copy_segments(const CopyTable& t, cudaStream_t s) {
    if (t.count <= 0 && t.lit_count <= 0) return;
    CopyTable c = t;
    uint64_t ctas = 0;
    for (int i = 0; i < c.count; ++i) {
        c.first_cta[i] = (uint32_t)ctas;
        ctas += (c.seg[i].bytes + kCopyPiece - 1) / kCopyPiece;
    }
    c.first_cta[c.count] = (uint32_t)ctas;
    launch_pdl(copy_segments, dim3((unsigned)std::max<uint64_t>(ctas, 1)), dim3(256), 0, s, c);
}
void launch_iota_offset(uint32_t* out, uint64_t n, uint32_t offset, cudaStream_t s) {
    if (n == 0) return;
    const int grid = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)g_blocks_small);
    launch_pdl(iota_offset, dim3(grid), dim3(256), 0, s, out, n, offset);
}

}  // namespace dagc
