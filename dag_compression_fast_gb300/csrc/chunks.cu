// Batched form: the leaves of many chunks in one persistent launch, for
// sm_103a. Replaces, for dagc_create_batched, the fragment sort + unique +
// leaf build of every chunk (the reference runs SortKeys, SelectUnique and
// ReduceByKey once per subvolume, src/DAGCompression.cu:1026-1068, called per
// chunk from src/DAG_Compression_Fast.cpp:283-302).
//
// Every chunk's local brick space (bricks = local code >> 6, 3*chunk_depth - 6
// bits) is cut into 2^bin_bits bins of 2^D bricks each, D <= 13, so that one
// bin's leaf masks fit a direct-mapped array in shared memory, with a bitmap
// of the bricks present: the bricks of a bin come out in ascending order by
// walking the bitmap, with no sort. One
// persistent grid takes work items from a device counter, in this order:
//   COUNT(c, t)   tile t of chunk c: the chunk's bin histogram;
//   SCATTER(c, t) tile t of chunk c, after all of c's COUNT tiles: fragments
//                 to their bins (bin starts from the histogram, one global
//                 reservation per bin and tile);
//   LEAVES(c, g)  32 consecutive bins of chunk c, after all of c's SCATTER
//                 tiles: per bin, OR every fragment's voxel bit into its
//                 brick's mask, then emit the non-empty bricks in order.
// Small chunks (one bin) skip COUNT and SCATTER: their LEAVES item reads the
// input. A CTA waits only on items taken before its own (taken by running
// CTAs that wait only on earlier items still), so the waits end; each is
// bounded anyway. Two small launches then pack the bricks of all items into
// one ascending list: a scan of the items' brick counts and a copy.

#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

namespace dagc {
namespace {

constexpr int kT = kChunkThreads;
constexpr int kMaxBins = 1 << kChunkMaxBinBits;
constexpr int kDirect = 1 << kChunkDirectBits;
constexpr int kPerThread = kChunkTile / kT;
static_assert(kChunkTile % kT == 0 && kDirect % kT == 0 && kMaxBins % kT == 0, "chunk shapes");

constexpr int kBitmapWords = kDirect / 32;
static_assert(kBitmapWords <= kT, "one bitmap word per thread");

struct ChunkSmem {
    struct {
        uint32_t tcnt[kMaxBins];   // this tile's fragments per bin (then its reservation base)
        uint32_t start[kMaxBins];  // the chunk's bin starts (exclusive scan of its histogram)
    } bins;
    // One bin's leaf masks, by brick, as two 32-bit halves (native shared
    // atomics); zero between bins (the emission clears what it reads), and a
    // bitmap of the bricks present.
    uint32_t masks[2 * kDirect];
    uint32_t present[kBitmapWords];
    uint32_t bin_cnt[kChunkGroupBins];  // fragments of the LEAVES item's bins
    uint32_t scan[34];
    uint32_t item;
    uint64_t running;
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 waits (bounded) until *counter reaches target; then the CTA.
__device__ __forceinline__ void wait_counter(const uint32_t* counter, uint32_t target, uint32_t* err) {
    if (threadIdx.x == 0) {
        uint32_t it = 0;
        while (ld_acquire(counter) < target) {
            if (++it > kSpinLimit) { atomicOr(err, kErrTimeout); break; }
            backoff(it);
        }
    }
    __syncthreads();
}

// The chunk of a COUNT / SCATTER tile (tile_off ascending, k + 1 entries).
__device__ __forceinline__ uint32_t chunk_of_tile(const uint32_t* tile_off, uint32_t k, uint32_t t) {
    uint32_t lo = 0, hi = k;  // tile_off[lo] <= t < tile_off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(tile_off + mid) <= t) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(kT) chunk_leaves(ChunkArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ChunkSmem& S = *reinterpret_cast<ChunkSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x;
    const uint32_t nb = 1u << a.bin_bits;
    const int lb = 3 * a.chunk_depth - 6;                    // local brick bits
    const int dbits = lb - a.bin_bits;                        // direct-mapped brick bits of a bin
    const uint32_t dsize = 1u << dbits;
    const uint64_t code_limit = 1ull << (3 * a.chunk_depth);
    // The tile count comes from the device (tile_off[k]): a recorded graph
    // replayed for other chunk sizes still sees the current one.
    const uint32_t tiles = __ldg(a.tile_off + a.k);
    const uint32_t total = 2 * tiles + a.k * a.groups_per_chunk;
    bool bad = false;
    for (uint32_t x = tid; x < 2u * kDirect; x += kT) S.masks[x] = 0;
    while (true) {
        if (tid == 0) S.item = atomicAdd(a.work, 1u);
        __syncthreads();
        const uint32_t item = S.item;
        __syncthreads();
        if (item >= total) break;
        if (item < 2 * tiles) {
            // ------------------------------------------- COUNT / SCATTER ----
            const bool scatter = item >= tiles;
            const uint32_t t = scatter ? item - tiles : item;
            const uint32_t c = chunk_of_tile(a.tile_off, a.k, t);
            const uint32_t tc = __ldg(a.tile_off + c + 1) - __ldg(a.tile_off + c);
            const uint64_t c0 = __ldg(a.seg_offsets + c), c1 = __ldg(a.seg_offsets + c + 1);
            const uint64_t f0 = c0 + (uint64_t)(t - __ldg(a.tile_off + c)) * kChunkTile;
            const uint32_t fn = (uint32_t)min((uint64_t)kChunkTile, c1 - f0);
            uint32_t* hist = a.hist + (uint64_t)c * nb;
            if (scatter) {
                wait_counter(a.done + c, tc, a.err);
                // Bin starts: exclusive scan of the chunk's histogram.
                constexpr int kPer = kMaxBins / kT;
                uint32_t h[kPer], sum = 0, tot;
#pragma unroll
                for (int q = 0; q < kPer; ++q) {
                    const uint32_t b = tid * kPer + q;
                    h[q] = b < nb ? hist[b] : 0u;
                    sum += h[q];
                }
                uint32_t run = block_exclusive_sum<uint32_t>(sum, S.scan, &tot);
#pragma unroll
                for (int q = 0; q < kPer; ++q) {
                    S.bins.start[tid * kPer + q] = run;
                    run += h[q];
                }
            }
            for (uint32_t b = tid; b < nb; b += kT) S.bins.tcnt[b] = 0;
            __syncthreads();
            uint32_t br[kPerThread];  // bin << 16 | rank of the fragment among the tile's of its bin
#pragma unroll
            for (int q = 0; q < kPerThread; ++q) {
                const uint32_t i = q * kT + tid;
                br[q] = 0xFFFFFFFFu;
                if (i < fn) {
                    const uint64_t code = __ldg(a.frags + f0 + i);
                    if (code >= code_limit) bad = true;
                    uint32_t bin = (uint32_t)((code >> 6) >> dbits);
                    bin = bin < nb ? bin : nb - 1;
                    const uint32_t r = atomicAdd(&S.bins.tcnt[bin], 1u);
                    br[q] = bin << 16 | r;
                }
            }
            __syncthreads();
            if (!scatter) {
                for (uint32_t b = tid; b < nb; b += kT) {
                    const uint32_t x = S.bins.tcnt[b];
                    if (x) atomicAdd(hist + b, x);
                }
                __threadfence();  // every thread's counts land before the tile is marked done
                __syncthreads();
                if (tid == 0) {
                    __threadfence();
                    atomicAdd(a.done + c, 1u);
                }
                continue;
            }
            // One reservation per bin and tile.
            for (uint32_t b = tid; b < nb; b += kT) {
                const uint32_t x = S.bins.tcnt[b];
                if (x) S.bins.tcnt[b] = atomicAdd(a.cursor + (uint64_t)c * nb + b, x);
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < kPerThread; ++q) {
                if (br[q] == 0xFFFFFFFFu) continue;
                const uint32_t i = q * kT + tid, bin = br[q] >> 16;
                const uint64_t dst = c0 + S.bins.start[bin] + S.bins.tcnt[bin] + (br[q] & 0xFFFFu);
                if (dst < c1) a.scratch[dst] = __ldg(a.frags + f0 + i);
                else bad = true;  // only after a timed-out wait
            }
            __threadfence();  // every thread's fragments land before the tile is marked done
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                atomicAdd(a.done + a.k + c, 1u);
            }
            continue;
        }
        // --------------------------------------------------------- LEAVES ----
        const uint32_t gi = item - 2 * tiles;
        const uint32_t c = gi / a.groups_per_chunk, g = gi % a.groups_per_chunk;
        const uint64_t c0 = __ldg(a.seg_offsets + c), c1 = __ldg(a.seg_offsets + c + 1);
        const uint32_t b0 = g * kChunkGroupBins, b1 = min(nb, b0 + kChunkGroupBins);
        const uint64_t pbase = __ldg(a.seg_code + c) << (a.seg_shift - 6);  // global brick of local brick 0
        const uint32_t* hist = a.hist + (uint64_t)c * nb;
        const uint64_t* src = nb > 1 ? a.scratch : a.frags;
        uint64_t gstart = c0;  // fragment offset of bin b0 (and of the group's bricks)
        if (nb > 1) {
            const uint32_t tc = __ldg(a.tile_off + c + 1) - __ldg(a.tile_off + c);
            if (tc) wait_counter(a.done + a.k + c, tc, a.err);
            uint32_t part = 0;
            for (uint32_t b = tid; b < b0; b += kT) part += hist[b];
            uint32_t tot;
            block_exclusive_sum<uint32_t>(part, S.scan, &tot);
            gstart += tot;
        }
        if (tid == 0) S.running = 0;
        if (nb > 1 && tid < b1 - b0) S.bin_cnt[tid] = hist[b0 + tid];
        __syncthreads();
        uint64_t fstart = gstart;
        for (uint32_t b = b0; b < b1; ++b) {
            const uint64_t cnt = nb > 1 ? S.bin_cnt[b - b0] : c1 - c0;
            if (cnt == 0) continue;
            if (tid < (uint32_t)kBitmapWords) S.present[tid] = 0;
            __syncthreads();
            // Four fragments per thread in flight, then their updates: the
            // voxel bit goes to its brick's low or high half; the first bit
            // of a half marks the brick present.
            for (uint64_t i0 = tid; i0 < cnt; i0 += 4 * kT) {
                uint64_t code[4];
                bool in[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint64_t i = i0 + (uint64_t)u * kT;
                    in[u] = i < cnt;
                    code[u] = in[u] ? src[fstart + i] : 0ull;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (!in[u]) continue;
                    if (nb == 1 && code[u] >= code_limit) bad = true;
                    const uint32_t e = (uint32_t)(code[u] >> 6) & (dsize - 1);
                    const uint32_t v = (uint32_t)code[u] & 63u;
                    const uint32_t old = atomicOr(&S.masks[2 * e + (v >> 5)], 1u << (v & 31));
                    if (old == 0) atomicOr(&S.present[e >> 5], 1u << (e & 31));
                }
            }
            fstart += cnt;
            __syncthreads();
            // The bin's bricks in order: thread t owns bitmap word t (bricks
            // 32t .. 32t + 31); a block scan of the words' counts gives the
            // output positions. Every mask read is cleared for the next bin.
            const uint32_t word = tid < (uint32_t)kBitmapWords ? S.present[tid] : 0u;
            uint32_t tot;
            uint32_t pos = block_exclusive_sum<uint32_t>((uint32_t)__popc(word), S.scan, &tot);
            const uint64_t out0 = gstart + S.running;
            for (uint32_t w = word; w; w &= w - 1) {
                const uint32_t e = tid * 32 + (__ffs(w) - 1);
                const uint64_t m = (uint64_t)S.masks[2 * e] | (uint64_t)S.masks[2 * e + 1] << 32;
                S.masks[2 * e] = 0;
                S.masks[2 * e + 1] = 0;
                const uint64_t o = out0 + pos++;
                if (o < c1) {
                    a.stage_parent[o] = pbase | ((uint64_t)b << dbits) | e;
                    a.stage_mask[o] = m;
                }
            }
            __syncthreads();
            if (tid == 0) S.running += tot;
            __syncthreads();
        }
        if (tid == 0) {
            a.group_bricks[gi] = (uint32_t)S.running;
            a.group_src[gi] = gstart;
        }
    }
    if (__syncthreads_or(bad) && tid == 0) atomicOr(a.err, kErrBadInput);
}

// Exclusive scan of the items' brick counts (one CTA; items in order) and
// the total, clamped to the output capacity.
__global__ void __launch_bounds__(1024) chunk_scan(ChunkArgs a) {
    pdl_prologue();
    __shared__ uint32_t scan[34];
    const uint32_t g = a.k * a.groups_per_chunk;
    uint64_t carry = 0;
    for (uint32_t b = 0; b < g; b += 1024) {
        const uint32_t i = b + threadIdx.x;
        const uint32_t v = i < g ? a.group_bricks[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_sum<uint32_t>(v, scan, &tot);
        if (i < g) {
            const uint64_t d = carry + ex;
            a.group_dst[i] = d < 0xFFFFFFFFull ? (uint32_t)d : 0xFFFFFFFFu;
        }
        carry += tot;
    }
    if (threadIdx.x == 0) {
        if (carry > a.out_capacity) atomicOr(a.err, kErrCapacity);
        *a.d_out_n = carry < a.out_capacity ? carry : a.out_capacity;
    }
}

// Packs the items' bricks into the ascending list: every thread moves a run
// of consecutive output bricks (balanced whatever the items' sizes), finding
// the item of its first brick by binary search over the items' output
// starts and walking forward from there.
constexpr int kCopyPer = 8;
__global__ void __launch_bounds__(256) chunk_copy(ChunkArgs a) {
    pdl_prologue();
    const uint32_t g = a.k * a.groups_per_chunk;
    const uint64_t total = *a.d_out_n;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kCopyPer;
    for (uint64_t j0 = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kCopyPer; j0 < total; j0 += stride) {
        uint32_t lo = 0, hi = g;  // group_dst[lo] <= j0 < group_dst[hi] (ascending)
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (a.group_dst[mid] <= j0) lo = mid; else hi = mid;
        }
        uint32_t w = lo;
        for (uint64_t j = j0; j < j0 + kCopyPer && j < total; ++j) {
            while (w + 1 < g && a.group_dst[w + 1] <= j) ++w;
            const uint64_t src = a.group_src[w] + (j - a.group_dst[w]);
            a.parents[j] = a.stage_parent[src];
            a.leaves[j] = a.stage_mask[src];
        }
    }
}

int g_chunk_ctas = 0;

}  // namespace

void chunk_configure(int sms) {
    cudaFuncSetAttribute(chunk_leaves, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ChunkSmem));
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, chunk_leaves, kT, sizeof(ChunkSmem));
    g_chunk_ctas = (occ > 0 ? occ : 1) * (sms > 0 ? sms : 152);
}

int chunk_bin_bits(int chunk_depth) {
    const int lb = 3 * chunk_depth - 6;
    return lb > kChunkDirectBits ? lb - kChunkDirectBits : 0;
}

void launch_chunk_leaves(const ChunkArgs& a, cudaStream_t s) {
    const uint64_t items = 2ull * a.tiles + (uint64_t)a.k * a.groups_per_chunk;
    const int grid = (int)(items < (uint64_t)g_chunk_ctas ? (items ? items : 1) : g_chunk_ctas);
    launch_pdl(chunk_leaves, dim3(grid), dim3(kT), sizeof(ChunkSmem), s, a);
    launch_pdl(chunk_scan, dim3(1), dim3(1024), 0, s, a);
    // The brick total is on the device: the grid covers the bound and extra
    // threads leave at once.
    const uint64_t blocks = (a.out_capacity + 256ull * kCopyPer - 1) / (256ull * kCopyPer);
    launch_pdl(chunk_copy, dim3((unsigned)(blocks < 8192 ? (blocks ? blocks : 1) : 8192)), dim3(256), 0, s, a);
}

}  // namespace dagc
