// Fragment grouping by hash, for sm_103a: an alternative to the fragment sort
// + leaf build (src/DAGCompression.cu:1026-1068: SortKeys, SelectUnique,
// ReduceByKey) for inputs where many fragments share a brick. Both produce
// the same arrays: the distinct bricks (code >> 6) in ascending order and,
// per brick, the OR of 1 << (code & 63) over its fragments.
//
// Bricks are split into partitions by the top bits of a hash of the brick, so
// that one partition's distinct bricks fit a table in shared memory:
//
//   group_probe      reads one 64-byte line of fragments in 16 (every
//                    fragment of small inputs) into a HyperLogLog sketch
//                    (4096 registers) of their bricks;
//   group_plan       one CTA: grouping when the sample shows few enough
//                    distinct bricks for the redundancy the grouping needs
//                    (the limit comes from the sampling model, group_shape),
//                    else the sort path (every kernel of the other path reads
//                    the decision and does nothing); picks 2^k partitions
//                    from the estimated bricks and n, and their slabs;
//   group_scatter    the fragments, by partition, into the partitions' slabs:
//                    one CTA per SM walks its chunk of the input in tiles of
//                    8192 (the next tile streams into shared memory while one
//                    is processed), a counting sort per tile in shared memory,
//                    one atomic per partition and tile reserves the tile's
//                    runs; fragments past a full slab go to a shared overflow
//                    area; also the range check;
//   group_aggregate  one CTA per partition: a table in shared memory of the
//                    partition's bricks and their masks (an overfull table is
//                    redone in halves of the partition's hash range), then the
//                    brick list (brick, index) and the masks;
//   (then the brick list is sorted by brick with the radix sort, values =
//    indices: B items instead of N)
//   group_gather     parents and masks in sorted brick order.
//
// The scatter reads the fragments in order and writes one slab entry per
// fragment (4 bytes in the narrow form: the brick's 32-bit product without
// the partition bits, and the voxel index; else the 8-byte key), which the
// aggregation reads in order; only the B-sized brick list is sorted.

#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace dagc {
namespace {

__device__ __forceinline__ uint64_t fmix(uint64_t k) {
    // MurmurHash3's 64-bit finaliser (published constants).
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// The probe's hash: top 12 bits pick the register, the bits below give its
// rank (they must be close to uniform).
__device__ __forceinline__ uint64_t brick_hash(uint64_t brick) { return fmix(brick ^ 0x9E3779B97F4A7C15ull); }

constexpr uint32_t kNarrowMul = 0x9E3779B1u, kNarrowMulInv = 0x0E8B2F51u;
static_assert(kNarrowMul * kNarrowMulInv == 1u, "inverse mod 2^32");

// The partition's hash, one multiply (Fibonacci hashing): its top
// kGroupPartLog bits are the fine partition, the bits below them the slot in
// the partition's table. Narrow form (every brick below 2^31): a 32-bit
// multiply of the brick, and 32-bit table keys.
template <bool kNarrow>
__device__ __forceinline__ uint32_t fine_part(uint64_t brick) {
    if (kNarrow) return ((uint32_t)brick * kNarrowMul) >> (32 - kGroupPartLog);
    return (uint32_t)((brick * 0x9E3779B97F4A7C15ull) >> (64 - kGroupPartLog));
}
template <bool kNarrow>
__device__ __forceinline__ uint32_t part_of(uint64_t key, int lp) {
    return lp ? fine_part<kNarrow>(key >> 6) >> (kGroupPartLog - lp) : 0u;
}
// Sub-range of a brick within its partition: the low bits of the same
// product (the partition and the slot take the top ones).
template <bool kNarrow>
__device__ __forceinline__ uint32_t sub_of(uint64_t brick) {
    if (kNarrow) return (uint32_t)brick * kNarrowMul;
    return (uint32_t)(brick * 0x9E3779B97F4A7C15ull);
}
template <bool kNarrow>
__device__ __forceinline__ uint32_t slot_of(uint64_t brick, uint32_t lt) {
    if (kNarrow) return (((uint32_t)brick * kNarrowMul) >> (32 - kGroupPartLog - lt)) & ((1u << lt) - 1);
    return (uint32_t)((brick * 0x9E3779B97F4A7C15ull) >> (64 - kGroupPartLog - lt)) & ((1u << lt) - 1);
}

// Narrow form: the 32-bit product is a bijection of the brick (odd
// multiplier) and a partition's slab implies its top lp bits, so a slab entry
// is one word: the product's low 32 - lp bits, then the fragment's 6-bit
// voxel index (lp >= kCompactMinPartLog). The brick comes back as the product
// times the multiplier's inverse mod 2^32.
constexpr int kCompactMinPartLog = 6;
__device__ __forceinline__ uint32_t compact_word(uint64_t key, int lp) {
    const uint32_t h = (uint32_t)(key >> 6) * kNarrowMul;
    return ((h << lp) >> (lp - 6)) | (uint32_t)(key & 63);
}
// Slot and brick of a compact word's product remainder r = w >> 6 (the slot
// and sub-range bits lie within the remainder's 32 - lp bits).
__device__ __forceinline__ uint32_t compact_slot(uint32_t r, uint32_t lt) {
    return (r >> (32 - kGroupPartLog - lt)) & ((1u << lt) - 1);
}
__device__ __forceinline__ uint64_t compact_brick(uint32_t part, int lp, uint32_t r) {
    return (uint64_t)(((part << (32 - lp)) | r) * kNarrowMulInv);
}

__device__ __forceinline__ uint32_t segment_of(const uint64_t* off, uint32_t count, uint64_t i) {
    uint32_t lo = 0, hi = count;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// Key of fragment i: the code, or for batched input the composite
// (segment << seg_shift) | local code. `bad` flags codes out of range.
__device__ __forceinline__ uint64_t key_of(const GroupArgs& a, uint64_t i, uint64_t code, bool* bad) {
    if (a.validate_bits > 0 && a.validate_bits < 64 && (code >> a.validate_bits)) *bad = true;
    if (a.seg_offsets) code |= (uint64_t)segment_of(a.seg_offsets, a.seg_count, i) << a.seg_shift;
    return code;
}

__device__ __forceinline__ void chunk_range(const GroupArgs& a, uint64_t* lo, uint64_t* hi) {
    const uint64_t len = (a.n + a.chunks - 1) / a.chunks;
    const uint64_t l = (uint64_t)blockIdx.x * len;
    *lo = l < a.n ? l : a.n;
    *hi = *lo + len < a.n ? *lo + len : a.n;
}

constexpr int kSketchLog = 12;
constexpr int kSketchRegs = 1 << kSketchLog;
static_assert(kSketchRegs == kGroupSketchRegs, "sketch size");
constexpr int kFrontThreads = 512;
// The probe samples one 64-byte line (8 fragments) in kProbeStride, or every
// fragment of inputs up to kProbeAllMax.
constexpr uint32_t kProbeStride = 16;
constexpr uint64_t kProbeAllMax = 1ull << 20;

__device__ __forceinline__ void sketch_add(uint32_t* reg, uint64_t brick) {
    const uint64_t h = brick_hash(brick);
    const uint32_t rank = (uint32_t)__clzll((h << kSketchLog) | (1ull << (kSketchLog - 1))) + 1;
    atomicMax(&reg[h >> (64 - kSketchLog)], rank);
}

__global__ void __launch_bounds__(kFrontThreads) group_probe(GroupArgs a) {
    pdl_prologue();
    __shared__ uint32_t reg[kSketchRegs];
    for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x) reg[i] = 0;
    __syncthreads();
    bool unused = false;  // the range check is the scatter's
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a.n <= kProbeAllMax) {
        for (uint64_t i = t0; i < a.n; i += stride) sketch_add(reg, key_of(a, i, __ldcs(a.frags + i), &unused) >> 6);
    } else {
        // Line u of the sample: fragments [8 * (u * kProbeStride + kProbeStride / 2), + 8).
        const uint64_t lines = a.n / 8 / kProbeStride;
        for (uint64_t u = t0; u < lines; u += stride) {
            const uint64_t i0 = 8 * (u * kProbeStride + kProbeStride / 2);
            uint64_t c[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) c[k] = __ldcs(a.frags + i0 + k);
#pragma unroll
            for (int k = 0; k < 8; ++k) sketch_add(reg, key_of(a, i0 + k, c[k], &unused) >> 6);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x)
        if (reg[i]) atomicMax(a.sketch + i, reg[i]);
}

// Distinct-brick estimate from the sketch (HyperLogLog with the linear
// counting correction for small counts); the whole CTA takes part. The
// register sum is exact in fixed point (2^(52 - rank), rank >= 1, at most
// 4096 * 2^51 < 2^64); one thread finishes it in double precision, which is
// slow on this GPU.
__device__ float sketch_estimate(const uint32_t* sketch, unsigned long long* red, float* out) {
    unsigned long long sum = 0, zeros = 0;
    for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x) {
        const uint32_t r = sketch[i];
        sum += 1ull << (52 - (r < 52 ? r : 52));
        zeros += r == 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
        zeros += __shfl_xor_sync(0xFFFFFFFFu, zeros, o);
    }
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { red[2 * warp] = sum; red[2 * warp + 1] = zeros; }
    __syncthreads();
    if (threadIdx.x == 0) {
        sum = 0;
        zeros = 0;
        for (int w = 0; w < nw; ++w) { sum += red[2 * w]; zeros += red[2 * w + 1]; }
        // Single precision: the estimate only steers a choice, and double
        // precision is slow on this part.
        const float m = (float)kSketchRegs;
        const float e = 0.7213f / (1.0f + 1.079f / m) * m * m / ((float)sum * 0x1p-52f);
        *out = e <= 2.5f * m && zeros > 0 ? m * logf(m / (float)zeros) : e;
    }
    __syncthreads();
    return *out;
}

constexpr int kPlanThreads = 1024;

// Fragments per distinct brick in the probe's sample when every brick of the
// input holds rho fragments and the sample keeps each fragment with
// probability q: q * rho / (1 - (1 - q)^rho) (rho itself when q = 1).
__global__ void __launch_bounds__(kPlanThreads) group_plan(GroupArgs a) {
    pdl_prologue();
    __shared__ unsigned long long red[2 * (kPlanThreads / 32)];
    __shared__ float est_s;
    const float est = sketch_estimate(a.sketch, red, &est_s);
    __shared__ uint32_t shape[2];
    if (threadIdx.x == 0) {
        // The path: grouping when the sample holds at most probe_max_distinct
        // distinct bricks (group_shape derives it from the sampling model).
        const bool redundant = est > 0.0f && est <= a.probe_max_distinct;
        const bool group = a.mode == 2 || (a.mode == 1 && redundant);
        // The bricks: the sample's distinct count, scaled back by the
        // sampling model (the redundancy whose sampled ratio matches, by
        // bisection; the model grows with the redundancy).
        float bricks = est;
        if (a.n > kProbeAllMax && est > 0.0f) {
            const float q = 1.0f / kProbeStride;
            const float r = (float)(a.n / 8 / kProbeStride) * 8.0f / est;
            float lo = 1.0f, hi = (float)a.n;
            for (int it = 0; it < 40; ++it) {
                const float mid = 0.5f * (lo + hi);
                if (q * mid / (1.0f - powf(1.0f - q, mid)) < r) lo = mid; else hi = mid;
            }
            bricks = (float)a.n / lo;
        }
        // Partitions: at most kGroupMaxParts, and enough that each holds
        // ~kGroupTargetBricksPerPart bricks (table load ~0.35), at most 65536
        // fragments on average, and that small inputs still spread over 256
        // CTAs (4096 fragments each). Fewer, larger partitions make the
        // scatter's runs per tile longer.
        const uint64_t spread = a.n / 4096 < 256 ? a.n / 4096 : 256;
        int lp = 0;
        while (lp < kGroupPartLog && ((float)(1u << lp) * kGroupTargetBricksPerPart < bricks ||
                                      (a.n >> lp) > 65536 || (1ull << lp) < spread))
            ++lp;
        if (a.narrow && lp < kCompactMinPartLog) lp = kCompactMinPartLog;  // compact slab entries
        const uint64_t mean = (a.n + (1ull << lp) - 1) >> lp;
        shape[0] = (uint32_t)lp;
        shape[1] = (uint32_t)(mean + mean / 4 + 1024);
        a.path[0] = group ? 1u : 0u;
        a.path[1] = (uint32_t)lp;
        a.path[2] = (uint32_t)kGroupPartSlotsLog;
        a.path[3] = shape[1];
    }
    __syncthreads();
    // Partition p fills the slab [p * slab_cap, (p + 1) * slab_cap).
    for (uint32_t p = threadIdx.x; p < (1u << shape[0]); p += blockDim.x) a.cursor[p] = (uint64_t)p * shape[1];
}

// 8-byte asynchronous copy global -> shared (cp.async), and its completion.
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

constexpr int kScatterThreads = 1024;  // one CTA per SM
constexpr int kScatterPer = 8;
constexpr int kScatterTile = kScatterThreads * kScatterPer;
constexpr int kScatterMaxPer = (kGroupMaxParts + kScatterThreads - 1) / kScatterThreads;  // partitions per thread
static_assert(kScatterTile <= 65536 && kGroupMaxParts <= 65536, "rank and partition share a word");

struct ScatterSmem {
    uint64_t in[kScatterTile];       // the next tile's keys, copied in while this tile is processed
    uint64_t stage[kScatterTile];    // this tile's keys, by partition (narrow: words + partition ids)
    uint32_t cnt[kGroupMaxParts];    // the tile's count per partition, then its offset in the tile
    int64_t delta[kGroupMaxParts];   // output position - tile position, per partition
    uint32_t scan[34];
};

__device__ __forceinline__ void scatter_prefetch(ScatterSmem& sm, const uint64_t* frags, uint64_t base, uint64_t hi) {
    for (uint32_t q = threadIdx.x; q < (uint32_t)kScatterTile && base + q < hi; q += kScatterThreads)
        cp_async8(&sm.in[q], frags + base + q);
    cp_async_commit();
}

template <bool kNarrow>
__global__ void __launch_bounds__(kScatterThreads) group_scatter(GroupArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ScatterSmem& sm = *reinterpret_cast<ScatterSmem*>(smem_raw);
    // Narrow form: compact words (4 bytes) staged with their partition ids.
    uint32_t* stage_w = reinterpret_cast<uint32_t*>(sm.stage);
    uint16_t* stage_p = reinterpret_cast<uint16_t*>(stage_w + kScatterTile);
    uint32_t* parts_w = reinterpret_cast<uint32_t*>(a.parts);
    if (a.path[0] != 1u) return;
    const int lp = (int)a.path[1];
    const int parts = 1 << lp;
    const uint64_t slab_cap = a.path[3];
    uint64_t lo, hi;
    chunk_range(a, &lo, &hi);
    bool bad = false, over = false;  // codes out of range; the overflow area full
    const int per = (parts + kScatterThreads - 1) / kScatterThreads;
    for (int p = threadIdx.x; p < parts; p += kScatterThreads) sm.cnt[p] = 0;
    if (lo < hi) scatter_prefetch(sm, a.frags, lo, hi);
    for (uint64_t base = lo; base < hi; base += kScatterTile) {
        cp_async_wait_all();
        __syncthreads();  // the tile is in `in`; cnt is zero
        uint64_t key[kScatterPer];
#pragma unroll
        for (int k = 0; k < kScatterPer; ++k) key[k] = sm.in[k * kScatterThreads + threadIdx.x];
        __syncthreads();  // `in` is free for the next tile
        if (base + kScatterTile < hi) scatter_prefetch(sm, a.frags, base + kScatterTile, hi);
        uint32_t pr[kScatterPer], w[kScatterPer];
#pragma unroll
        for (int k = 0; k < kScatterPer; ++k) {
            const uint64_t i = base + (uint64_t)k * kScatterThreads + threadIdx.x;
            if (i >= hi) continue;
            key[k] = key_of(a, i, key[k], &bad);
            const uint32_t pid = part_of<kNarrow>(key[k], lp);
            if (kNarrow) w[k] = compact_word(key[k], lp);
            pr[k] = (pid << 16) | atomicAdd(&sm.cnt[pid], 1u);
        }
        __syncthreads();
        const int p0 = threadIdx.x * per;
        uint32_t sum = 0;
        for (int j = 0; j < per; ++j)
            if (p0 + j < parts) sum += sm.cnt[p0 + j];
        uint32_t tile_total;
        uint32_t run = block_exclusive_sum<uint32_t>(sum, sm.scan, &tile_total);
        // The tile's run of each partition goes right after the runs that
        // tiles reserved before it, so that the partially written sectors of
        // a partition's frontier are completed while they are in the L2.
        uint32_t c[kScatterMaxPer];
        unsigned long long g[kScatterMaxPer];
#pragma unroll
        for (int j = 0; j < kScatterMaxPer; ++j) {
            const int p = p0 + j;
            c[j] = j < per && p < parts ? sm.cnt[p] : 0u;
            g[j] = c[j] ? atomicAdd((unsigned long long*)(a.cursor + p), (unsigned long long)c[j]) : 0ull;
        }
#pragma unroll
        for (int j = 0; j < kScatterMaxPer; ++j) {
            const int p = p0 + j;
            if (j >= per || p >= parts) break;
            sm.cnt[p] = run;
            sm.delta[p] = (int64_t)g[j] - (int64_t)run;
            run += c[j];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kScatterPer; ++k) {
            const uint64_t i = base + (uint64_t)k * kScatterThreads + threadIdx.x;
            if (i >= hi) continue;
            const uint32_t off = sm.cnt[pr[k] >> 16] + (pr[k] & 0xFFFFu);
            if (kNarrow) {
                stage_w[off] = w[k];
                stage_p[off] = (uint16_t)(pr[k] >> 16);
            } else {
                sm.stage[off] = key[k];
            }
        }
        __syncthreads();
        // Write-out in tile order: runs of one partition are contiguous. The
        // wide form recomputes the partition from the key.
        const uint32_t m = (uint32_t)(hi - base < (uint64_t)kScatterTile ? hi - base : (uint64_t)kScatterTile);
        const uint32_t lane = threadIdx.x & 31;
#pragma unroll 4
        for (uint32_t q0 = 0; q0 < m; q0 += kScatterThreads) {  // uniform over the CTA: every lane votes
            const uint32_t q = q0 + threadIdx.x;
            uint64_t k = 0;  // wide: the key; narrow: the word, with the partition above it for the overflow area
            bool spill = false;
            if (q < m) {
                uint32_t pid;
                if (kNarrow) {
                    pid = stage_p[q];
                    k = ((uint64_t)pid << 32) | stage_w[q];
                } else {
                    k = sm.stage[q];
                    pid = part_of<kNarrow>(k, lp);
                }
                const uint64_t pos = (uint64_t)((int64_t)sm.delta[pid] + q);
                if (pos < (uint64_t)(pid + 1) * slab_cap) {
                    if (kNarrow) parts_w[pos] = (uint32_t)k;
                    else a.parts[pos] = k;
                } else {
                    // The partition's slab is full (a brick with very many
                    // fragments): to the shared overflow area.
                    spill = true;
                    a.part_over[pid] = 1u;
                }
            }
            const uint32_t sm_mask = __ballot_sync(0xFFFFFFFFu, spill);
            if (sm_mask) {
                unsigned long long ob = 0;
                if (lane == 0) ob = atomicAdd((unsigned long long*)a.overflow_count, (unsigned long long)__popc(sm_mask));
                ob = __shfl_sync(0xFFFFFFFFu, ob, 0);
                if (spill) {
                    const uint64_t o = ob + __popc(sm_mask & lanemask_lt());
                    if (o < a.overflow_cap) a.overflow[o] = k;
                    else over = true;
                }
            }
        }
        for (int p = threadIdx.x; p < parts; p += kScatterThreads) sm.cnt[p] = 0;  // read last before the stage barrier
    }
    if (bad) atomicOr(a.err, kErrBadInput);
    if (over) atomicOr(a.err, kErrFallback);
}

constexpr int kAggThreads = 512;
constexpr int kAggIlp = 4;
// Longest probe chain before a partition's table counts as full: at the
// planned load (< 0.45) chains stay far shorter.
constexpr uint32_t kAggMaxProbe = 256;
// A partition whose bricks overfill its table is done again in halves of its
// hash range, down to 1/2^kAggMaxSplitLog of it.
constexpr uint32_t kAggMaxSplitLog = 6;
static_assert((1 << 9) >= kAggThreads, "at least one table slot per thread");

template <bool kNarrow>
struct AggSmem {
    using Key = typename std::conditional<kNarrow, uint32_t, unsigned long long>::type;
    uint32_t full;                   // a probe chain ran out: the partition gives up
    uint64_t mask[kGroupPartSlots];  // OR of the fragments' bits
    Key key[kGroupPartSlots];        // tag (wide: brick + 1; narrow: product remainder + 1), 0 = empty
    uint32_t scan[34];
    uint64_t base;
};

// One fragment into the partition's table: find or claim its brick's slot
// (linear probing from `s`; the brick's tag is nonzero), OR its bit into the
// mask. False when the table is full.
template <bool kNarrow>
__device__ __forceinline__ bool agg_insert(AggSmem<kNarrow>& sm, typename AggSmem<kNarrow>::Key tag, uint32_t s,
                                           uint32_t bit, uint32_t slots) {
    using Key = typename AggSmem<kNarrow>::Key;
    Key cur = *reinterpret_cast<volatile Key*>(&sm.key[s]);
    if (cur != tag) {
        // Rare: the brick's first fragment here, or a collision.
        for (uint32_t probe = 0;; ) {
            if (cur == 0) {
                cur = atomicCAS(&sm.key[s], (Key)0, tag);
                if (cur == 0 || cur == tag) break;
            }
            if (++probe == kAggMaxProbe) return false;  // the table is (nearly) full: the sort path
            s = (s + 1) & (slots - 1);
            cur = *reinterpret_cast<volatile Key*>(&sm.key[s]);
            if (cur == tag) break;
        }
    }
    atomicOr(reinterpret_cast<uint32_t*>(&sm.mask[s]) + (bit >> 5), 1u << (bit & 31));
    return true;
}

// A slab entry into the table. Wide: the key, tag brick + 1. Narrow: the
// compact word, tag (product remainder) + 1, unique within the partition.
template <bool kNarrow>
__device__ __forceinline__ bool agg_entry(AggSmem<kNarrow>& sm, uint64_t e, uint32_t lt, uint32_t slots) {
    if constexpr (kNarrow) {
        const uint32_t r = (uint32_t)e >> 6;
        return agg_insert<true>(sm, r + 1, compact_slot(r, lt), (uint32_t)e & 63, slots);
    } else {
        const uint64_t brick = e >> 6;
        return agg_insert<false>(sm, brick + 1, slot_of<false>(brick, lt), (uint32_t)(e & 63), slots);
    }
}
// Sub-range bits of a slab entry: the low bits of the partition's product.
template <bool kNarrow>
__device__ __forceinline__ uint32_t entry_sub(uint64_t e) {
    return kNarrow ? (uint32_t)e >> 6 : sub_of<false>(e >> 6);
}

template <bool kNarrow>
__global__ void __launch_bounds__(kAggThreads) group_aggregate(GroupArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Smem = AggSmem<kNarrow>;
    using Key = typename Smem::Key;
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    if (a.path[0] != 1u) return;
    const int lp = (int)a.path[1];
    const uint32_t parts = 1u << lp, lt = a.path[2], slots = 1u << lt;
    const uint32_t* parts_w = reinterpret_cast<const uint32_t*>(a.parts);  // narrow: compact words
    const uint64_t slab_cap = a.path[3];
    bool full = false;
    for (uint32_t p = blockIdx.x; p < parts; p += gridDim.x) {
        const uint64_t lo = (uint64_t)p * slab_cap;
        const uint64_t hi = a.cursor[p] < lo + slab_cap ? a.cursor[p] : lo + slab_cap;
        // Work list of sub-ranges (low `level` bits of the brick's sub-hash
        // equal to `sub`), depth first: a sub-range whose bricks overfill the
        // table is done again as its two halves. The whole partition is the
        // one sub-range of level 0.
        uint32_t todo_sub[kAggMaxSplitLog + 2], todo_level[kAggMaxSplitLog + 2];
        int ntodo = 1;
        todo_sub[0] = 0;
        todo_level[0] = 0;
        while (ntodo > 0) {  // uniform over the CTA
            --ntodo;
            const uint32_t sub = todo_sub[ntodo], level = todo_level[ntodo];
            const uint32_t sub_mask = (1u << level) - 1;
            for (uint32_t s = threadIdx.x; s < slots; s += kAggThreads) {
                sm.key[s] = 0;
                sm.mask[s] = 0;
            }
            if (threadIdx.x == 0) sm.full = 0;
            __syncthreads();
            for (uint64_t i0 = lo + threadIdx.x; i0 < hi; i0 += (uint64_t)kAggIlp * kAggThreads) {
                uint64_t k[kAggIlp];
#pragma unroll
                for (int u = 0; u < kAggIlp; ++u) {
                    const uint64_t i = i0 + (uint64_t)u * kAggThreads;
                    if (kNarrow) k[u] = i < hi ? __ldcs(parts_w + i) : 0u;
                    else k[u] = i < hi ? __ldcs(a.parts + i) : 0ull;
                }
#pragma unroll
                for (int u = 0; u < kAggIlp; ++u)
                    if (i0 + (uint64_t)u * kAggThreads < hi &&
                        (level == 0 || (entry_sub<kNarrow>(k[u]) & sub_mask) == sub) &&
                        !agg_entry<kNarrow>(sm, k[u], lt, slots))
                        sm.full = 1;
                if (*reinterpret_cast<volatile uint32_t*>(&sm.full)) break;  // fail fast
            }
            if (a.part_over[p]) {
                // The partition's slab was full: the rest of its fragments are
                // in the shared overflow area, among other partitions'.
                const uint64_t no = *a.overflow_count;
                for (uint64_t i = threadIdx.x; i < no; i += kAggThreads) {
                    // Narrow entries carry their partition in the high word.
                    const uint64_t k = a.overflow[i];
                    const uint32_t kp = kNarrow ? (uint32_t)(k >> 32) : part_of<kNarrow>(k, lp);
                    const uint64_t e = kNarrow ? (uint64_t)(uint32_t)k : k;
                    if (kp == p && (level == 0 || (entry_sub<kNarrow>(e) & sub_mask) == sub) &&
                        !agg_entry<kNarrow>(sm, e, lt, slots))
                        sm.full = 1;
                    if (*reinterpret_cast<volatile uint32_t*>(&sm.full)) break;
                }
            }
            __syncthreads();
            if (sm.full) {
                __syncthreads();  // everyone has read the flag before the table is cleared again
                if (level < kAggMaxSplitLog) {
                    todo_sub[ntodo] = sub | (1u << level);
                    todo_level[ntodo++] = level + 1;
                    todo_sub[ntodo] = sub;
                    todo_level[ntodo++] = level + 1;
                } else {
                    full = true;  // too many bricks even in a 1/64 sub-range: the call reruns on the sort path
                }
                continue;
            }
            const uint32_t per = slots / kAggThreads, s0 = threadIdx.x * per;
            uint32_t cnt = 0;
            for (uint32_t j = 0; j < per; ++j) cnt += sm.key[s0 + j] != 0;
            uint32_t total;
            const uint32_t ex = block_exclusive_sum<uint32_t>(cnt, sm.scan, &total);
            if (threadIdx.x == 0)
                sm.base = total ? atomicAdd((unsigned long long*)a.d_count, (unsigned long long)total) : 0ull;
            __syncthreads();
            uint64_t pos = sm.base + ex;
            for (uint32_t j = 0; j < per; ++j) {
                const uint64_t t = (uint64_t)sm.key[s0 + j];
                if (t == 0) continue;
                if (pos < a.cap) {
                    a.bricks[pos] = kNarrow ? compact_brick(p, lp, (uint32_t)t - 1) : t - 1;
                    a.idx[pos] = (uint32_t)pos;
                    a.masks[pos] = sm.mask[s0 + j];
                } else {
                    full = true;
                }
                ++pos;
            }
            __syncthreads();  // the table is cleared for the next sub-range
        }
    }
    if (full) atomicOr(a.err, kErrFallback);
}

constexpr int kGatherIlp = 4;

__global__ void __launch_bounds__(256) group_gather(GroupArgs a) {
    pdl_prologue();
    if (a.path[0] != 1u) return;
    const uint64_t count = *a.d_count < a.cap ? *a.d_count : a.cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.d_count = count;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t lmask = a.seg_code ? (1ull << (a.seg_shift - 6)) - 1 : 0;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < count; i0 += stride * kGatherIlp) {
        uint32_t j[kGatherIlp];
        uint64_t b[kGatherIlp], m[kGatherIlp];
#pragma unroll
        for (int k = 0; k < kGatherIlp; ++k) {
            const uint64_t i = i0 + k * stride;
            j[k] = i < count ? a.sorted_idx[i] : 0xFFFFFFFFu;
            b[k] = i < count ? a.sorted_bricks[i] : 0;
        }
#pragma unroll
        for (int k = 0; k < kGatherIlp; ++k) m[k] = j[k] < a.cap ? a.masks[j[k]] : 0;
#pragma unroll
        for (int k = 0; k < kGatherIlp; ++k) {
            const uint64_t i = i0 + k * stride;
            if (i >= count) continue;
            // Batched input: composite brick (segment << (seg_shift - 6)) | local
            // brick -> the chunk's Morton index in place of the segment.
            uint64_t parent = b[k];
            if (a.seg_code) parent = (__ldg(a.seg_code + (b[k] >> (a.seg_shift - 6))) << (a.seg_shift - 6)) | (b[k] & lmask);
            a.parents[i] = parent;
            a.leaves[i] = m[k];
        }
    }
}

int g_group_sms = 152;

}  // namespace

void group_configure(int sms) {
    g_group_sms = sms > 0 ? sms : 152;
    cudaFuncSetAttribute(group_scatter<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ScatterSmem));
    cudaFuncSetAttribute(group_scatter<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(ScatterSmem));
    cudaFuncSetAttribute(group_aggregate<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(AggSmem<false>));
    cudaFuncSetAttribute(group_aggregate<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sizeof(AggSmem<true>));
}

int group_chunks(uint64_t n) {
    const uint64_t want = (n + kScatterTile - 1) / kScatterTile;
    const uint64_t most = (uint64_t)(g_group_sms < kGroupMaxChunks ? g_group_sms : kGroupMaxChunks);
    return (int)(want < 1 ? 1 : (want < most ? want : most));
}

void launch_group_probe(const GroupArgs& a, cudaStream_t s) {
    const uint64_t units = a.n <= kProbeAllMax ? a.n : a.n / 8 / kProbeStride;
    const uint64_t want = (units + kFrontThreads - 1) / kFrontThreads;
    const int g = (int)(want < (uint64_t)(2 * g_group_sms) ? (want > 0 ? want : 1) : 2 * g_group_sms);
    launch_pdl(group_probe, dim3(g), dim3(kFrontThreads), 0, s, a);
}

void group_shape(uint64_t n, uint64_t* slab_total, float* probe_max_distinct) {
    // The partitions (2^k of them, chosen on the device) split the slab
    // region into slabs of 1.25 x the mean + 1024 fragments.
    *slab_total = n + n / 4 + (uint64_t)kGroupMaxParts * 1026;
    const int lp = kGroupPartLog;
    // The path's test. If every brick held rho fragments, a sample keeping
    // each fragment with probability q would hold q * rho / (1 - (1 - q)^rho)
    // fragments per distinct brick (rho when q = 1), a ratio that grows with
    // rho. Grouping needs kGroupMinRedundancy fragments per brick, and the
    // tables' capacity needs n / (kGroupMaxBricksPerPart * partitions): the
    // larger bound sets the least ratio, hence the most distinct bricks the
    // sample may show.
    const bool all = n <= kProbeAllMax;
    const double q = all ? 1.0 : 1.0 / kProbeStride;
    const double sampled = all ? (double)n : (double)(n / 8 / kProbeStride) * 8.0;
    const double rho = std::max(kGroupMinRedundancy, (double)n / (kGroupMaxBricksPerPart * (double)(1ull << lp)));
    const double ratio = all ? rho : q * rho / (1.0 - std::pow(1.0 - q, rho));
    *probe_max_distinct = (float)(sampled / ratio);
}
void launch_group_plan(const GroupArgs& a, cudaStream_t s) { launch_pdl(group_plan, dim3(1), dim3(kPlanThreads), 0, s, a); }
void launch_group_scatter(const GroupArgs& a, cudaStream_t s) {
    if (a.narrow) launch_pdl(group_scatter<true>, dim3(a.chunks), dim3(kScatterThreads), sizeof(ScatterSmem), s, a);
    else launch_pdl(group_scatter<false>, dim3(a.chunks), dim3(kScatterThreads), sizeof(ScatterSmem), s, a);
}
void launch_group_aggregate(const GroupArgs& a, cudaStream_t s) {
    if (a.narrow)  // 48 KB of table: four CTAs per SM
        launch_pdl(group_aggregate<true>, dim3(4 * g_group_sms), dim3(kAggThreads), sizeof(AggSmem<true>), s, a);
    else
        launch_pdl(group_aggregate<false>, dim3(3 * g_group_sms), dim3(kAggThreads), sizeof(AggSmem<false>), s, a);
}

void launch_group_gather(const GroupArgs& a, cudaStream_t s) {
    const uint64_t want = (a.cap + 1023) / 1024;
    const int g = (int)(want < (uint64_t)(8 * g_group_sms) ? (want > 0 ? want : 1) : 8 * g_group_sms);
    launch_pdl(group_gather, dim3(g), dim3(256), 0, s, a);
}

}  // namespace dagc
