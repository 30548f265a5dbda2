// Stable LSD radix sort of uint64 keys (optionally with uint32 values) on a
// bit range, for sm_103a. Replaces cub::DeviceRadixSort::SortKeys/SortPairs
// (src/DAGCompression.cu:336-394) and thrust::sequence (:743-750).
//
// Structure (one-sweep style):
//   1. radix_histogram: one read of the keys builds the histogram of every
//      digit pass at once (shared-memory counters, then global atomics),
//      validates the key range and clears the first pass's look-back status.
//   2. onesweep_pass, once per digit: a persistent grid takes tiles of keys in
//      order from an atomic counter, ranks keys inside each warp with
//      __match_any_sync or per-bit ballots, publishes per-digit tile counts,
//      finds the tile's global digit offsets by decoupled look-back (bounded
//      waits), stages the tile in shared memory in digit order and writes it
//      out so that equal digits land in contiguous runs.
// Digits are 8 bits wide for key/value sorts and 8 to 11 bits for keys-only
// sorts (fewer passes over the keys; the digit width and the pass shape are
// chosen per sort, see sort_plan_valid and the context's tuning table). The
// digits of a sort are balanced: a 33-bit range in four passes takes widths
// 9, 8, 8, 8.
// All counts can be device-resident (d_n), so a whole pipeline runs without a
// host round trip.

#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

#include <algorithm>
#include <cstddef>

namespace dagc {
namespace {

// Look-back status word of one digit of one tile: 0 until the tile publishes;
// then the count + 1 in bits 0-30 (counts up to 2^31 - 2) and bit 31 set once
// the count is the inclusive prefix over all tiles up to this one (clear: the
// tile's own count).
constexpr uint32_t kSInc = 1u << 31;
constexpr uint32_t kSVal = (1u << 31) - 1;

constexpr int kPassThreads = 256;

// A device-resident count never exceeds the bound its buffers were sized for.
__device__ __forceinline__ uint64_t load_n(const uint64_t* d_n, uint64_t n) {
    if (!d_n) return n;
    const uint64_t v = *d_n;
    return v < n ? v : n;
}

// Segment of position i (seg_offsets ascending, count + 1 entries): binary
// search for the first position of a block, then `segment_advance` follows it.
__device__ __forceinline__ uint32_t segment_search(const uint64_t* off, uint32_t count, uint64_t i) {
    uint32_t lo = 0, hi = count;  // invariant: off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}
// Segment of a later position from the segment of an earlier one (`hint`):
// a few steps forward, then a binary search over the rest.
__device__ __forceinline__ uint32_t segment_advance(const uint64_t* off, uint32_t count, uint64_t i, uint32_t hint) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (hint + 1 >= count || __ldg(off + hint + 1) > i) return hint;
        ++hint;
    }
    uint32_t lo = hint, hi = count;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

constexpr uint64_t kHistMinPerThread = 16;

struct HistParams {
    const uint64_t* keys;
    const uint64_t* d_n;
    uint64_t n_host;
    int lo_bit, hi_bit, passes, stride;  // digit layout (pass_digit), words between passes
    int validate_bits;
    uint32_t* hist;
    uint32_t* status0;                   // first pass's look-back status, cleared here
    uint32_t first_tile, first_radix;    // its tile size and digit count
    uint32_t* err;
    const uint64_t* seg_offsets;
    uint32_t seg_count;
    int seg_shift;
    const uint32_t* gate;
    uint32_t gate_run;
};

__global__ void __launch_bounds__(kSortThreads) radix_histogram(HistParams h) {
    pdl_prologue();
    __shared__ uint32_t s_hist[kSortHistWords];
    if (h.gate && *h.gate != h.gate_run) return;
    const uint64_t n = load_n(h.d_n, h.n_host);
    const int passes = h.passes;
    const int words = passes * h.stride;
    for (int i = threadIdx.x; i < words; i += blockDim.x) s_hist[i] = 0;
    // Clear the first pass's look-back status for this n.
    const uint64_t status_words = (n + h.first_tile - 1) / h.first_tile * h.first_radix;
    const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t gstride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = gtid; i < status_words; i += gstride) h.status0[i] = 0;
    int shift[kMaxPasses];
    uint32_t mask[kMaxPasses];
#pragma unroll
    for (int p = 0; p < kMaxPasses; ++p) {
        int b = 0;
        shift[p] = 0;
        if (p < passes) pass_digit(h.lo_bit, h.hi_bit, passes, p, &shift[p], &b);
        mask[p] = (1u << b) - 1u;
    }
    __syncthreads();
    // Only the CTAs the keys need (at least kHistMinPerThread keys per
    // thread) build histograms: the grid is sized by the bound, and for a
    // small count each CTA's flush of ~1000 bins into the global histogram
    // would cost more than its keys.
    const uint64_t per_cta = (uint64_t)blockDim.x * kHistMinPerThread;
    const uint64_t want = (n + per_cta - 1) / per_cta;
    const uint32_t active = (uint32_t)(want < gridDim.x ? (want > 0 ? want : 1) : gridDim.x);
    if (blockIdx.x >= active) return;
    const uint64_t astride = (uint64_t)active * blockDim.x;

    // Eight independent loads in flight per thread (grid-stride, unrolled):
    // the pass is bound by the bytes in flight. A thread's positions only
    // grow, so its segment (batched input) is found once by binary search and
    // then followed forward.
    constexpr int kHistIlp = 8;
    uint64_t bad = 0;
    uint32_t sg = h.seg_offsets && gtid < n ? segment_search(h.seg_offsets, h.seg_count, gtid) : 0u;
    for (uint64_t i0 = gtid; i0 < n; i0 += kHistIlp * astride) {
        uint64_t k[kHistIlp];
        bool in[kHistIlp];
#pragma unroll
        for (int u = 0; u < kHistIlp; ++u) {
            const uint64_t i = i0 + u * astride;
            in[u] = i < n;
            k[u] = in[u] ? __ldg(h.keys + i) : 0;
        }
#pragma unroll
        for (int u = 0; u < kHistIlp; ++u) {
            if (!in[u]) continue;
            if (h.validate_bits > 0 && h.validate_bits < 64) bad |= k[u] >> h.validate_bits;
            if (h.seg_offsets) {
                sg = segment_advance(h.seg_offsets, h.seg_count, i0 + u * astride, sg);
                k[u] |= (uint64_t)sg << h.seg_shift;
            }
#pragma unroll
            for (int p = 0; p < kMaxPasses; ++p) {
                if (p >= passes) break;
                const uint32_t d = (uint32_t)(k[u] >> shift[p]) & mask[p];
                atomicAdd(&s_hist[p * h.stride + d], 1u);
            }
        }
    }
    if (__any_sync(0xFFFFFFFFu, bad != 0) && (threadIdx.x & 31) == 0) atomicOr(h.err, kErrBadInput);
    __syncthreads();
    for (int i = threadIdx.x; i < words; i += blockDim.x) {
        const uint32_t c = s_hist[i];
        if (c) atomicAdd(h.hist + i, c);
    }
}

struct PassParams {
    const uint64_t* keys_in;
    uint64_t* keys_out;
    const uint32_t* vals_in;  // null -> iota
    uint32_t* vals_out;
    const uint64_t* d_n;
    uint64_t n_host;
    const uint32_t* hist;     // this pass's digit counts (2^bits of them)
    uint32_t* status;         // this pass
    uint32_t* status_clear;   // next pass's status (null for the last pass)
    uint32_t clear_radix;     // digits of the next pass (its tiles are this pass's)
    uint32_t* tile_counter;
    uint32_t* err;
    int shift, bits;
    const uint64_t* seg_offsets;  // first pass of a segmented sort only
    uint32_t seg_count;
    int seg_shift;
    const uint32_t* gate;
    uint32_t gate_run;
    uint32_t spin_limit;      // polls before a look-back wait gives up (kSpinLimit)
    int stall_first_tile;     // test hook: tile 0 never publishes (its successors' waits run out)
};

// Loads / stores kN consecutive shared (or global) words as vectors.
template <int kN>
__device__ __forceinline__ void load_words(const uint32_t* p, uint32_t (&v)[kN]) {
    if constexpr (kN % 4 == 0) {
#pragma unroll
        for (int q = 0; q < kN; q += 4) {
            const uint4 x = *reinterpret_cast<const uint4*>(p + q);
            v[q] = x.x; v[q + 1] = x.y; v[q + 2] = x.z; v[q + 3] = x.w;
        }
    } else if constexpr (kN == 2) {
        const uint2 x = *reinterpret_cast<const uint2*>(p);
        v[0] = x.x; v[1] = x.y;
    } else {
#pragma unroll
        for (int q = 0; q < kN; ++q) v[q] = p[q];
    }
}
template <int kN>
__device__ __forceinline__ void store_words(uint32_t* p, const uint32_t (&v)[kN]) {
    if constexpr (kN % 4 == 0) {
#pragma unroll
        for (int q = 0; q < kN; q += 4) *reinterpret_cast<uint4*>(p + q) = make_uint4(v[q], v[q + 1], v[q + 2], v[q + 3]);
    } else if constexpr (kN == 2) {
        *reinterpret_cast<uint2*>(p) = make_uint2(v[0], v[1]);
    } else {
#pragma unroll
        for (int q = 0; q < kN; ++q) p[q] = v[q];
    }
}
// Relaxed (look-back) loads and stores of kN consecutive status words.
template <int kN>
__device__ __forceinline__ void ld_status(const uint32_t* p, uint32_t (&v)[kN]) {
    if constexpr (kN % 4 == 0) {
#pragma unroll
        for (int q = 0; q < kN; q += 4)
            asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                         : "=r"(v[q]), "=r"(v[q + 1]), "=r"(v[q + 2]), "=r"(v[q + 3])
                         : "l"(p + q)
                         : "memory");
    } else if constexpr (kN == 2) {
        asm volatile("ld.relaxed.gpu.global.v2.u32 {%0, %1}, [%2];" : "=r"(v[0]), "=r"(v[1]) : "l"(p) : "memory");
    } else {
        v[0] = ld_relaxed(p);
    }
}
template <int kN>
__device__ __forceinline__ void st_status(uint32_t* p, const uint32_t (&v)[kN]) {
    if constexpr (kN % 4 == 0) {
#pragma unroll
        for (int q = 0; q < kN; q += 4)
            asm volatile("st.relaxed.gpu.global.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p + q), "r"(v[q]),
                         "r"(v[q + 1]), "r"(v[q + 2]), "r"(v[q + 3])
                         : "memory");
    } else if constexpr (kN == 2) {
        asm volatile("st.relaxed.gpu.global.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(v[0]), "r"(v[1]) : "memory");
    } else {
        st_relaxed(p, v[0]);
    }
}

// Exclusive prefixes of a thread's kDPT consecutive digits (starting at d0)
// over the tiles before `tile`: walks back over their published counts
// several tiles per round trip, each digit stopping at its first inclusive
// prefix; waits (bounded) on tiles that have published nothing yet. All
// digits advance over the same tiles: a round consumes the tiles up to the
// first one some unfinished digit still waits for.
template <int kDPT>
__device__ __forceinline__ void lookback_digits(const uint32_t* status, uint32_t radix, uint32_t tile, uint32_t d0,
                                                uint32_t (&excl)[kDPT], uint32_t* err, uint32_t spin_limit) {
    constexpr int kLB = kDPT >= 4 ? 4 : 16 / kDPT;  // tiles per round trip
    uint32_t done = 0, iter = 0;
    constexpr uint32_t kAll = (1u << kDPT) - 1u;
#pragma unroll
    for (int q = 0; q < kDPT; ++q) excl[q] = 0;
    int64_t t = (int64_t)tile - 1;
    while (done != kAll) {
        uint32_t st[kLB][kDPT];
#pragma unroll
        for (int k = 0; k < kLB; ++k) {
            if (t - k >= 0) {
                ld_status<kDPT>(status + (uint64_t)(t - k) * radix + d0, st[k]);
            } else {
#pragma unroll
                for (int q = 0; q < kDPT; ++q) st[k][q] = kSInc | 1u;  // before the first tile: 0
            }
        }
        // Tiles every unfinished digit can take: up to the first unpublished
        // one before that digit's inclusive prefix.
        int consumed = kLB;
#pragma unroll
        for (int q = 0; q < kDPT; ++q) {
            if (done >> q & 1u) continue;
#pragma unroll
            for (int k = 0; k < kLB; ++k) {
                const uint32_t w = st[k][q];
                if (w >> 31) break;
                if (w == 0) { consumed = min(consumed, k); break; }
            }
        }
#pragma unroll
        for (int q = 0; q < kDPT; ++q) {
            if (done >> q & 1u) continue;
#pragma unroll
            for (int k = 0; k < kLB; ++k) {
                if (k >= consumed) break;
                excl[q] += (st[k][q] & kSVal) - 1u;
                if (st[k][q] >> 31) { done |= 1u << q; break; }
            }
        }
        t -= consumed;
        if (consumed == 0) {
            if (++iter > spin_limit) { atomicOr(err, kErrTimeout); break; }
            backoff(iter);
        }
    }
}

// Shared memory of one onesweep CTA: the staging tile, per-warp digit
// counters (turned into per-warp output offsets) and per-digit offsets.
// Matching by shared-memory atomicOr (kMatch 3) adds, per warp, two sets of
// per-digit lane masks used by alternate rows (zero between uses). They are
// live only while the tile is ranked and the staging tile only after that,
// so the masks share the staging tile's bytes where they fit (cleared at the
// start of every tile) and follow the other arrays otherwise (cleared once).
template <int kBits, int kItems, bool kValues, int kMatch = 0>
struct PassSmem {
    static constexpr int kRadix = 1 << kBits;
    static constexpr int kTile = kPassThreads * kItems;
    static constexpr int kWarpsPerCta = kPassThreads / 32;
    static constexpr bool kOrMatch = kMatch == 3;
    static constexpr int kPeerWords = kWarpsPerCta * 2 * kRadix;
    static constexpr bool kPeerInTile = kOrMatch && kPeerWords * 4 <= kTile * 8;
    union {
        uint64_t keys[kTile];
        uint32_t peer_tile[kPeerInTile ? kPeerWords : 4];
    };
    uint32_t vals[kValues ? kTile : 4];
    uint32_t whist[kWarpsPerCta][kRadix];
    uint32_t gbase[kRadix];
    uint32_t adj[kRadix];
    uint32_t scan[34];
    uint32_t tile_id;
    // Last, so that the arrays above keep their 16-byte alignment (they are
    // read and written as vectors).
    uint32_t peer_own[kOrMatch && !kPeerInTile ? kPeerWords : 1];
    __device__ uint32_t* peer() { return kPeerInTile ? peer_tile : peer_own; }
};

// The vector accesses of whist, gbase and adj need 16-byte alignment.
template <int kBits, int kItems, bool kValues, int kMatch>
constexpr bool pass_smem_aligned() {
    using S = PassSmem<kBits, kItems, kValues, kMatch>;
    return offsetof(S, whist) % 16 == 0 && offsetof(S, gbase) % 16 == 0 && offsetof(S, adj) % 16 == 0;
}

// Ranks one warp's kItems rows of 32 keys stably: per row, the lanes holding
// the same digit are found (match.any on the ADU pipe, one ballot per digit
// bit on the ALU pipe, both alternating, or each lane ORing its bit into its
// digit's word in shared memory and reading the word back), the highest of
// them adds the group's size to the warp's counter for that digit and the
// count before it is broadcast. dr[j] holds the digit in its high half and
// receives the rank (< 2^16) in its low half. kFull: every lane of every row
// is valid. `peer` (kMatch 3): the warp's two sets of kRadix zero words.
template <int kBits, int kItems, int kMatch, bool kFull>
__device__ __forceinline__ void rank_warp(uint32_t (&dr)[kItems], uint32_t* wh, uint32_t wofs, uint32_t tile_n,
                                          uint32_t lane, uint32_t* peer) {
    constexpr uint32_t kRadixW = 1u << kBits;
#pragma unroll
    for (int j = 0; j < kItems; ++j) {
        const bool valid = kFull || wofs + j * 32 + lane < tile_n;
        const uint32_t d = dr[j] >> 16;
        // Every warp collective below is executed by all 32 lanes (valid or
        // not); only the results are masked, never the calls.
        uint32_t peers;
        if (kMatch == 3) {
            // Row j uses word set j & 1; the row before cleared it (its
            // leaders, after the row's second __syncwarp), and the
            // __syncwarp calls of row j - 1 order that clear before this OR.
            uint32_t* pw = peer + (j & 1) * kRadixW;
            const uint32_t vmask = kFull ? 0xFFFFFFFFu : __ballot_sync(0xFFFFFFFFu, valid);
            if (valid) atomicOr(&pw[d], 1u << lane);
            __syncwarp();
            peers = valid ? pw[d] : ~vmask;  // invalid lanes: a group of their own, unused
            __syncwarp();
            if (valid && lane == 31 - __clz(peers)) pw[d] = 0;
        } else if (kMatch == 1 || (kMatch == 2 && (j & 1))) {
            peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 0xFFFFFFFFu);
        } else {
            // Bits above the pass's width are zero in every lane's digit, so
            // their ballots leave `peers` unchanged.
            const uint32_t vmask = kFull ? 0xFFFFFFFFu : __ballot_sync(0xFFFFFFFFu, valid);
            peers = vmask;
#pragma unroll
            for (int b = 0; b < kBits; ++b) {
                const bool bit = (d >> b) & 1u;
                const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
                peers &= bit ? m : ~m;
            }
            if (!kFull && !valid) peers = ~vmask;  // invalid lanes: a group of their own, unused
        }
        const uint32_t upto = __popc(peers & lanemask_le());
        const uint32_t leader = 31 - __clz(peers);
        uint32_t prior = 0;
        if (valid && lane == leader) prior = atomicAdd(&wh[d], upto);
        prior = __shfl_sync(0xFFFFFFFFu, prior, leader);
        dr[j] |= prior + upto - 1;
    }
}

// One digit pass (digits of at most kBits bits). Tiles of kTile keys are
// taken in increasing order from an atomic counter by a persistent grid. Per
// tile:
//   1. each thread loads its keys (warp-striped, coalesced) and keeps only
//      their digits in registers;
//   2. each warp ranks its 32*kItems keys stably (rank_warp) with a
//      warp-private counter per digit;
//   3. each thread sums its kRadix/256 digits over the warps, publishes the
//      tile counts for the decoupled look-back, and a block scan gives the
//      tile-local offsets; the per-warp counters become per-warp output
//      offsets in place;
//   4. keys are fetched again (the tile was just read: cache hits) and staged
//      in digit order in shared memory; values, if any, are fetched here;
//   5. each thread looks back over earlier tiles for its digits' global
//      offsets and publishes the inclusive prefixes (after the staging: the
//      earlier tiles have published their counts by then, so the walk
//      rarely waits);
//   6. the staged tile is written out so that equal digits form contiguous
//      runs.
template <int kBits, int kItems, bool kValues, int kMinCtas, int kMatch>
__global__ void __launch_bounds__(kPassThreads, kMinCtas) onesweep_pass(PassParams p) {
    pdl_prologue();
    using Smem = PassSmem<kBits, kItems, kValues, kMatch>;
    static_assert(pass_smem_aligned<kBits, kItems, kValues, kMatch>(), "vector-accessed arrays misaligned");
    constexpr int kTile = Smem::kTile;
    constexpr int kW = Smem::kWarpsPerCta;
    constexpr int kRadix = Smem::kRadix;
    constexpr int kDPT = kRadix / kPassThreads;  // digits per thread: 1, 2, 4 or 8
    static_assert(kDPT >= 1 && kRadix % kPassThreads == 0, "digits per thread");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t d0 = tid * kDPT;
    if (p.gate && *p.gate != p.gate_run) return;
    const uint64_t n64 = load_n(p.d_n, p.n_host);
    const uint32_t n = (uint32_t)n64;
    const uint32_t ntiles = (uint32_t)((n64 + kTile - 1) / kTile);
    // CTAs beyond the live tile count leave at once (grids are sized by an
    // upper bound when the count is device-resident).
    const uint32_t active = min(gridDim.x, max(ntiles, 1u));
    if (blockIdx.x >= active) return;
    const uint32_t dmask = (1u << p.bits) - 1u;

    if (p.status_clear) {
        const uint64_t words = (uint64_t)ntiles * p.clear_radix;
        for (uint64_t i = (uint64_t)blockIdx.x * kPassThreads + tid; i < words; i += (uint64_t)active * kPassThreads)
            p.status_clear[i] = 0;
    }
    {
        // Global digit starts: exclusive scan of the pass histogram.
        uint32_t h[kDPT], sum = 0, total;
#pragma unroll
        for (int q = 0; q < kDPT; ++q) {
            h[q] = d0 + q < (1u << p.bits) ? p.hist[d0 + q] : 0u;
            sum += h[q];
        }
        uint32_t run = block_exclusive_sum<uint32_t>(sum, S.scan, &total);
#pragma unroll
        for (int q = 0; q < kDPT; ++q) {
            S.gbase[d0 + q] = run;
            run += h[q];
        }
    }
    uint32_t* wh = S.whist[warp];
    if constexpr (Smem::kOrMatch && !Smem::kPeerInTile)
        for (int i = tid; i < Smem::kPeerWords; i += kPassThreads) S.peer_own[i] = 0;
    while (true) {
        if (tid == 0) S.tile_id = atomicAdd(p.tile_counter, 1u);
        {
            const uint4 z = make_uint4(0, 0, 0, 0);
            for (int i = tid; i < kW * kRadix / 4; i += kPassThreads) reinterpret_cast<uint4*>(&S.whist[0][0])[i] = z;
            if constexpr (Smem::kPeerInTile)
                for (int i = tid; i < Smem::kPeerWords / 4; i += kPassThreads) reinterpret_cast<uint4*>(S.peer_tile)[i] = z;
        }
        __syncthreads();
        const uint32_t tile = S.tile_id;
        if (tile >= ntiles) break;
        const uint32_t base = tile * kTile;
        const uint32_t tile_n = min((uint32_t)kTile, n - base);
        const uint32_t wofs = warp * (kItems * 32);

        // 1. Digits of this thread's keys (composite keys on the first pass
        //    of a segmented sort).
        uint32_t dr[kItems];
        {
            uint64_t k[kItems];
#pragma unroll
            for (int j = 0; j < kItems; ++j) {
                const uint32_t i = wofs + j * 32 + lane;
                k[j] = i < tile_n ? __ldg(p.keys_in + base + i) : 0ull;
            }
            if (p.seg_offsets) {
                uint32_t sg = segment_search(p.seg_offsets, p.seg_count, base + wofs + lane);
#pragma unroll
                for (int j = 0; j < kItems; ++j) {
                    const uint32_t i = wofs + j * 32 + lane;
                    if (i < tile_n) {
                        sg = segment_advance(p.seg_offsets, p.seg_count, base + i, sg);
                        k[j] |= (uint64_t)sg << p.seg_shift;
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < kItems; ++j) dr[j] = ((uint32_t)(k[j] >> p.shift) & dmask) << 16;
        }
        // 2. Ranks within the warp.
        uint32_t* peer = Smem::kOrMatch ? S.peer() + warp * 2 * kRadix : nullptr;
        if (tile_n == (uint32_t)kTile) rank_warp<kBits, kItems, kMatch, true>(dr, wh, wofs, tile_n, lane, peer);
        else rank_warp<kBits, kItems, kMatch, false>(dr, wh, wofs, tile_n, lane, peer);
        __syncthreads();

        // 3. This thread's digits: count over the warps, publish the tile
        //    counts, block scan for the tile-local offsets; the per-warp
        //    counters become per-warp output offsets in place.
        uint32_t cnt[kDPT], local[kDPT];
        {
            uint32_t acc[kDPT];
#pragma unroll
            for (int q = 0; q < kDPT; ++q) acc[q] = 0;
#pragma unroll
            for (int w = 0; w < kW; ++w) {
                uint32_t c[kDPT];
                load_words<kDPT>(&S.whist[w][d0], c);
                store_words<kDPT>(&S.whist[w][d0], acc);
#pragma unroll
                for (int q = 0; q < kDPT; ++q) acc[q] += c[q];
            }
            uint32_t pub[kDPT], sum = 0;
#pragma unroll
            for (int q = 0; q < kDPT; ++q) {
                cnt[q] = acc[q];
                pub[q] = (tile == 0 ? kSInc : 0u) | (cnt[q] + 1u);
                sum += cnt[q];
            }
            if (!(p.stall_first_tile && tile == 0)) st_status<kDPT>(p.status + (uint64_t)tile * kRadix + d0, pub);
            uint32_t total;
            uint32_t run = block_exclusive_sum<uint32_t>(sum, S.scan, &total);
#pragma unroll
            for (int q = 0; q < kDPT; ++q) {
                local[q] = run;
                run += cnt[q];
            }
#pragma unroll
            for (int w = 0; w < kW; ++w) {
                uint32_t c[kDPT];
                load_words<kDPT>(&S.whist[w][d0], c);
#pragma unroll
                for (int q = 0; q < kDPT; ++q) c[q] += local[q];
                store_words<kDPT>(&S.whist[w][d0], c);
            }
        }
        __syncthreads();
        // 4. Stage in tile-local digit order: the keys are fetched again
        //    (cache hits), values (if any) here for the first time.
        {
            uint32_t sg = 0;
            if (p.seg_offsets) sg = segment_search(p.seg_offsets, p.seg_count, base + wofs + lane);
#pragma unroll
            for (int j = 0; j < kItems; ++j) {
                const uint32_t i = wofs + j * 32 + lane;
                if (i < tile_n) {
                    uint64_t key = __ldg(p.keys_in + base + i);
                    if (p.seg_offsets) {
                        sg = segment_advance(p.seg_offsets, p.seg_count, base + i, sg);
                        key |= (uint64_t)sg << p.seg_shift;
                    }
                    const uint32_t pos = wh[dr[j] >> 16] + (dr[j] & 0xFFFFu);
                    S.keys[pos] = key;
                    if (kValues) S.vals[pos] = p.vals_in ? p.vals_in[base + i] : base + i;
                }
            }
        }
        // 5. Look back for this thread's digits' offsets among earlier
        //    tiles, publish the inclusive prefixes.
        {
            uint32_t excl[kDPT];
            if (tile > 0) {
                lookback_digits<kDPT>(p.status, kRadix, tile, d0, excl, p.err, p.spin_limit);
                uint32_t pub[kDPT];
#pragma unroll
                for (int q = 0; q < kDPT; ++q) pub[q] = kSInc | (excl[q] + cnt[q] + 1u);
                st_status<kDPT>(p.status + (uint64_t)tile * kRadix + d0, pub);
            } else {
#pragma unroll
                for (int q = 0; q < kDPT; ++q) excl[q] = 0;
            }
            uint32_t adj[kDPT], gb[kDPT];
            load_words<kDPT>(&S.gbase[d0], gb);
#pragma unroll
            for (int q = 0; q < kDPT; ++q) adj[q] = gb[q] + excl[q] - local[q];
            store_words<kDPT>(&S.adj[d0], adj);
        }
        __syncthreads();
        // 6. Write-out.
        bool oob = false;
#pragma unroll 4
        for (uint32_t i = tid; i < tile_n; i += kPassThreads) {
            const uint64_t key = S.keys[i];
            const uint32_t dst = S.adj[(uint32_t)(key >> p.shift) & dmask] + i;
            if (dst < n) {
                p.keys_out[dst] = key;
                if (kValues) p.vals_out[dst] = S.vals[i];
            } else {
                oob = true;  // only after a timed-out wait; never writes out of bounds
            }
        }
        if (oob) atomicOr(p.err, kErrCapacity);
        __syncthreads();
    }
}

__global__ void copy_keys(const uint64_t* in, uint64_t* out, const uint32_t* vin, uint32_t* vout,
                          bool with_values, const uint64_t* d_n, uint64_t n_host, const uint32_t* gate,
                          uint32_t gate_run) {
    pdl_prologue();
    if (gate && *gate != gate_run) return;
    const uint64_t n = load_n(d_n, n_host);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        out[i] = in[i];
        if (with_values) vout[i] = vin ? vin[i] : (uint32_t)i;
    }
}

// Synthetic keys for the autotuner: a SplitMix64 sequence (Steele, Lea and
// Flood, 2014) of the index, placed in bits [lo, hi).
// One-CTA LSD sort of at most kSmallSortMax 64-bit keys on bits [0, 64)
// (eight 8-bit digits), the keys held in shared memory from the first load
// to the last store: for small unique lists, where the grid-wide passes are
// all launch and look-back latency. Each warp owns a contiguous segment of
// the keys; per pass the warps count their segment's digits, the counts
// become per-warp output offsets (digit start over all warps, then the
// earlier warps' counts), and each warp places its segment row by row with
// the digit pass's stable in-warp ranking. Runs when the device count fits,
// and then sets *done, on which the grid-wide sort's kernels return at once.
constexpr int kSmallSortThreads = 1024;
constexpr int kSmallSortWarps = kSmallSortThreads / 32;
constexpr int kSmallSortRows = 4;  // rows of 32 keys per warp and step
struct SmallSortSmem {
    uint64_t keys[2][kSmallSortMax];
    uint32_t whist[kSmallSortWarps][256];
    uint32_t scan[34];
};

__global__ void __launch_bounds__(kSmallSortThreads) small_sort(const uint64_t* in, uint64_t* out, const uint64_t* d_n,
                                                                 uint64_t n_bound, uint32_t* done) {
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SmallSortSmem& S = *reinterpret_cast<SmallSortSmem*>(smem_raw);
    const uint64_t n64 = load_n(d_n, n_bound);
    if (n64 > kSmallSortMax) return;  // the grid-wide sort takes it
    const uint32_t n = (uint32_t)n64;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) *done = 1u;
    for (uint32_t i = tid; i < n; i += kSmallSortThreads) S.keys[0][i] = in[i];
    const uint32_t seg = (n + kSmallSortWarps - 1) / kSmallSortWarps;
    const uint32_t s0 = min(n, warp * seg), len = min(n, s0 + seg) - s0;
    uint32_t* wh = S.whist[warp];
    __syncthreads();
#pragma unroll 1
    for (int p = 0; p < 8; ++p) {
        const uint64_t* src = S.keys[p & 1];
        uint64_t* dst = S.keys[(p & 1) ^ 1];
        const int shift = 8 * p;
        for (int d = lane; d < 256; d += 32) wh[d] = 0;
        __syncwarp();
        for (uint32_t i = lane; i < len; i += 32) atomicAdd(&wh[(uint32_t)(src[s0 + i] >> shift) & 255u], 1u);
        __syncthreads();
        uint32_t tot = 0;
        if (tid < 256)
            for (int w = 0; w < kSmallSortWarps; ++w) tot += S.whist[w][tid];
        uint32_t total;
        const uint32_t start = block_exclusive_sum<uint32_t>(tid < 256 ? tot : 0u, S.scan, &total);
        if (tid < 256) {
            uint32_t run = start;
            for (int w = 0; w < kSmallSortWarps; ++w) {
                const uint32_t c = S.whist[w][tid];
                S.whist[w][tid] = run;
                run += c;
            }
        }
        __syncthreads();
        for (uint32_t b = 0; b < len; b += kSmallSortRows * 32) {
            uint64_t k[kSmallSortRows];
            uint32_t dr[kSmallSortRows];
#pragma unroll
            for (int j = 0; j < kSmallSortRows; ++j) {
                const uint32_t i = b + j * 32 + lane;
                k[j] = i < len ? src[s0 + i] : 0ull;
                dr[j] = ((uint32_t)(k[j] >> shift) & 255u) << 16;
            }
            // Ranks are absolute positions (the counters start at the
            // warp's offsets): below n <= 2^16, as the low half holds them.
            rank_warp<8, kSmallSortRows, 2, false>(dr, wh, b, len, lane, nullptr);
#pragma unroll
            for (int j = 0; j < kSmallSortRows; ++j)
                if (b + j * 32 + lane < len) dst[dr[j] & 0xFFFFu] = k[j];
        }
        __syncthreads();
    }
    for (uint32_t i = tid; i < n; i += kSmallSortThreads) out[i] = S.keys[0][i];
}

__global__ void fill_tune_keys(uint64_t* out, uint64_t n, int lo, int hi, uint64_t seed) {
    const uint64_t mask = hi - lo >= 64 ? ~0ull : ((1ull << (hi - lo)) - 1ull) << lo;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        out[i] = (z << lo) & mask;
    }
}

}  // namespace

void launch_fill_tune_keys(uint64_t* out, uint64_t n, int lo_bit, int hi_bit, uint64_t seed, cudaStream_t s) {
    const uint64_t blocks = (n + 255) / 256;
    fill_tune_keys<<<(unsigned)(blocks < 4096 ? (blocks ? blocks : 1) : 4096), 256, 0, s>>>(out, n, lo_bit, hi_bit, seed);
}

// Keys-only shapes: (items per thread, minimum CTAs per SM, match mode); each
// is built for digits of 8, 9, 10 and 11 bits.
#define DAGC_KEY_SHAPES(X) \
    X(0, 16, 3, 2) X(1, 16, 2, 2) X(2, 16, 4, 2) X(3, 12, 4, 2) X(4, 16, 3, 0) X(5, 16, 3, 1) X(6, 16, 4, 3) X(7, 12, 4, 3) X(8, 24, 3, 3)
// Key/value shapes (8-bit digits).
#define DAGC_PAIR_SHAPES(X) \
    X(0, 16, 2, 0) X(1, 16, 3, 0) X(2, 12, 3, 0) X(3, 8, 4, 0) X(4, 16, 3, 1) X(5, 16, 3, 2) X(6, 16, 2, 2) X(7, 12, 3, 2) \
    X(8, 8, 4, 3) X(9, 16, 3, 3)

namespace {
struct PassKernel {
    void (*fn)(PassParams);
    size_t smem;
};
struct KeyShape {
    int items, min_ctas;
    PassKernel by_bits[kMaxRadixBits - kRadixBits + 1];  // digit widths 8..11
};
struct PairShape {
    int items, min_ctas;
    PassKernel kernel;
};
#define DAGC_KEY_KERNEL(items, ctas, match, bits) \
    {onesweep_pass<bits, items, false, ctas, match>, sizeof(PassSmem<bits, items, false, match>)}
#define DAGC_KEY_SHAPE_ENTRY(id, items, ctas, match)                                                      \
    {items, ctas, {DAGC_KEY_KERNEL(items, ctas, match, 8), DAGC_KEY_KERNEL(items, ctas, match, 9),      \
                   DAGC_KEY_KERNEL(items, ctas, match, 10), DAGC_KEY_KERNEL(items, ctas, match, 11)}},
#define DAGC_PAIR_SHAPE_ENTRY(id, items, ctas, match) \
    {items, ctas, {onesweep_pass<8, items, true, ctas, match>, sizeof(PassSmem<8, items, true, match>)}},
const KeyShape kKeyShapes[kNumKeyShapes] = {DAGC_KEY_SHAPES(DAGC_KEY_SHAPE_ENTRY)};
const PairShape kPairShapes[kNumPairShapes] = {DAGC_PAIR_SHAPES(DAGC_PAIR_SHAPE_ENTRY)};
#undef DAGC_KEY_KERNEL
#undef DAGC_KEY_SHAPE_ENTRY
#undef DAGC_PAIR_SHAPE_ENTRY

int clamp_shape(int shape, bool with_values) {
    const int count = with_values ? kNumPairShapes : kNumKeyShapes;
    return shape < 0 || shape >= count ? 0 : shape;
}
int plan_bits(const SortArgs& a) {
    if (a.with_values || a.radix_bits <= kRadixBits) return kRadixBits;
    return a.radix_bits > kMaxRadixBits ? kMaxRadixBits : a.radix_bits;
}
// The kernel of one pass: the shape's, built for the pass's digit width.
const PassKernel& pass_kernel(int shape, bool with_values, int bits) {
    if (with_values) return kPairShapes[clamp_shape(shape, true)].kernel;
    const int b = bits < kRadixBits ? kRadixBits : (bits > kMaxRadixBits ? kMaxRadixBits : bits);
    return kKeyShapes[clamp_shape(shape, false)].by_bits[b - kRadixBits];
}
uint32_t pass_radix(int bits) { return 1u << (bits < kRadixBits ? kRadixBits : bits); }
}  // namespace

int sort_shape_items(int shape, bool with_values) {
    return with_values ? kPairShapes[clamp_shape(shape, true)].items : kKeyShapes[clamp_shape(shape, false)].items;
}

// Shared memory a CTA may opt in to on sm_103a; kernels needing more (wide
// digits with per-warp match words) are never planned.
constexpr size_t kMaxPassSmem = 227 * 1024;

void sort_configure() {
    cudaFuncSetAttribute(small_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmallSortSmem));
    for (const KeyShape& e : kKeyShapes)
        for (const PassKernel& k : e.by_bits)
            if (k.smem <= kMaxPassSmem) cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
    for (const PairShape& e : kPairShapes)
        if (e.kernel.smem <= kMaxPassSmem)
            cudaFuncSetAttribute(e.kernel.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.kernel.smem);
    cudaGetLastError();  // an attribute the device refuses leaves no error behind for later checks
}

// CTAs of radix_histogram resident per SM: its grid, so that no second wave
// of CTAs with a full grid-stride share runs at a fraction of the occupancy.
int occupancy_sort_histogram() {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, radix_histogram, kSortThreads, 0) != cudaSuccess) {
        cudaGetLastError();
        occ = 0;
    }
    return occ;
}

int occupancy_sort_shape(int shape, bool with_values, int radix_bits) {
    const PassKernel& k = pass_kernel(shape, with_values, with_values ? kRadixBits : radix_bits);
    if (k.smem > kMaxPassSmem) return 0;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k.fn, kPassThreads, k.smem) != cudaSuccess) {
        cudaGetLastError();
        occ = 0;
    }
    return occ;
}

bool sort_plan_valid(int shape, bool with_values, int radix_bits, int lo_bit, int hi_bit) {
    if (with_values && radix_bits > kRadixBits) return false;
    if (radix_bits < kRadixBits || radix_bits > kMaxRadixBits) return false;
    const int passes = sort_passes_r(lo_bit, hi_bit, radix_bits);
    if (passes > kMaxPasses) return false;
    if (pass_kernel(shape, with_values, radix_bits).smem > kMaxPassSmem) return false;
    if (passes && passes * pass_hist_stride(lo_bit, hi_bit, passes) > kSortHistWords) return false;
    // Look-back status room (sort_status_words): at most one digit word per
    // two keys of a tile.
    const int tile = kPassThreads * sort_shape_items(shape, with_values);
    return (int)pass_radix(radix_bits) * 2 <= tile;
}

int sort_plan_passes(const SortArgs& a) { return sort_passes_r(a.lo_bit, a.hi_bit, plan_bits(a)); }

// Launch parameters of digit pass i: the passes ping-pong so that the last
// one always writes keys_out (pass i writes keys_out when passes-1-i is even).
static PassParams pass_params(const SortArgs& a, int i) {
    const int passes = sort_plan_passes(a);
    const bool to_out = ((passes - 1 - i) & 1) == 0;
    PassParams p;
    p.keys_in = i == 0 ? a.keys_in : (to_out ? a.keys_alt : a.keys_out);
    p.keys_out = to_out ? a.keys_out : a.keys_alt;
    p.vals_in = i == 0 ? a.vals_in : (to_out ? a.vals_alt : a.vals_out);
    p.vals_out = to_out ? a.vals_out : a.vals_alt;
    p.d_n = a.d_n;
    p.n_host = a.n;
    p.hist = a.hist + i * pass_hist_stride(a.lo_bit, a.hi_bit, passes);
    p.status = a.status[i & 1];
    p.status_clear = i + 1 < passes ? a.status[(i + 1) & 1] : nullptr;
    pass_digit(a.lo_bit, a.hi_bit, passes, i, &p.shift, &p.bits);
    p.clear_radix = 0;
    if (i + 1 < passes) {
        int sh, b;
        pass_digit(a.lo_bit, a.hi_bit, passes, i + 1, &sh, &b);
        p.clear_radix = pass_radix(b);
    }
    p.tile_counter = a.tile_counters + i;
    p.err = a.err;
    p.seg_offsets = i == 0 ? a.seg_offsets : nullptr;
    p.seg_count = a.seg_count;
    p.seg_shift = a.seg_shift;
    p.gate = a.gate;
    p.gate_run = a.gate_run;
    p.spin_limit = a.spin_limit ? a.spin_limit : kSpinLimit;
    p.stall_first_tile = i == 0 ? a.stall_first_tile : 0;
    return p;
}

void launch_sort_histogram(const SortArgs& a, cudaStream_t s) {
    // The histogram pass also validates the key range, so it runs even when
    // there is no digit to sort.
    const int passes = sort_plan_passes(a);
    HistParams h{};
    h.keys = a.keys_in;
    h.d_n = a.d_n;
    h.n_host = a.n;
    h.lo_bit = a.lo_bit;
    h.hi_bit = a.hi_bit;
    h.passes = passes;
    h.stride = pass_hist_stride(a.lo_bit, a.hi_bit, passes);
    h.validate_bits = a.validate_bits;
    h.hist = a.hist;
    h.status0 = a.status[0];
    h.first_tile = kPassThreads * sort_shape_items(a.shape, a.with_values);
    h.first_radix = 0;
    if (passes) {
        int sh, b;
        pass_digit(a.lo_bit, a.hi_bit, passes, 0, &sh, &b);
        h.first_radix = pass_radix(b);
    }
    h.err = a.err;
    h.seg_offsets = a.seg_offsets;
    h.seg_count = a.seg_count;
    h.seg_shift = a.seg_shift;
    h.gate = a.gate;
    h.gate_run = a.gate_run;
    launch_pdl(radix_histogram, dim3(a.grid_hist), dim3(kSortThreads), 0, s, h);
    if (passes == 0)
        launch_pdl(copy_keys, dim3(a.grid_hist), dim3(256), 0, s, a.keys_in, a.keys_out, a.vals_in, a.vals_out,
                   a.with_values, a.d_n, a.n, a.gate, a.gate_run);
}

void launch_sort_pass(const SortArgs& a, int i, cudaStream_t s) {
    const PassParams p = pass_params(a, i);
    const PassKernel& k = pass_kernel(a.shape, a.with_values, p.bits);
    void* args[] = {const_cast<PassParams*>(&p)};
    launch_pdl_c((const void*)k.fn, dim3(a.grid_pass), dim3(kPassThreads), args, k.smem, s);
}

void launch_small_sort(const uint64_t* keys_in, uint64_t* keys_out, const uint64_t* d_n, uint64_t n_bound,
                       uint32_t* done, cudaStream_t s) {
    launch_pdl(small_sort, dim3(1), dim3(kSmallSortThreads), sizeof(SmallSortSmem), s, keys_in, keys_out, d_n, n_bound,
               done);
}

void launch_sort(const SortArgs& a, cudaStream_t s) {
    launch_sort_histogram(a, s);
    for (int i = 0; i < sort_plan_passes(a); ++i) launch_sort_pass(a, i, s);
}

}  // namespace dagc
