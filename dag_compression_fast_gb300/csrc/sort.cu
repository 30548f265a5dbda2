// Stable LSD radix sort of uint64 keys (optionally with uint32 values) on a
// bit range, for sm_103a. Replaces cub::DeviceRadixSort::SortKeys/SortPairs
// (src/DAGCompression.cu:336-394) and thrust::sequence (:743-750).
//
// Structure (one-sweep style):
//   1. radix_histogram: one read of the keys builds the 256-bin histogram of
//      every digit pass at once (shared-memory counters, then global atomics),
//      validates the key range and clears the first pass's look-back status.
//   2. onesweep_pass, once per 8-bit digit: a persistent grid takes 4096-key
//      tiles in order from an atomic counter, ranks keys inside each warp with
//      __match_any_sync, publishes per-digit tile counts, finds the tile's
//      global digit offsets by decoupled look-back (bounded waits), stages the
//      tile in shared memory in digit order and writes it out so that equal
//      digits land in contiguous runs.
// All counts can be device-resident (d_n), so a whole pipeline runs without a
// host round trip.

#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

#include <algorithm>

namespace dagc {
namespace {

constexpr uint32_t kSAgg = 1u << 30;
constexpr uint32_t kSInc = 2u << 30;
constexpr uint32_t kSVal = (1u << 30) - 1;
constexpr int kRadix = 1 << kRadixBits;

constexpr int kPassThreads = 256;  // one thread per digit

// A device-resident count never exceeds the bound its buffers were sized for.
__device__ __forceinline__ uint64_t load_n(const uint64_t* d_n, uint64_t n) {
    if (!d_n) return n;
    const uint64_t v = *d_n;
    return v < n ? v : n;
}

// Segment of position i (seg_offsets ascending, count + 1 entries): binary
// search for the first position of a block, then `segment_from` walks forward.
__device__ __forceinline__ uint32_t segment_search(const uint64_t* off, uint32_t count, uint64_t i) {
    uint32_t lo = 0, hi = count;  // invariant: off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}
__device__ __forceinline__ uint32_t segment_from(const uint64_t* off, uint32_t count, uint64_t i, uint32_t hint) {
    while (hint + 1 < count && __ldg(off + hint + 1) <= i) ++hint;
    return hint;
}

constexpr uint64_t kHistMinPerThread = 16;

__global__ void __launch_bounds__(kSortThreads)
radix_histogram(const uint64_t* __restrict__ keys, const uint64_t* d_n, uint64_t n_host, int lo_bit,
                int hi_bit, int validate_bits, uint32_t* __restrict__ hist, uint32_t* status0,
                uint32_t* err, const uint64_t* seg_offsets, uint32_t seg_count, int seg_shift,
                const uint32_t* gate, uint32_t gate_run) {
    pdl_prologue();
    __shared__ uint32_t s_hist[kMaxPasses][kRadix];
    if (gate && *gate != gate_run) return;
    const uint64_t n = load_n(d_n, n_host);
    const int passes = sort_passes(lo_bit, hi_bit);
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) (&s_hist[0][0])[i] = 0;
    // Clear the first pass's look-back status for this n.
    const uint64_t status_words = (uint64_t)sort_tiles(n) * kRadix;
    const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t gstride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = gtid; i < status_words; i += gstride) status0[i] = 0;
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

    // Four independent loads in flight per thread (grid-stride, unrolled).
    uint64_t bad = 0;
    for (uint64_t i0 = gtid; i0 < n; i0 += 4 * astride) {
        uint64_t k[4];
        bool in[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint64_t i = i0 + u * astride;
            in[u] = i < n;
            k[u] = in[u] ? __ldg(keys + i) : 0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (!in[u]) continue;
            if (validate_bits > 0 && validate_bits < 64) bad |= k[u] >> validate_bits;
            if (seg_offsets)
                k[u] |= (uint64_t)segment_search(seg_offsets, seg_count, i0 + u * astride) << seg_shift;
            for (int p = 0; p < passes; ++p) {
                const int shift = lo_bit + p * kRadixBits;
                const int bits = min(kRadixBits, hi_bit - shift);
                const uint32_t d = (uint32_t)(k[u] >> shift) & ((1u << bits) - 1u);
                atomicAdd(&s_hist[p][d], 1u);
            }
        }
    }
    if (__any_sync(0xFFFFFFFFu, bad != 0) && (threadIdx.x & 31) == 0) atomicOr(err, kErrBadInput);
    __syncthreads();
    for (int i = threadIdx.x; i < passes * kRadix; i += blockDim.x) {
        const uint32_t c = (&s_hist[0][0])[i];
        if (c) atomicAdd(hist + i, c);
    }
}

struct PassParams {
    const uint64_t* keys_in;
    uint64_t* keys_out;
    const uint32_t* vals_in;  // null -> iota
    uint32_t* vals_out;
    const uint64_t* d_n;
    uint64_t n_host;
    const uint32_t* hist;     // 256 digit counts of this pass
    uint32_t* status;         // this pass
    uint32_t* status_clear;   // next pass's status (null for the last pass)
    uint32_t* tile_counter;
    uint32_t* err;
    int shift, bits;
    const uint64_t* seg_offsets;  // first pass of a segmented sort only
    uint32_t seg_count;
    int seg_shift;
    const uint32_t* gate;
    uint32_t gate_run;
};

// Exclusive prefix of one digit over the tiles before `tile`: walks back over
// their published counts 16 tiles per round trip, stopping at the first
// inclusive prefix; waits (bounded) on tiles that have published nothing yet.
// (When every tile of a small sort runs at once, inclusive prefixes spread
// about one window per round trip, so the window width sets the latency.)
__device__ __forceinline__ uint32_t lookback_digit(const uint32_t* status, uint32_t tile, uint32_t d,
                                                   uint32_t* err) {
    constexpr int kLB = 16;
    uint32_t excl = 0, iter = 0;
    int64_t t = (int64_t)tile - 1;
    while (true) {
        uint32_t st[kLB];
#pragma unroll
        for (int k = 0; k < kLB; ++k)
            st[k] = t - k >= 0 ? ld_relaxed(status + (uint64_t)(t - k) * kRadix + d) : kSInc;
        int consumed = kLB;
        bool done = false;
#pragma unroll
        for (int k = 0; k < kLB; ++k) {
            if (done || k >= consumed) continue;
            const uint32_t f = st[k] >> 30;
            if (f == 0) {
                consumed = k;  // not published yet: resume here
            } else {
                excl += st[k] & kSVal;
                done = f == 2;
            }
        }
        if (done) break;
        t -= consumed;
        if (consumed == 0) {
            if (++iter > kSpinLimit) { atomicOr(err, kErrTimeout); break; }
            backoff(iter);
        }
    }
    return excl;
}

// Shared memory of one onesweep CTA: the staging tile, per-warp digit
// counters (turned into per-warp output offsets) and per-digit offsets.
template <int kThreads, int kItems, bool kValues>
struct PassSmem {
    static constexpr int kTile = kThreads * kItems;
    static constexpr int kWarpsPerCta = kThreads / 32;
    uint64_t keys[kTile];
    uint32_t vals[kValues ? kTile : 4];
    uint32_t whist[kWarpsPerCta][kRadix];
    uint32_t gbase[kRadix];
    uint32_t adj[kRadix];
    uint32_t scan[34];
    uint32_t tile_id;
};

// One 8-bit digit pass. Tiles of kTile keys are taken in increasing order from
// an atomic counter by a persistent grid. Per tile:
//   1. each thread loads its keys straight into registers (warp-striped,
//      coalesced), so shared memory only carries the counters and the
//      staged output;
//   2. each warp ranks its 32*kItems keys stably with __match_any_sync and a
//      warp-private counter per digit;
//   3. thread d sums digit d over the warps, publishes the tile count for the
//      decoupled look-back, and a block scan gives the tile-local offsets;
//      the per-warp counters become per-warp output offsets in place;
//   4. thread d looks back over earlier tiles (8 per round trip, bounded
//      waits) for digit d's global offset and publishes the inclusive prefix;
//   5. keys are staged in digit order and written out so that equal digits
//      form contiguous runs.
// kMatch: how lanes with equal digits are found. 0: one ballot per digit bit
// (ALU pipe), 1: match.any (ADU pipe), 2: alternate per item, which spreads
// the work over both pipes.
template <int kThreads, int kItems, bool kValues, int kMinCtas, int kMatch>
__global__ void __launch_bounds__(kThreads, kMinCtas) onesweep_pass(PassParams p) {
    pdl_prologue();
    using Smem = PassSmem<kThreads, kItems, kValues>;
    constexpr int kTile = Smem::kTile;
    constexpr int kW = Smem::kWarpsPerCta;
    static_assert(kThreads == kRadix, "one thread per digit");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
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
        const uint64_t words = (uint64_t)ntiles * kRadix;
        for (uint64_t i = (uint64_t)blockIdx.x * kThreads + tid; i < words; i += (uint64_t)active * kThreads)
            p.status_clear[i] = 0;
    }
    {
        uint32_t total;
        S.gbase[tid] = block_exclusive_sum<uint32_t>(p.hist[tid], S.scan, &total);
    }
    uint32_t* wh = S.whist[warp];
    while (true) {
        if (tid == 0) S.tile_id = atomicAdd(p.tile_counter, 1u);
        for (int i = tid; i < kW * kRadix; i += kThreads) (&S.whist[0][0])[i] = 0;
        __syncthreads();
        const uint32_t tile = S.tile_id;
        if (tile >= ntiles) break;
        const uint32_t base = tile * kTile;
        const uint32_t tile_n = min((uint32_t)kTile, n - base);
        const uint32_t wofs = warp * (kItems * 32);

        uint64_t k[kItems];
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            const uint32_t i = wofs + j * 32 + lane;
            if (i < tile_n) k[j] = p.keys_in[base + i];
        }
        if (p.seg_offsets) {  // first pass of a segmented sort: build composite keys
            uint32_t sg = segment_search(p.seg_offsets, p.seg_count, base + wofs + lane);
#pragma unroll
            for (int j = 0; j < kItems; ++j) {
                const uint32_t i = wofs + j * 32 + lane;
                if (i < tile_n) {
                    sg = segment_from(p.seg_offsets, p.seg_count, base + i, sg);
                    k[j] |= (uint64_t)sg << p.seg_shift;
                }
            }
        }
        // Ranks within the warp fit 16 bits: two per register.
        uint32_t rank2[kItems / 2];
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            const bool valid = wofs + j * 32 + lane < tile_n;
            const uint32_t d = (uint32_t)(k[j] >> p.shift) & dmask;
            // Lanes holding the same digit. Every warp collective below is
            // executed by all 32 lanes (valid or not); only the results are
            // masked, never the calls.
            uint32_t peers;
            if (kMatch == 1 || (kMatch == 2 && (j & 1))) {
                peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 0xFFFFFFFFu);
            } else {
                // One ballot per digit bit; bits above p.bits are zero in every
                // lane's digit, so their ballot leaves `peers` unchanged.
                const uint32_t vmask = __ballot_sync(0xFFFFFFFFu, valid);
                peers = vmask;
#pragma unroll
                for (int b = 0; b < kRadixBits; ++b) {
                    const bool bit = (d >> b) & 1u;
                    const uint32_t m = __ballot_sync(0xFFFFFFFFu, bit);
                    peers &= bit ? m : ~m;
                }
                if (!valid) peers = ~vmask;  // invalid lanes: a group of their own, unused
            }
            // The highest peer adds the group's size to the warp's digit
            // counter and broadcasts the count before it.
            const uint32_t upto = __popc(peers & lanemask_le());
            const uint32_t leader = 31 - __clz(peers);
            uint32_t prior = 0;
            if (valid && lane == leader) prior = atomicAdd(&wh[d], upto);
            prior = __shfl_sync(0xFFFFFFFFu, prior, leader);
            const uint32_t r = prior + upto - 1;
            if (j & 1) rank2[j / 2] |= r << 16;
            else rank2[j / 2] = r;
        }
        __syncthreads();

        // Digit d = tid: count over the warps, publish the tile count, block
        // scan for the tile-local offsets; the per-warp counters become
        // per-warp output offsets in place.
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < kW; ++w) {
            const uint32_t c = S.whist[w][tid];
            S.whist[w][tid] = cnt;
            cnt += c;
        }
        uint32_t* my = p.status + (uint64_t)tile * kRadix + tid;
        st_relaxed(my, (tile == 0 ? kSInc : kSAgg) | cnt);
        uint32_t total;
        const uint32_t local = block_exclusive_sum<uint32_t>(cnt, S.scan, &total);
#pragma unroll
        for (int w = 0; w < kW; ++w) S.whist[w][tid] += local;
        __syncthreads();
        // Stage in tile-local digit order; values (if any) are fetched here,
        // they play no part in the ranking.
#pragma unroll
        for (int j = 0; j < kItems; ++j) {
            const uint32_t i = wofs + j * 32 + lane;
            if (i < tile_n) {
                const uint32_t r = (rank2[j / 2] >> ((j & 1) * 16)) & 0xFFFFu;
                const uint32_t pos = wh[(uint32_t)(k[j] >> p.shift) & dmask] + r;
                S.keys[pos] = k[j];
                if (kValues) S.vals[pos] = p.vals_in ? p.vals_in[base + i] : base + i;
            }
        }
        // Look back for digit d's offset among earlier tiles, publish the
        // inclusive prefix.
        uint32_t excl = 0;
        if (tile > 0) {
            excl = lookback_digit(p.status, tile, tid, p.err);
            st_relaxed(my, kSInc | (excl + cnt));
        }
        S.adj[tid] = S.gbase[tid] + excl - local;
        __syncthreads();
        bool oob = false;
#pragma unroll 4
        for (uint32_t i = tid; i < tile_n; i += kThreads) {
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

}  // namespace

// Shape table: (items per thread, minimum CTAs per SM, match mode).
#define DAGC_SORT_SHAPES(X) \
    X(0, 16, 2, 0) X(1, 16, 3, 0) X(2, 12, 3, 0) X(3, 8, 4, 0) X(4, 16, 3, 1) X(5, 16, 3, 2) X(6, 16, 2, 2) X(7, 12, 3, 2)

namespace {
struct ShapeEntry {
    int items, min_ctas;
    void (*keys)(PassParams);
    void (*pairs)(PassParams);
    size_t smem_keys, smem_pairs;
};
#define DAGC_SHAPE_ENTRY(id, items, ctas, match)                                                     \
    {items, ctas, onesweep_pass<kPassThreads, items, false, ctas, match>,                             \
     onesweep_pass<kPassThreads, items, true, ctas, match>, sizeof(PassSmem<kPassThreads, items, false>), \
     sizeof(PassSmem<kPassThreads, items, true>)},
const ShapeEntry kShapes[kNumSortShapes] = {DAGC_SORT_SHAPES(DAGC_SHAPE_ENTRY)};
#undef DAGC_SHAPE_ENTRY
}  // namespace

int sort_shape_items(int shape) { return kShapes[shape].items; }
int sort_shape_min_ctas(int shape) { return kShapes[shape].min_ctas; }

size_t sort_pass_smem(bool with_values) {
    size_t m = 0;
    for (const ShapeEntry& e : kShapes) m = std::max(m, with_values ? e.smem_pairs : e.smem_keys);
    return m;
}

void sort_configure() {
    for (const ShapeEntry& e : kShapes) {
        cudaFuncSetAttribute(e.keys, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem_keys);
        cudaFuncSetAttribute(e.pairs, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e.smem_pairs);
    }
}

int occupancy_sort_shape(int shape, bool with_values) {
    const ShapeEntry& e = kShapes[shape];
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, with_values ? e.pairs : e.keys, kPassThreads,
                                                  with_values ? e.smem_pairs : e.smem_keys);
    return occ;
}

int occupancy_sort_pass(bool with_values) { return occupancy_sort_shape(1, with_values); }

// Launch parameters of digit pass i: the passes ping-pong so that the last
// one always writes keys_out (pass i writes keys_out when passes-1-i is even).
static PassParams pass_params(const SortArgs& a, int i) {
    const int passes = sort_passes(a.lo_bit, a.hi_bit);
    const bool to_out = ((passes - 1 - i) & 1) == 0;
    PassParams p;
    p.keys_in = i == 0 ? a.keys_in : (to_out ? a.keys_alt : a.keys_out);
    p.keys_out = to_out ? a.keys_out : a.keys_alt;
    p.vals_in = i == 0 ? a.vals_in : (to_out ? a.vals_alt : a.vals_out);
    p.vals_out = to_out ? a.vals_out : a.vals_alt;
    p.d_n = a.d_n;
    p.n_host = a.n;
    p.hist = a.hist + i * 256;
    p.status = a.status[i & 1];
    p.status_clear = i + 1 < passes ? a.status[(i + 1) & 1] : nullptr;
    p.tile_counter = a.tile_counters + i;
    p.err = a.err;
    p.shift = a.lo_bit + i * kRadixBits;
    p.bits = a.hi_bit - p.shift < kRadixBits ? a.hi_bit - p.shift : kRadixBits;
    p.seg_offsets = i == 0 ? a.seg_offsets : nullptr;
    p.seg_count = a.seg_count;
    p.seg_shift = a.seg_shift;
    p.gate = a.gate;
    p.gate_run = a.gate_run;
    return p;
}

void launch_sort_histogram(const SortArgs& a, cudaStream_t s) {
    // The histogram pass also validates the key range, so it runs even when
    // there is no digit to sort.
    launch_pdl(radix_histogram, dim3(a.grid_hist), dim3(kSortThreads), 0, s, a.keys_in, a.d_n, a.n, a.lo_bit, a.hi_bit,
                                                         a.validate_bits, a.hist, a.status[0], a.err,
                                                         a.seg_offsets, a.seg_count, a.seg_shift, a.gate,
                                                         a.gate_run);
    if (sort_passes(a.lo_bit, a.hi_bit) == 0)
        launch_pdl(copy_keys, dim3(a.grid_hist), dim3(256), 0, s, a.keys_in, a.keys_out, a.vals_in, a.vals_out, a.with_values,
                                              a.d_n, a.n, a.gate, a.gate_run);
}

void launch_sort_pass(const SortArgs& a, int i, cudaStream_t s) {
    const PassParams p = pass_params(a, i);
    const ShapeEntry& e = kShapes[a.shape < 0 || a.shape >= kNumSortShapes ? 1 : a.shape];
    void* args[] = {const_cast<PassParams*>(&p)};
    launch_pdl_c(a.with_values ? (const void*)e.pairs : (const void*)e.keys, dim3(a.grid_pass), dim3(kPassThreads),
                 args, a.with_values ? e.smem_pairs : e.smem_keys, s);
}

void launch_sort(const SortArgs& a, cudaStream_t s) {
    launch_sort_histogram(a, s);
    for (int i = 0; i < sort_passes(a.lo_bit, a.hi_bit); ++i) launch_sort_pass(a, i, s);
}

}  // namespace dagc
