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

namespace dagc {
namespace {

constexpr uint32_t kSAgg = 1u << 30;
constexpr uint32_t kSInc = 2u << 30;
constexpr uint32_t kSVal = (1u << 30) - 1;
constexpr int kWarps = kSortThreads / 32;
constexpr int kRadix = 1 << kRadixBits;
static_assert(kSortThreads == kRadix, "one thread per digit");

__device__ __forceinline__ uint64_t load_n(const uint64_t* d_n, uint64_t n) {
    return d_n ? *d_n : n;
}

__global__ void __launch_bounds__(kSortThreads)
radix_histogram(const uint64_t* __restrict__ keys, const uint64_t* d_n, uint64_t n_host, int lo_bit,
                int hi_bit, int validate_bits, uint32_t* __restrict__ hist, uint32_t* status0,
                uint32_t* err) {
    __shared__ uint32_t s_hist[kMaxPasses][kRadix];
    const uint64_t n = load_n(d_n, n_host);
    const int passes = sort_passes(lo_bit, hi_bit);
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += blockDim.x) (&s_hist[0][0])[i] = 0;
    // Clear the first pass's look-back status for this n.
    const uint64_t status_words = (uint64_t)sort_tiles(n) * kRadix;
    const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t gstride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = gtid; i < status_words; i += gstride) status0[i] = 0;
    __syncthreads();

    uint64_t bad = 0;
    for (uint64_t i = gtid; i < n; i += gstride) {
        const uint64_t k = __ldg(keys + i);
        if (validate_bits > 0 && validate_bits < 64) bad |= k >> validate_bits;
        for (int p = 0; p < passes; ++p) {
            const int shift = lo_bit + p * kRadixBits;
            const int bits = min(kRadixBits, hi_bit - shift);
            const uint32_t d = (uint32_t)(k >> shift) & ((1u << bits) - 1u);
            atomicAdd(&s_hist[p][d], 1u);
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
};

template <bool kValues>
__global__ void __launch_bounds__(kSortThreads, 2) onesweep_pass(PassParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(smem);                        // kSortTile
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + kSortTile);          // kSortTile if kValues
    uint32_t* s_whist = s_vals + (kValues ? kSortTile : 0);                      // kWarps * 256
    uint32_t* s_gbase = s_whist + kWarps * kRadix;                               // 256
    uint32_t* s_adj = s_gbase + kRadix;                                          // 256
    uint32_t* s_local = s_adj + kRadix;                                          // 256
    uint32_t* s_scan = s_local + kRadix;                                         // 33
    uint32_t* s_tile = s_scan + 33;                                              // 1

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t n64 = load_n(p.d_n, p.n_host);
    const uint32_t n = (uint32_t)n64;
    const uint32_t ntiles = sort_tiles(n64);
    const uint32_t dmask = (1u << p.bits) - 1u;

    if (p.status_clear) {
        const uint64_t words = (uint64_t)ntiles * kRadix;
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + tid; i < words; i += (uint64_t)gridDim.x * blockDim.x)
            p.status_clear[i] = 0;
    }
    {
        uint32_t total;
        const uint32_t c = p.hist[tid];
        s_gbase[tid] = block_exclusive_sum<uint32_t>(c, s_scan, &total);
    }

    while (true) {
        if (tid == 0) *s_tile = atomicAdd(p.tile_counter, 1u);
        for (int i = tid; i < kWarps * kRadix; i += kSortThreads) s_whist[i] = 0;
        __syncthreads();
        const uint32_t tile = *s_tile;
        if (tile >= ntiles) break;
        const uint32_t base = tile * kSortTile;
        const uint32_t tile_n = min((uint32_t)kSortTile, n - base);
        const uint32_t wbase = base + warp * (kSortItems * 32);

        uint64_t k[kSortItems];
        uint32_t v[kValues ? kSortItems : 1];
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            const uint32_t idx = wbase + j * 32 + lane;
            if (idx < n) {
                k[j] = p.keys_in[idx];
                if (kValues) v[j] = p.vals_in ? p.vals_in[idx] : idx;
            }
        }
        // Warp-level multisplit ranking (stable: item order = (j, lane)).
        uint32_t rank[kSortItems];
        uint32_t* wh = s_whist + warp * kRadix;
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            const bool valid = wbase + j * 32 + lane < n;
            const uint32_t d = valid ? ((uint32_t)(k[j] >> p.shift) & dmask) : 0xFFFFFFFFu;
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
            uint32_t prior = 0;
            if (valid) {
                prior = wh[d];
                rank[j] = prior + __popc(peers & lanemask_lt());
            }
            __syncwarp();
            if (valid && lane == (uint32_t)(__ffs(peers) - 1)) wh[d] = prior + __popc(peers);
            __syncwarp();
        }
        __syncthreads();

        // Per digit (thread tid = digit): exclusive over warps, tile count,
        // publish, local offset, look-back.
        {
            const uint32_t d = tid;
            uint32_t cnt = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = s_whist[w * kRadix + d];
                s_whist[w * kRadix + d] = cnt;
                cnt += c;
            }
            uint32_t* st = p.status + (uint64_t)tile * kRadix + d;
            st_relaxed(st, (tile == 0 ? kSInc : kSAgg) | cnt);
            uint32_t total;
            const uint32_t local = block_exclusive_sum<uint32_t>(cnt, s_scan, &total);
            uint32_t excl = 0;
            if (tile > 0) {
                int64_t t = (int64_t)tile - 1;
                uint32_t iter = 0;
                while (t >= 0) {
                    const uint32_t s = ld_relaxed(p.status + (uint64_t)t * kRadix + d);
                    const uint32_t flag = s >> 30;
                    if (flag == 0) {
                        if (++iter > kSpinLimit) { atomicOr(p.err, kErrTimeout); break; }
                        backoff(iter);
                        continue;
                    }
                    excl += s & kSVal;
                    if (flag == 2) break;
                    --t;
                }
                st_relaxed(st, kSInc | (excl + cnt));
            }
            s_local[d] = local;
            s_adj[d] = s_gbase[d] + excl - local;
        }
        __syncthreads();

        // Stage in local digit order.
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            if (wbase + j * 32 + lane < n) {
                const uint32_t d = (uint32_t)(k[j] >> p.shift) & dmask;
                const uint32_t pos = s_local[d] + s_whist[warp * kRadix + d] + rank[j];
                s_keys[pos] = k[j];
                if (kValues) s_vals[pos] = v[j];
            }
        }
        __syncthreads();
        for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
            const uint64_t key = s_keys[i];
            const uint32_t d = (uint32_t)(key >> p.shift) & dmask;
            const uint32_t dst = s_adj[d] + i;
            p.keys_out[dst] = key;
            if (kValues) p.vals_out[dst] = s_vals[i];
        }
        __syncthreads();
    }
}

__global__ void copy_keys(const uint64_t* in, uint64_t* out, const uint32_t* vin, uint32_t* vout,
                          bool with_values, const uint64_t* d_n, uint64_t n_host) {
    const uint64_t n = load_n(d_n, n_host);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        out[i] = in[i];
        if (with_values) vout[i] = vin ? vin[i] : (uint32_t)i;
    }
}

}  // namespace

size_t sort_pass_smem(bool with_values) {
    return (size_t)kSortTile * 8 + (with_values ? (size_t)kSortTile * 4 : 0) +
           (size_t)(kWarps * kRadix + 3 * kRadix + 34) * 4;
}

void sort_configure() {
    cudaFuncSetAttribute(onesweep_pass<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sort_pass_smem(true));
    cudaFuncSetAttribute(onesweep_pass<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)sort_pass_smem(false));
}

int occupancy_sort_pass(bool with_values) {
    int occ = 0;
    if (with_values)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, onesweep_pass<true>, kSortThreads, sort_pass_smem(true));
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, onesweep_pass<false>, kSortThreads, sort_pass_smem(false));
    return occ;
}

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
    return p;
}

void launch_sort_histogram(const SortArgs& a, cudaStream_t s) {
    // The histogram pass also validates the key range, so it runs even when
    // there is no digit to sort.
    radix_histogram<<<a.grid_hist, kSortThreads, 0, s>>>(a.keys_in, a.d_n, a.n, a.lo_bit, a.hi_bit,
                                                         a.validate_bits, a.hist, a.status[0], a.err);
    if (sort_passes(a.lo_bit, a.hi_bit) == 0)
        copy_keys<<<a.grid_hist, 256, 0, s>>>(a.keys_in, a.keys_out, a.vals_in, a.vals_out, a.with_values,
                                              a.d_n, a.n);
}

void launch_sort_pass(const SortArgs& a, int i, cudaStream_t s) {
    const PassParams p = pass_params(a, i);
    if (a.with_values)
        onesweep_pass<true><<<a.grid_pass, kSortThreads, sort_pass_smem(true), s>>>(p);
    else
        onesweep_pass<false><<<a.grid_pass, kSortThreads, sort_pass_smem(false), s>>>(p);
}

void launch_sort(const SortArgs& a, cudaStream_t s) {
    launch_sort_histogram(a, s);
    for (int i = 0; i < sort_passes(a.lo_bit, a.hi_bit); ++i) launch_sort_pass(a, i, s);
}

}  // namespace dagc
