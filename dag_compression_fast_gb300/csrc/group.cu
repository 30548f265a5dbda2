// Fragment grouping by hash, for sm_103a: an alternative to the fragment sort
// + leaf build (src/DAGCompression.cu:1026-1068: SortKeys, SelectUnique,
// ReduceByKey) for inputs where many fragments share a brick. Both produce
// the same arrays: the distinct bricks (code >> 6) in ascending order and,
// per brick, the OR of 1 << (code & 63) over its fragments.
//
//   group_sketch  one read of the fragments: range check and a HyperLogLog
//                 sketch (4096 registers) of the distinct bricks;
//   group_insert  estimates the distinct bricks B from the sketch and picks
//                 the path: grouping when the fragments hold at least
//                 kGroupMinRedundancy per brick and a table of ~2.5 B slots
//                 fits, else the sort path (every kernel of the other path
//                 reads the decision and does nothing). Grouping: each
//                 fragment finds or claims its brick's slot (linear probing,
//                 atomicCAS) and ORs its bit into the slot's mask;
//   group_collect the occupied slots become the brick list (brick, slot);
//   (then the brick list is sorted by brick with the radix sort, values =
//    slots: B items instead of N)
//   group_gather  leaf masks read from the slots in sorted brick order,
//                 parents written, slots cleared.
//
// The table holds kGroupMaxSlots keys (brick + 1) and, beside them,
// kGroupMaxSlots masks; zero on entry, and left zero by the gather (each used
// slot once). (Reading key and mask together, to skip the OR of a bit already
// set, measured slower: the reads, not the fire-and-forget ORs, bound it.)

#include "dagc_device.cuh"
#include "dagc_kernels.h"

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

__device__ __forceinline__ uint32_t segment_of(const uint64_t* off, uint32_t count, uint64_t i) {
    uint32_t lo = 0, hi = count;  // off[lo] <= i < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(off + mid) <= i) lo = mid; else hi = mid;
    }
    return lo;
}

// Brick key of fragment i: code >> 6, or for batched input the composite
// ((segment << seg_shift) | local) >> 6. `bad` flags codes out of range.
__device__ __forceinline__ uint64_t brick_of(const GroupArgs& a, uint64_t i, uint64_t code, bool* bad) {
    if (a.validate_bits > 0 && a.validate_bits < 64 && (code >> a.validate_bits)) *bad = true;
    if (a.seg_offsets) code |= (uint64_t)segment_of(a.seg_offsets, a.seg_count, i) << a.seg_shift;
    return code >> 6;
}

constexpr int kSketchLog = 12;
constexpr int kSketchRegs = 1 << kSketchLog;

__global__ void __launch_bounds__(256) group_sketch(GroupArgs a) {
    __shared__ uint32_t reg[kSketchRegs];
    for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x) reg[i] = 0;
    __syncthreads();
    bool bad = false;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < a.n; i0 += 4 * stride) {
        uint64_t c[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) c[u] = i0 + u * stride < a.n ? __ldg(a.frags + i0 + u * stride) : 0;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (i0 + u * stride >= a.n) continue;
            const uint64_t h = fmix(brick_of(a, i0 + u * stride, c[u], &bad) ^ 0x9E3779B97F4A7C15ull);
            const uint32_t idx = (uint32_t)(h >> (64 - kSketchLog));
            const uint32_t rank = (uint32_t)__clzll((h << kSketchLog) | (1ull << (kSketchLog - 1))) + 1;
            atomicMax(&reg[idx], rank);
        }
    }
    if (__any_sync(0xFFFFFFFFu, bad) && (threadIdx.x & 31) == 0) atomicOr(a.err, kErrBadInput);
    __syncthreads();
    for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x)
        if (reg[i]) atomicMax(a.sketch + i, reg[i]);
}

constexpr int kIlp = 4;


// Distinct-brick estimate from the sketch (HyperLogLog with the linear
// counting correction for small counts); the whole CTA takes part.
__device__ double sketch_estimate(const uint32_t* sketch, double* red) {
    double sum = 0.0, zeros = 0.0;
    for (int i = threadIdx.x; i < kSketchRegs; i += blockDim.x) {
        const uint32_t r = sketch[i];
        sum += ldexp(1.0, -(int)r);
        zeros += r == 0 ? 1.0 : 0.0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
        zeros += __shfl_xor_sync(0xFFFFFFFFu, zeros, o);
    }
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { red[2 * warp] = sum; red[2 * warp + 1] = zeros; }
    __syncthreads();
    sum = 0.0;
    zeros = 0.0;
    for (int w = 0; w < nw; ++w) { sum += red[2 * w]; zeros += red[2 * w + 1]; }
    __syncthreads();
    const double m = (double)kSketchRegs;
    const double e = 0.7213 / (1.0 + 1.079 / m) * m * m / sum;
    if (e <= 2.5 * m && zeros > 0) return m * log(m / zeros);
    return e;
}

__global__ void __launch_bounds__(256) group_insert(GroupArgs a) {
    __shared__ double red[2 * 8];
    const double est = sketch_estimate(a.sketch, red);
    // Path: group when bricks hold kGroupMinRedundancy fragments on average
    // and ~2.5 slots per estimated brick fit the table and the L2 (random
    // atomics on a table in HBM are slower than the sort).
    uint64_t S = 1024;
    while ((double)S < 2.5 * est + 1.0 && S < kGroupMaxSlots) S <<= 1;
    const bool group = a.mode == 2 ||
                       (a.mode == 1 && est * kGroupMinRedundancy <= (double)a.n && (double)S >= 2.5 * est);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.path[0] = group ? 1u : 0u;
        a.path[1] = (uint32_t)(63 - __clzll(S));
    }
    if (!group) return;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gsize = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t warps = gsize / 32, warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
    bool bad = false, full = false;
    // Each lane runs kIlp fragments' probes side by side; a probe reads the
    // slot and takes an atomicCAS only when it is empty.
    for (uint64_t base = warp * 32 * kIlp; base < a.n; base += warps * 32 * kIlp) {
        uint64_t key[kIlp], s[kIlp], bit[kIlp];
        bool live[kIlp];
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = base + k * 32 + lane;
            live[k] = i < a.n;
            const uint64_t code = live[k] ? __ldg(a.frags + i) : 0;
            key[k] = live[k] ? brick_of(a, i, code, &bad) + 1 : 1;  // 0 marks an empty slot
            bit[k] = 1ull << (code & 63);
            s[k] = fmix(key[k]) & (S - 1);
        }
        // At most 4096 probes: an overfull table (a forced grouping) ends in
        // kErrFallback and a rerun, not in a long walk.
        const uint64_t max_probe = S < 4096 ? S : 4096;
        for (uint64_t probe = 0; probe < max_probe; ++probe) {
            bool any = false;
#pragma unroll
            for (int k = 0; k < kIlp; ++k) {
                if (!live[k]) continue;
                uint64_t cur = ld_relaxed(a.table + s[k]);
                if (cur == 0) cur = atomicCAS((unsigned long long*)(a.table + s[k]), 0ull, (unsigned long long)key[k]);
                if (cur == 0 || cur == key[k]) {
                    atomicOr((unsigned long long*)(a.table + kGroupMaxSlots + s[k]), (unsigned long long)bit[k]);
                    live[k] = false;
                } else {
                    s[k] = (s[k] + 1) & (S - 1);
                    any = true;
                }
            }
            if (!any) break;
        }
#pragma unroll
        for (int k = 0; k < kIlp; ++k) full |= live[k];  // table full: cannot happen below ~40% load
    }
    if (bad) atomicOr(a.err, kErrBadInput);
    if (full) atomicOr(a.err, kErrFallback);
}

// The brick list: every occupied slot of the table, (brick, slot), in slot
// order per 2048-slot tile, tiles in any order (the list is sorted next).
// One atomicAdd per tile reserves its place.
constexpr int kCollectItems = 8;
__global__ void __launch_bounds__(256) group_collect(GroupArgs a) {
    __shared__ uint64_t scan[34];
    __shared__ uint64_t base_s;
    if (a.path[0] != 1u) return;
    const uint64_t S = (1ull << a.path[1]) < kGroupMaxSlots ? (1ull << a.path[1]) : kGroupMaxSlots;
    const uint64_t tile = 256ull * kCollectItems;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < S; t0 += (uint64_t)gridDim.x * tile) {
        const uint64_t s0 = t0 + (uint64_t)threadIdx.x * kCollectItems;
        uint64_t key[kCollectItems];
        uint64_t cnt = 0;
#pragma unroll
        for (int j = 0; j < kCollectItems; ++j) {
            key[j] = s0 + j < S ? a.table[s0 + j] : 0;
            cnt += key[j] != 0;
        }
        uint64_t total;
        const uint64_t excl = block_exclusive_sum<uint64_t>(cnt, scan, &total);
        if (threadIdx.x == 0) base_s = total ? atomicAdd((unsigned long long*)a.d_count, (unsigned long long)total) : 0;
        __syncthreads();
        uint64_t pos = base_s + excl;
#pragma unroll
        for (int j = 0; j < kCollectItems; ++j) {
            if (key[j] == 0) continue;
            if (pos < a.cap) {
                a.bricks[pos] = key[j] - 1;
                a.slots[pos] = (uint32_t)(s0 + j);
            } else {
                atomicOr(a.err, kErrFallback);
            }
            ++pos;
        }
        __syncthreads();  // base_s and scan are reused by the next tile
    }
}

__global__ void __launch_bounds__(256) group_gather(GroupArgs a) {
    if (a.path[0] != 1u) return;
    const uint64_t count = *a.d_count < a.cap ? *a.d_count : a.cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.d_count = count;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t lmask = a.seg_code ? (1ull << (a.seg_shift - 6)) - 1 : 0;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < count; i0 += stride * kIlp) {
        uint32_t s[kIlp];
        uint64_t b[kIlp], m[kIlp];
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = i0 + k * stride;
            s[k] = i < count ? a.sorted_slots[i] : 0xFFFFFFFFu;
            b[k] = i < count ? a.sorted_bricks[i] : 0;
        }
#pragma unroll
        for (int k = 0; k < kIlp; ++k) m[k] = s[k] < kGroupMaxSlots ? a.table[kGroupMaxSlots + s[k]] : 0;
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = i0 + k * stride;
            if (i >= count) continue;
            // Batched input: composite brick (segment << (seg_shift - 6)) | local
            // brick -> the chunk's Morton index in place of the segment.
            uint64_t parent = b[k];
            if (a.seg_code) parent = (__ldg(a.seg_code + (b[k] >> (a.seg_shift - 6))) << (a.seg_shift - 6)) | (b[k] & lmask);
            a.parents[i] = parent;
            a.leaves[i] = m[k];
            if (s[k] < kGroupMaxSlots) {
                a.table[s[k]] = 0;  // leave the table empty
                a.table[kGroupMaxSlots + s[k]] = 0;
            }
        }
    }
}

int g_group_sms = 152;

}  // namespace

void group_configure(int sms) { g_group_sms = sms > 0 ? sms : 152; }

static int front_grid(const GroupArgs& a) {
    const uint64_t want = (a.n + 1023) / 1024;
    return (int)(want < (uint64_t)(8 * g_group_sms) ? (want > 0 ? want : 1) : 8 * g_group_sms);
}
void launch_group_sketch(const GroupArgs& a, cudaStream_t s) { group_sketch<<<front_grid(a), 256, 0, s>>>(a); }
void launch_group_insert(const GroupArgs& a, cudaStream_t s) { group_insert<<<front_grid(a), 256, 0, s>>>(a); }
void launch_group_collect(const GroupArgs& a, cudaStream_t s) { group_collect<<<8 * g_group_sms, 256, 0, s>>>(a); }

void launch_group_gather(const GroupArgs& a, cudaStream_t s) {
    const uint64_t want = (a.cap + 1023) / 1024;
    const int g = (int)(want < (uint64_t)(8 * g_group_sms) ? (want > 0 ? want : 1) : 8 * g_group_sms);
    group_gather<<<g, 256, 0, s>>>(a);
}

}  // namespace dagc
