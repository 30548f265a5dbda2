// Device-side building blocks shared by the dagc kernels: error bits, relaxed
// global loads/stores for decoupled look-back, bounded waits and the node hash.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dagc_hash.h"
#include "dagc_kernels.h"

namespace dagc {

// Programmatic dependent launch. Every kernel of a call first lets the next
// kernel of its stream be scheduled (once all of its own CTAs run), then
// waits until the previous kernel has completed and its memory is visible:
// the next kernel's launch and CTA start-up overlap this kernel's tail, and no
// kernel touches memory before its predecessor is done. Without the launch
// attribute (dagc::launch_pdl) both instructions do nothing.
__device__ __forceinline__ void pdl_prologue() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ------------------------------------------------ hash-set dedup table ----

__device__ __forceinline__ uint64_t slot_hash(uint64_t k) {
    // Finaliser of MurmurHash3 (published constants): spreads leaf masks,
    // whose bits are far from uniform, over the table.
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// A key's first slot in a table of S slots (any S): the high word of
// slot_hash(k) * S; probing goes on to the next slot, wrapping at S.
__device__ __forceinline__ uint64_t home_slot(uint64_t k, uint64_t S) { return __umul64hi(slot_hash(k), S); }
__device__ __forceinline__ uint64_t next_slot(uint64_t s, uint64_t S) { return s + 1 == S ? 0 : s + 1; }
__device__ __forceinline__ uint32_t next_slot(uint32_t s, uint32_t S) { return s + 1 == S ? 0u : s + 1; }

// Buckets of the top-bit form: a power of two with ~kDedupPerBucket keys each
// for u keys; a key's bucket is key >> *shift.
__device__ __forceinline__ uint32_t topbit_buckets(uint64_t u, int* shift) {
    uint32_t nb = 1;
    int lg = 0;
    while ((uint64_t)nb * kDedupPerBucket < u && nb < kDedupMaxBuckets) { nb <<= 1; ++lg; }
    *shift = 64 - lg;
    return nb;
}

// Up to this many items a node level claims its slot with one atomicCAS (one
// round trip, latency-bound sizes); above it, it reads first and claims only
// an empty slot (L2 atomic throughput).
constexpr uint64_t kDedupClaimFirstMax = 1ull << 20;

// Upper limit on waits: ~2^20 polls with exponential back-off capped at 1 us,
// i.e. about one second, after which the waiter flags kErrTimeout.
constexpr uint32_t kSpinLimit = 1u << 20;

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t lanemask_le() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_le;" : "=r"(m));
    return m;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Shared-memory address of a generic pointer (for cp.async operands).
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void backoff(uint32_t iter) {
    __nanosleep(iter < 10 ? (32u << (iter / 2)) : 1000u);
}

// ------------------------------------------------- single-value look-back ----
// Status word per tile: bits 63..62 = flag (0 not ready, 1 aggregate,
// 2 inclusive prefix), bits 61..0 = value. The array must be zero before use.
constexpr uint64_t kSvAggregate = 1ull << 62;
constexpr uint64_t kSvInclusive = 2ull << 62;
constexpr uint64_t kSvValueMask = (1ull << 62) - 1;

// Called by all 32 lanes of ONE warp. Publishes this tile's aggregate, walks
// back over predecessors 32 at a time and returns the exclusive prefix (same
// value in every lane); publishes the inclusive prefix before returning.
__device__ __forceinline__ uint64_t sv_lookback(uint64_t* status, uint32_t tile, uint64_t aggregate,
                                                uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) st_relaxed(status, kSvInclusive | aggregate);
        return 0;
    }
    if (lane == 0) st_relaxed(status + tile, kSvAggregate | aggregate);
    uint64_t exclusive = 0;
    int64_t base = (int64_t)tile - 1;
    uint32_t iter = 0;
    while (true) {
        const int64_t idx = base - (int64_t)lane;
        uint64_t s = idx >= 0 ? ld_relaxed(status + idx) : kSvInclusive;
        while (__any_sync(0xFFFFFFFFu, (s >> 62) == 0)) {
            if (++iter > kSpinLimit) {
                if (lane == 0) atomicOr(err, kErrTimeout);
                s = kSvInclusive;  // give up: treat as a zero prefix so the walk ends
                break;
            }
            backoff(iter);
            if ((s >> 62) == 0) s = ld_relaxed(status + idx);
        }
        if ((s >> 62) == 0) s = kSvInclusive;
        const uint32_t inc = __ballot_sync(0xFFFFFFFFu, (s >> 62) == 2);
        uint64_t v = s & kSvValueMask;
        if (inc) {
            const uint32_t first = __ffs(inc) - 1;  // nearest tile with an inclusive prefix
            if (lane > first) v = 0;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        exclusive += v;
        if (inc) break;
        base -= 32;
    }
    if (lane == 0) st_relaxed(status + tile, kSvInclusive | (exclusive + aggregate));
    return exclusive;
}

// Block-wide exclusive sum over blockDim.x threads (blockDim.x a multiple of
// 32, at most 1024). `scratch` holds >= 33 words of shared memory. Returns the
// exclusive prefix; *total receives the block total (all threads).
template <typename T>
__device__ __forceinline__ T block_exclusive_sum(T v, T* scratch, T* total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nwarps = blockDim.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) scratch[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nwarps ? scratch[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        if (lane < nwarps) scratch[lane] = w;  // inclusive warp prefixes
        if (lane == 31) scratch[32] = w;
    }
    __syncthreads();
    const T warp_excl = warp ? scratch[warp - 1] : T(0);
    *total = scratch[32];
    const T r = warp_excl + x - v;
    __syncthreads();  // scratch may be reused by the caller
    return r;
}

}  // namespace dagc
