// The node hash, usable from host C++ and device code.
//
// MurmurHash128xN over the 8 child hashes seen as 4 x 128-bit blocks, seed 0,
// Size = 4 (the block count, not a byte length), low 64 bits of the result;
// a zero hash becomes 1 so that 0 can mark an empty child. Restates
// src/Utils.h:86-94 (MurmurHash64), :119-154 (MurmurHash128xN) and
// HashChildrenHashes, src/DAGCompression.cu:758-763.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define DAGC_HD __host__ __device__ __forceinline__
#else
#define DAGC_HD inline
#endif

namespace dagc {

DAGC_HD uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

DAGC_HD uint64_t fmix64(uint64_t h) {
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}

DAGC_HD uint64_t hash_children(const uint64_t c[8]) {
    const uint64_t k1m = 0x87c37b91114253d5ull, k2m = 0x4cf5ad432745937full;
    uint64_t h1 = 0, h2 = 0;
#if defined(__CUDACC__)
#pragma unroll
#endif
    for (int b = 0; b < 4; ++b) {
        uint64_t k1 = c[2 * b], k2 = c[2 * b + 1];
        k1 *= k1m; k1 = rotl64(k1, 31); k1 *= k2m; h1 ^= k1;
        h1 = rotl64(h1, 27); h1 += h2; h1 = h1 * 5 + 0x52dce729;
        k2 *= k2m; k2 = rotl64(k2, 33); k2 *= k1m; h2 ^= k2;
        h2 = rotl64(h2, 31); h2 += h1; h2 = h2 * 5 + 0x38495ab5;
    }
    h1 ^= 4; h2 ^= 4;
    h1 += h2; h2 += h1;
    h1 = fmix64(h1); h2 = fmix64(h2);
    h1 += h2;
    return h1 == 0 ? 1 : h1;
}

}  // namespace dagc
