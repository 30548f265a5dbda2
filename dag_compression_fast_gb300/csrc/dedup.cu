// Level deduplication by hash set + ordering of the distinct keys, for
// sm_103a. Replaces, for one level (or the leaves), the reference's SortLevel
// (src/DAGCompression.cu:864-914): sort (hash, index) pairs, flag runs, scan,
// scatter to unique ids. Same result: the distinct keys in ascending order,
// their payloads, and a map item -> unique id. Instead of eight 8-bit radix
// passes over every item, the distinct keys are found first and only those
// are ordered:
//
//   dedup_insert   every item inserts its key into an open-addressing table
//                  (linear probing, atomicCAS on the key); the first inserter
//                  of a key records itself as the slot's representative and
//                  appends its key to the unique list (leaf masks) or
//                  (key, slot, itself) straight to its bucket (node hashes:
//                  MurmurHash outputs, so their top bits are the bucket and
//                  the bucket count follows from the item count; dedup_map of
//                  the previous level zeroed the bucket counters);
//   leaf masks     (far from uniform) the unique list is ordered by a 64-bit
//                  keys-only radix sort (the caller's sort), then
//   dedup_assign   finds each sorted key's slot (probing as the insert did)
//                  and gives it its unique id (its rank);
//   dedup_sort     (node hashes) each bucket is ranked in shared memory (rank
//                  = number of smaller keys) and written at its global ranks,
//                  with the representative's payload; the unique id goes to
//                  the slot and the slot's key is cleared;
//   dedup_map      every item reads its unique id and representative through
//                  its slot, duplicates are compared in full with their
//                  representative (collision check). Every slot's key is
//                  cleared once per distinct key: by dedup_sort (node hashes)
//                  or here by the key's representative (leaf masks, after
//                  every probe of dedup_assign); items sharing a slot
//                  otherwise only read its aux word.
//
// What the fixed sizes cannot hold (table, unique list, a bucket) sets
// kErrFallback, and the caller reruns the call with the radix-sort form.

#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

namespace dagc {
namespace {

__device__ __forceinline__ uint64_t unique_count(const DedupArgs& a) {
    const uint64_t u = a.state->u;
    return u < a.uniq_cap ? u : a.uniq_cap;
}

// Items per lane in flight at once (independent probe chains).
constexpr int kIlp = 4;

__global__ void __launch_bounds__(256, 4) dedup_insert(DedupArgs a) {
    pdl_prologue();
    if (!a.to_list && a.state->inserted) return;  // extract_level inserted this level's hashes
    const uint64_t n = *a.d_n;
    const uint64_t S = table_size_for(n, a.to_list);
    const uint32_t S32 = (uint32_t)S;
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t gtid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t gsize = (uint64_t)gridDim.x * blockDim.x;
    // Node hashes are uniform, so their top bits give the bucket at once:
    // winners append straight to their bucket (the previous level's
    // dedup_map left the counters zero). Leaf masks go to the unique list.
    if (S > a.table_cap || n > a.item_cap) {
        if (gtid == 0) atomicOr(a.err, kErrFallback);
        return;
    }
    int shift = 64;
    const uint32_t nb = a.to_list ? 0u : topbit_buckets(n, &shift);
    if (!a.to_list) {
        if ((uint64_t)nb * kDedupTopBitCap > a.bucket_area) {
            if (gtid == 0) { atomicOr(a.err, kErrFallback); a.state->nbuckets = 0; }
            return;
        }
        if (gtid == 0) a.state->nbuckets = nb;
    }
    uint32_t* aux = reinterpret_cast<uint32_t*>(a.table_aux);  // slot s: [4s] representative, [4s+1] unique id
    const uint64_t warps = gsize / 32;
    const uint64_t warp = gtid / 32;
    bool bad = false, full = false;
    // Each lane takes kIlp items (32 apart) per round and runs their probe
    // chains side by side. A probe reads the slot first and only an empty
    // slot takes an atomicCAS: duplicated keys (common leaf masks) would
    // otherwise serialise on their slot's atomics.
    for (uint64_t base = warp * 32 * kIlp; base < n; base += warps * 32 * kIlp) {
        uint64_t h[kIlp];
        uint32_t s[kIlp];  // slot indices (tables hold fewer than 2^32 slots)
        bool live[kIlp], won[kIlp];
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = base + k * 32 + lane;
            won[k] = false;
            live[k] = i < n;
            h[k] = live[k] ? a.keys[i] : 0;
            if (live[k] && h[k] == 0) { bad = true; live[k] = false; }  // 0 marks an empty slot
            s[k] = (uint32_t)home_slot(h[k], S);
        }
        bool found[kIlp];
#pragma unroll
        for (int k = 0; k < kIlp; ++k) found[k] = false;
        // Leaf masks repeat (many items per key), and large levels are bound
        // by L2 atomic throughput: read first, claim only an empty slot. The
        // read takes a slot and the one after it (two loads in flight,
        // usually one sector), so that a key displaced by one slot, or an
        // empty slot right after an occupied one, costs no second round
        // trip. Small node levels are bound by latency: claim directly (one
        // round trip instead of two). Each round issues every pending item's
        // reads, then every claim, back to back (no result is used before
        // the last one is issued).
        const bool read_first = a.to_list || n > kDedupClaimFirstMax;
        for (uint64_t round = 0; round < S; ++round) {
            bool pend[kIlp], claim[kIlp];
            uint64_t cur[kIlp], nxt[kIlp];
#pragma unroll
            for (int k = 0; k < kIlp; ++k) {
                pend[k] = live[k] && !won[k] && !found[k];
                claim[k] = pend[k];
                cur[k] = 0;
                nxt[k] = 0;
            }
            if (read_first) {
#pragma unroll
                for (int k = 0; k < kIlp; ++k) {
                    if (pend[k]) {
                        cur[k] = ld_relaxed(a.table_key + 2ull * s[k]);
                        nxt[k] = ld_relaxed(a.table_key + 2ull * next_slot(s[k], S32));
                    }
                }
                // In probe order: a match ends the search; the first empty
                // slot is claimed; two other keys move the probe on by two.
#pragma unroll
                for (int k = 0; k < kIlp; ++k) {
                    if (!pend[k]) continue;
                    if (cur[k] == h[k]) { found[k] = true; claim[k] = false; continue; }
                    if (cur[k] == 0) continue;
                    s[k] = next_slot(s[k], S32);
                    if (nxt[k] == h[k]) { found[k] = true; claim[k] = false; continue; }
                    if (nxt[k] != 0) { s[k] = next_slot(s[k], S32); claim[k] = false; }
                }
            }
#pragma unroll
            for (int k = 0; k < kIlp; ++k)
                if (claim[k]) cur[k] = atomicCAS((unsigned long long*)(a.table_key + 2ull * s[k]), 0ull, (unsigned long long)h[k]);
            bool any = false;
#pragma unroll
            for (int k = 0; k < kIlp; ++k) {
                if (!pend[k] || found[k]) continue;
                if (!claim[k]) { any = true; continue; }  // both slots held other keys
                if (cur[k] == 0) won[k] = true;
                else if (cur[k] == h[k]) found[k] = true;
                else { s[k] = next_slot(s[k], S32); any = true; }
            }
            if (!any) break;
        }
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = base + k * 32 + lane;
            if (i < n) {
                const bool placed = live[k] && (won[k] || found[k]);
                if (live[k] && !placed) full = true;  // cannot happen below half load; rerun rather than guess
                a.item_slot[i] = placed ? s[k] : 0xFFFFFFFFu;
            }
        }
        // Winners append to the unique list: one atomic per warp for all its
        // item rows. Every lane takes part in the ballots and shuffles.
        uint32_t wm[kIlp];
        uint32_t wtotal = 0;
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            wm[k] = __ballot_sync(0xFFFFFFFFu, won[k]);
            wtotal += __popc(wm[k]);
        }
        uint64_t pos0 = 0;
        if (lane == 0 && wtotal)
            pos0 = atomicAdd((unsigned long long*)&a.state->u, (unsigned long long)wtotal);
        pos0 = __shfl_sync(0xFFFFFFFFu, pos0, 0);
        if (a.to_list) {
#pragma unroll
            for (int k = 0; k < kIlp; ++k) {
                if (won[k]) {
                    const uint64_t i = base + k * 32 + lane;
                    const uint64_t pos = pos0 + __popc(wm[k] & lanemask_lt());
                    aux[4ull * s[k]] = (uint32_t)i;
                    if (pos < a.uniq_cap) {
                        a.uniq_key[pos] = h[k];
                    } else {
                        full = true;
                    }
                }
                pos0 += __popc(wm[k]);
            }
        } else {
            // Every winner's bucket slot is reserved before any is used.
            uint32_t bslot[kIlp];
#pragma unroll
            for (int k = 0; k < kIlp; ++k) {
                const uint32_t b = shift >= 64 ? 0u : (uint32_t)(h[k] >> shift);
                bslot[k] = won[k] ? atomicAdd(a.bucket_count + b, 1u) : 0u;
            }
#pragma unroll
            for (int k = 0; k < kIlp; ++k) {
                if (won[k]) {
                    const uint64_t i = base + k * 32 + lane;
                    const uint64_t pos = pos0 + __popc(wm[k] & lanemask_lt());
                    const uint32_t b = shift >= 64 ? 0u : (uint32_t)(h[k] >> shift);
                    aux[4ull * s[k]] = (uint32_t)i;
                    if (pos < a.uniq_cap && bslot[k] < kDedupTopBitCap) {
                        const uint64_t e = (uint64_t)b * kDedupTopBitCap + bslot[k];
                        a.bucket[e] = make_uint4((uint32_t)h[k], (uint32_t)(h[k] >> 32), s[k], (uint32_t)i);
                    } else {
                        full = true;
                    }
                }
                pos0 += __popc(wm[k]);
            }
        }
    }
    if (bad) atomicOr(a.err, kErrBadInput);
    if (full) atomicOr(a.err, kErrFallback);
}

// Leaf masks, after the sort of the unique list: the key of rank r is the
// r-th distinct key; the slot holding it (found by the insert's probe
// sequence, every key being in the table) gets unique id r. The keys stay
// until dedup_map: clearing one here could cut another key's probe sequence.
__global__ void __launch_bounds__(256) dedup_assign(DedupArgs a, const uint64_t* sorted) {
    pdl_prologue();
    const uint64_t u = unique_count(a);
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.d_out_n = u < a.out_capacity ? u : a.out_capacity;
    const uint64_t n = *a.d_n;
    const uint64_t S = table_size_for(n, true);
    if (S > a.table_cap || n > a.item_cap) return;  // insert did nothing (fallback set)
    const uint32_t S32 = (uint32_t)S;
    uint32_t* aux = reinterpret_cast<uint32_t*>(a.table_aux);
    bool lost = false;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < u; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = sorted[r];
        uint32_t sl = (uint32_t)home_slot(key, S);
        bool hit = false;
        for (uint32_t probe = 0; probe < S32; ++probe) {
            const uint64_t cur = a.table_key[2ull * sl];
            if (cur == key) { hit = true; break; }
            if (cur == 0) break;
            sl = next_slot(sl, S32);
        }
        if (hit && r < a.out_capacity) aux[4ull * sl + 1] = (uint32_t)r;
        else lost = true;
    }
    if (lost) atomicOr(a.err, kErrCapacity);
}

// Each CTA takes a contiguous range of buckets; a bucket's keys are distinct,
// so a key's rank is the number of smaller keys in its bucket.
constexpr int kBucketThreads = 256;

__global__ void __launch_bounds__(kBucketThreads) dedup_sort(DedupArgs a) {
    pdl_prologue();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t* key = reinterpret_cast<uint64_t*>(smem_raw);  // bucket room: kDedupTopBitCap
    __shared__ uint32_t red[kBucketThreads / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t nb = a.state->nbuckets;
    if (blockIdx.x == 0) {
        // The distinct keys are the bucket entries (the insert appended every
        // first inserter to its bucket).
        __shared__ uint32_t tot[kBucketThreads / 32];
        uint32_t part = 0;
        for (uint32_t b = tid; b < nb; b += kBucketThreads) part += min(a.bucket_count[b], kDedupTopBitCap);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
        if (lane == 0) tot[warp] = part;
        __syncthreads();
        if (tid == 0) {
            uint64_t u = 0;
            for (int w = 0; w < kBucketThreads / 32; ++w) u += tot[w];
            if (u > a.uniq_cap) atomicOr(a.err, kErrFallback);
            *a.d_out_n = u < a.uniq_cap ? u : a.uniq_cap;
        }
    }
    if (nb == 0) return;
    constexpr uint32_t cap = kDedupTopBitCap;
    const uint32_t b0 = (uint32_t)((uint64_t)nb * blockIdx.x / gridDim.x);
    const uint32_t b1 = (uint32_t)((uint64_t)nb * (blockIdx.x + 1) / gridDim.x);
    if (b0 >= b1) return;
    // Keys in the buckets before this range (8 independent loads per thread
    // in flight).
    uint32_t part = 0;
    for (uint32_t x0 = 0; x0 < b0; x0 += 8 * kBucketThreads) {
        uint32_t c[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const uint32_t x = x0 + u * kBucketThreads + tid;
            c[u] = x < b0 ? a.bucket_count[x] : 0u;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) part += min(c[u], cap);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
    if (lane == 0) red[warp] = part;
    __syncthreads();
    uint64_t start = 0;
    for (int w = 0; w < kBucketThreads / 32; ++w) start += red[w];
    uint32_t* aux = reinterpret_cast<uint32_t*>(a.table_aux);
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t cnt = min(a.bucket_count[b], cap);
        const uint64_t src = (uint64_t)b * cap;
        __syncthreads();  // the previous bucket's keys are no longer read
        for (uint32_t j = tid; j < cnt; j += kBucketThreads) {
            const uint4 e = a.bucket[src + j];
            key[j] = (uint64_t)e.x | (uint64_t)e.y << 32;
        }
        __syncthreads();
        for (uint32_t j = tid; j < cnt; j += kBucketThreads) {
            // Slot and representative come with the key; their loads (and the
            // payload's) are in flight while the rank is counted.
            const uint4 ent = a.bucket[src + j];
            const uint32_t s = ent.z;
            const uint32_t rep = ent.w;
            uint8_t m = 0;
            uint4 c0 = make_uint4(0, 0, 0, 0), c1 = c0;
            if (a.out_masks) {
                m = a.masks[rep];
                const uint4* s4 = reinterpret_cast<const uint4*>(a.children + (uint64_t)rep * 8);
                c0 = s4[0];
                c1 = s4[1];
            }
            const uint64_t k = key[j];
            uint32_t r = 0;
#pragma unroll 8
            for (uint32_t x = 0; x < cnt; ++x) r += key[x] < k;
            const uint64_t uid = start + r;
            if (uid < a.out_capacity && s < a.table_cap) {
                a.out_keys[uid] = k;
                aux[4 * (uint64_t)s + 1] = (uint32_t)uid;
                a.table_key[2 * (uint64_t)s] = 0;  // the slot is empty for the next level (dedup_map reads only aux)
                if (a.out_masks) {
                    a.out_masks[uid] = m;
                    uint4* d4 = reinterpret_cast<uint4*>(a.out_children + uid * 8);
                    d4[0] = c0;
                    d4[1] = c1;
                }
            } else {
                atomicOr(a.err, kErrCapacity);
            }
        }
        start += cnt;
    }
}

__global__ void __launch_bounds__(256) dedup_map(DedupArgs a) {
    pdl_prologue();
    // The bucket counters, read by dedup_sort, start the next level at zero.
    for (uint64_t b = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b < kDedupMaxBuckets;
         b += (uint64_t)gridDim.x * blockDim.x)
        a.bucket_count[b] = 0;
    const uint64_t n = *a.d_n;
    if (table_size_for(n, a.to_list) > a.table_cap || n > a.item_cap) return;  // insert did nothing
    const uint32_t last = a.out_capacity ? (uint32_t)(a.out_capacity - 1) : 0u;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool collision = false;
    // kIlp items per thread per round, their slot reads in flight together.
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += stride * kIlp) {
        uint32_t s[kIlp];
        uint64_t aux[kIlp];
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = i0 + k * stride;
            s[k] = i < n ? a.item_slot[i] : 0xFFFFFFFFu;
        }
#pragma unroll
        for (int k = 0; k < kIlp; ++k) aux[k] = s[k] < a.table_cap ? a.table_aux[2 * (uint64_t)s[k]] : 0;
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
            const uint64_t i = i0 + k * stride;
            if (i >= n) continue;
            uint32_t uid = 0;
            if (s[k] < a.table_cap) {
                const uint32_t rep = (uint32_t)aux[k];
                uid = (uint32_t)(aux[k] >> 32);
                if (a.to_list && rep == (uint32_t)i) a.table_key[2 * (uint64_t)s[k]] = 0;  // empty for the next level
                if (a.masks && rep != (uint32_t)i && rep < n) {
                    const uint4* x = reinterpret_cast<const uint4*>(a.children + i * 8);
                    const uint4* y = reinterpret_cast<const uint4*>(a.children + (uint64_t)rep * 8);
                    const uint4 x0 = x[0], x1 = x[1], y0 = y[0], y1 = y[1];
                    collision |= a.masks[i] != a.masks[rep] || x0.x != y0.x || x0.y != y0.y || x0.z != y0.z ||
                                 x0.w != y0.w || x1.x != y1.x || x1.y != y1.y || x1.z != y1.z || x1.w != y1.w;
                }
            }
            // Ids stay inside the next level's arrays even when a fallback or
            // an error discards this call.
            a.map[i] = uid <= last ? uid : last;
        }
    }
    if (collision) atomicOr(a.err, kErrCollision);
}

int g_sms = 152;

}  // namespace

void dedup_configure(int sms) {
    cudaFuncSetAttribute(dedup_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kDedupTopBitCap * 8));
    g_sms = sms > 0 ? sms : 152;
}

namespace {
int item_grid(const DedupArgs& a) {
    const uint64_t want = (a.item_cap + 255) / 256;
    const int g = 8 * g_sms;  // full occupancy: 8 CTAs of 256 threads per SM
    return (int)(want < (uint64_t)g ? (want > 0 ? want : 1) : g);
}
}  // namespace

void launch_dedup_insert(const DedupArgs& a, cudaStream_t s) {
    launch_pdl(dedup_insert, dim3(item_grid(a)), dim3(256), 0, s, a);
}

void launch_dedup_assign(const DedupArgs& a, const uint64_t* sorted, cudaStream_t s) {
    const uint64_t want = (a.uniq_cap + 255) / 256;
    const int g = (int)(want < (uint64_t)(8 * g_sms) ? (want > 0 ? want : 1) : 8 * g_sms);
    launch_pdl(dedup_assign, dim3(g), dim3(256), 0, s, a, sorted);
}

void launch_dedup_map(const DedupArgs& a, cudaStream_t s) {
    launch_pdl(dedup_map, dim3(item_grid(a)), dim3(256), 0, s, a);
}

int launch_dedup(const DedupArgs& a, cudaStream_t s) {
    launch_dedup_insert(a, s);  // returns at once when extract_level inserted
    const uint64_t nbmax = (a.uniq_cap + kDedupPerBucket - 1) / kDedupPerBucket;
    const int gs = (int)(nbmax < (uint64_t)(8 * g_sms) ? (nbmax > 0 ? nbmax : 1) : 8 * g_sms);
    launch_pdl(dedup_sort, dim3(gs), dim3(kBucketThreads), kDedupTopBitCap * 8, s, a);
    launch_dedup_map(a, s);
    return 3;
}

}  // namespace dagc
