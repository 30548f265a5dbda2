// CPU oracle for the DAG compression path of Phyronnaz/DAG_Compression_Fast.
//
// TEST INFRASTRUCTURE ONLY. This file is a plain restatement of the reference
// algorithm, used as the checker for the CUDA library and as the timed CPU
// baseline. Nothing in the product (the dagc library) links, loads or calls it.
//
// Every function cites the reference file:line it restates (paths are relative
// to the reference project root). Parity pins:
//   * the node hash is checked against known answers produced by compiling the
//     reference's own src/Utils.h (see ref_hash.cpp / tests/golden/hash_kats.json);
//   * sort / unique / reduce-by-key / scan / merge are exact integer library
//     operations in the reference (CUB 1.8, moderngpu 2.x, Thrust of CUDA 10.1);
//     they are restated here with std::sort / std::unique or a radix sort and
//     are defined by their mathematical result.
//
// Two execution modes share the same results:
//   threads == 1 : std::sort based, the most literal restatement;
//   threads  > 1 : parallel LSD radix sort (std::thread) for the sorts, used as
//                  the multi-core CPU baseline.

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <thread>
#include <vector>

namespace {

enum OracleStatus : int {
    ORACLE_OK = 0,
    ORACLE_ERR_INVALID_ARGUMENT = 1,
    ORACLE_ERR_BAD_INPUT = 3,
    ORACLE_ERR_HASH_COLLISION = 4,
    ORACLE_ERR_TOO_LARGE = 7,
};

constexpr uint32_t kEmpty = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Hash: src/Utils.h:40-42 (Rotl64), :86-94 (MurmurHash64), :119-154
// (MurmurHash128xN with Size = 4 blocks, Seed = 0) and the 0 -> 1 rule of
// HashChildrenHashes, src/DAGCompression.cu:758-763.
// ---------------------------------------------------------------------------
inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

inline uint64_t fmix64(uint64_t h) {
    h ^= h >> 33;
    h *= 0xff51afd7ed558ccdull;
    h ^= h >> 33;
    h *= 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 33;
    return h;
}

uint64_t hash_children(const uint64_t c[8]) {
    const uint64_t k_c1 = 0x87c37b91114253d5ull;
    const uint64_t k_c2 = 0x4cf5ad432745937full;
    uint64_t h1 = 0, h2 = 0;
    for (int b = 0; b < 4; ++b) {
        uint64_t k1 = c[2 * b + 0];
        uint64_t k2 = c[2 * b + 1];
        k1 *= k_c1; k1 = rotl64(k1, 31); k1 *= k_c2; h1 ^= k1;
        h1 = rotl64(h1, 27); h1 += h2; h1 = h1 * 5 + 0x52dce729;
        k2 *= k_c2; k2 = rotl64(k2, 33); k2 *= k_c1; h2 ^= k2;
        h2 = rotl64(h2, 31); h2 += h1; h2 = h2 * 5 + 0x38495ab5;
    }
    h1 ^= 4; h2 ^= 4;
    h1 += h2; h2 += h1;
    h1 = fmix64(h1); h2 = fmix64(h2);
    h1 += h2;
    return h1 == 0 ? 1 : h1;
}

inline uint32_t popc8(uint32_t m) { return (uint32_t)__builtin_popcount(m & 0xFFu); }

// src/Utils.h:72-75
inline uint32_t child_offset(uint32_t mask, uint32_t child) {
    return popc8(mask & ((1u << child) - 1u)) + 1;
}

// ---------------------------------------------------------------------------
// Parallel LSD radix sort (baseline mode). Stable, 8-bit digits.
// ---------------------------------------------------------------------------
template <typename F>
void parallel_for_chunks(int threads, uint64_t n, F&& fn) {
    if (threads <= 1 || n < (1u << 16)) { fn(0, 0, n); return; }
    std::vector<std::thread> pool;
    const uint64_t per = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const uint64_t lo = std::min<uint64_t>(n, per * t);
        const uint64_t hi = std::min<uint64_t>(n, lo + per);
        pool.emplace_back([&, t, lo, hi] { fn(t, lo, hi); });
    }
    for (auto& th : pool) th.join();
}

// Sorts keys (and optional u32 values) on bits [lo_bit, hi_bit).
void radix_sort(std::vector<uint64_t>& keys, std::vector<uint32_t>* vals,
                int lo_bit, int hi_bit, int threads) {
    const uint64_t n = keys.size();
    if (n < 2 || hi_bit <= lo_bit) return;
    if (threads < 1) threads = 1;
    if (n < (1u << 16)) threads = 1;
    std::vector<uint64_t> ktmp(n);
    std::vector<uint32_t> vtmp(vals ? n : 0);
    std::vector<uint64_t> hist((size_t)threads * 256);
    for (int shift = lo_bit; shift < hi_bit; shift += 8) {
        const int bits = std::min(8, hi_bit - shift);
        const uint64_t dmask = (1ull << bits) - 1;
        std::fill(hist.begin(), hist.end(), 0);
        parallel_for_chunks(threads, n, [&](int t, uint64_t lo, uint64_t hi) {
            uint64_t* h = &hist[(size_t)t * 256];
            for (uint64_t i = lo; i < hi; ++i) h[(keys[i] >> shift) & dmask]++;
        });
        // Skip passes where every key has the same digit (identity permutation).
        {
            uint64_t nonzero = 0;
            for (int d = 0; d < 256; ++d) {
                uint64_t s = 0;
                for (int t = 0; t < threads; ++t) s += hist[(size_t)t * 256 + d];
                nonzero += (s != 0);
            }
            if (nonzero <= 1) continue;
        }
        // Exclusive offsets in (digit, thread) order -> stable.
        uint64_t sum = 0;
        for (int d = 0; d < 256; ++d)
            for (int t = 0; t < threads; ++t) {
                uint64_t c = hist[(size_t)t * 256 + d];
                hist[(size_t)t * 256 + d] = sum;
                sum += c;
            }
        parallel_for_chunks(threads, n, [&](int t, uint64_t lo, uint64_t hi) {
            uint64_t* h = &hist[(size_t)t * 256];
            for (uint64_t i = lo; i < hi; ++i) {
                const uint64_t k = keys[i];
                const uint64_t dst = h[(k >> shift) & dmask]++;
                ktmp[dst] = k;
                if (vals) vtmp[dst] = (*vals)[i];
            }
        });
        keys.swap(ktmp);
        if (vals) vals->swap(vtmp);
    }
}

// ---------------------------------------------------------------------------
// DAG data model: FCpuDag / FCpuLevel / FChildrenIndices,
// src/DAGCompression.h:6-40. Levels[0] is the root level.
// ---------------------------------------------------------------------------
struct Level {
    std::vector<uint8_t> masks;      // ChildMasks
    std::vector<uint32_t> children;  // ChildrenIndices, 8 per node
    std::vector<uint64_t> hashes;    // Hashes, ascending
    uint64_t size() const { return hashes.size(); }
};

struct Dag {
    std::vector<Level> levels;
    std::vector<uint64_t> leaves;  // ascending 4x4x4 masks
};

// SortLevel, src/DAGCompression.cu:864-914: sort (key, iota) pairs, flag
// "differs from previous", inclusive scan -> unique id, scatter the map and
// every payload array into NumUniques slots. Returns the orig -> unique map.
// `same_payload(a, b)` implements the full-compare collision check the
// reference does not have (it compares hashes only): equal keys must carry
// equal payloads.
template <typename SamePayload>
int sort_level(const std::vector<uint64_t>& keys, int threads,
               std::vector<uint32_t>& map, std::vector<uint32_t>& reps,
               SamePayload&& same_payload) {
    const uint64_t n = keys.size();
    std::vector<uint32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0u);
    if (threads > 1) {
        std::vector<uint64_t> k = keys;
        radix_sort(k, &perm, 0, 64, threads);
    } else {
        std::sort(perm.begin(), perm.end(),
                  [&](uint32_t a, uint32_t b) { return keys[a] < keys[b]; });
    }
    map.assign(n, 0);
    reps.clear();
    for (uint64_t i = 0; i < n; ++i) {
        const uint32_t p = perm[i];
        if (i == 0 || keys[p] != keys[perm[i - 1]]) {
            reps.push_back(p);
        } else if (!same_payload(reps.back(), p)) {
            return ORACLE_ERR_HASH_COLLISION;
        }
        map[p] = (uint32_t)(reps.size() - 1);
    }
    return ORACLE_OK;
}

// CreateDAG, src/DAGCompression.cu:1003-1107 (with ExtractLevel :916-974,
// ComputeHashes :827-833, HashChildren :765-774).
int create_dag(const uint64_t* in, uint64_t n, int depth, int threads, Dag& out) {
    if (depth < 2 || depth > 21) return ORACLE_ERR_INVALID_ARGUMENT;
    out.levels.assign(depth - 2, Level{});
    out.leaves.clear();
    if (n == 0) return ORACLE_OK;  // :1010-1013
    if (n >= (1ull << 31)) return ORACLE_ERR_TOO_LARGE;  // the reference casts counts to int32
    const int bits = 3 * depth;
    if (bits < 64) {
        for (uint64_t i = 0; i < n; ++i)
            if (in[i] >> bits) return ORACLE_ERR_BAD_INPUT;
    }

    // SortKeys on bits [0, 3*Depth) (:1026) + SelectUnique (:1036).
    std::vector<uint64_t> codes(in, in + n);
    if (threads > 1) radix_sort(codes, nullptr, 0, bits, threads);
    else std::sort(codes.begin(), codes.end());
    codes.erase(std::unique(codes.begin(), codes.end()), codes.end());

    // Leaves: ReduceByKey(code >> 6, 1 << (code & 63), |) (:1044-1068).
    std::vector<uint64_t> parents;
    std::vector<uint64_t> leaf_masks;
    for (uint64_t i = 0; i < codes.size(); ++i) {
        const uint64_t p = codes[i] >> 6;
        const uint64_t bit = 1ull << (codes[i] & 63);
        if (i == 0 || p != parents.back()) { parents.push_back(p); leaf_masks.push_back(bit); }
        else leaf_masks.back() |= bit;
    }

    // SortLevel on the leaves; the "hash" of a leaf is its mask (:1071).
    std::vector<uint32_t> map, reps;
    int st = sort_level(leaf_masks, threads, map, reps, [](uint32_t, uint32_t) { return true; });
    if (st) return st;
    out.leaves.resize(reps.size());
    for (size_t u = 0; u < reps.size(); ++u) out.leaves[u] = leaf_masks[reps[u]];

    const std::vector<uint64_t>* prev_hashes = &out.leaves;
    std::vector<uint64_t> child_codes = std::move(parents);
    for (int level = depth - 3; level >= 0; --level) {
        // ExtractLevel (:916-974).
        std::vector<uint64_t> node_codes;
        std::vector<uint8_t> masks;
        std::vector<uint32_t> children;
        for (uint64_t i = 0; i < child_codes.size(); ++i) {
            const uint64_t p = child_codes[i] >> 3;
            const uint32_t slot = (uint32_t)(child_codes[i] & 7);
            if (i == 0 || p != node_codes.back()) {
                node_codes.push_back(p);
                masks.push_back(0);
                children.insert(children.end(), 8, kEmpty);
            }
            masks.back() |= (uint8_t)(1u << slot);
            children[(node_codes.size() - 1) * 8 + slot] = map[i];
        }
        // ComputeHashes (:827-833).
        const uint64_t nn = node_codes.size();
        std::vector<uint64_t> hashes(nn);
        for (uint64_t i = 0; i < nn; ++i) {
            uint64_t h[8];
            for (int c = 0; c < 8; ++c) {
                const uint32_t idx = children[i * 8 + c];
                h[c] = idx == kEmpty ? 0 : (*prev_hashes)[idx];
            }
            hashes[i] = hash_children(h);
        }
        // SortLevel (:1087) with the full-compare collision check.
        st = sort_level(hashes, threads, map, reps, [&](uint32_t a, uint32_t b) {
            return masks[a] == masks[b] &&
                   std::memcmp(&children[(size_t)a * 8], &children[(size_t)b * 8], 32) == 0;
        });
        if (st) return st;
        Level& L = out.levels[level];
        const size_t u = reps.size();
        L.masks.resize(u);
        L.children.resize(u * 8);
        L.hashes.resize(u);
        for (size_t j = 0; j < u; ++j) {
            const uint32_t r = reps[j];
            L.masks[j] = masks[r];
            std::memcpy(&L.children[j * 8], &children[(size_t)r * 8], 32);
            L.hashes[j] = hashes[r];
        }
        prev_hashes = &L.hashes;
        child_codes = std::move(node_codes);
    }
    // check(PreviousLevelHashes.Num() == 1) (:1093)
    if (depth > 2 && out.levels[0].size() != 1) return ORACLE_ERR_BAD_INPUT;
    if (depth == 2 && out.leaves.size() != 1) return ORACLE_ERR_BAD_INPUT;
    return ORACLE_OK;
}

// Merge, src/DAGCompression.cu:1109-1163: merged sorted union of two ascending
// unique key arrays, A before B on ties; returns A->merged and B->merged maps.
void merge_keys(const std::vector<uint64_t>& a, const std::vector<uint64_t>& b,
                std::vector<uint64_t>& merged, std::vector<uint32_t>& map_a,
                std::vector<uint32_t>& map_b) {
    merged.clear();
    map_a.resize(a.size());
    map_b.resize(b.size());
    size_t i = 0, j = 0;
    while (i < a.size() || j < b.size()) {
        const bool take_a = j == b.size() || (i < a.size() && a[i] <= b[j]);
        const uint64_t k = take_a ? a[i] : b[j];
        if (merged.empty() || merged.back() != k) merged.push_back(k);
        if (take_a) map_a[i++] = (uint32_t)(merged.size() - 1);
        else map_b[j++] = (uint32_t)(merged.size() - 1);
    }
}

bool dag_empty(const Dag& d) { return d.leaves.empty(); }

// MergeDAGs(Pool, A, B), src/DAGCompression.cu:1165-1320.
int merge_pair(Dag& a, Dag& b, Dag& out) {
    if (a.levels.size() != b.levels.size()) return ORACLE_ERR_INVALID_ARGUMENT;
    if (dag_empty(a)) { out = std::move(b); return ORACLE_OK; }  // :1174-1178
    if (dag_empty(b)) { out = std::move(a); return ORACLE_OK; }  // :1179-1183
    Dag m;
    m.levels.resize(a.levels.size());
    std::vector<uint32_t> prev_a, prev_b, cur_a, cur_b;
    merge_keys(a.leaves, b.leaves, m.leaves, prev_a, prev_b);  // :1195-1217
    for (int l = (int)a.levels.size() - 1; l >= 0; --l) {     // :1224-1314
        const Level& la = a.levels[l];
        const Level& lb = b.levels[l];
        Level& lm = m.levels[l];
        merge_keys(la.hashes, lb.hashes, lm.hashes, cur_a, cur_b);
        const size_t u = lm.hashes.size();
        lm.masks.assign(u, 0);
        lm.children.assign(u * 8, kEmpty);
        std::vector<uint8_t> written(u, 0);
        auto put = [&](const Level& src, size_t i, const std::vector<uint32_t>& cur,
                       const std::vector<uint32_t>& prev) -> bool {
            const uint32_t t = cur[i];
            uint32_t ch[8];
            for (int c = 0; c < 8; ++c) {
                const uint32_t idx = src.children[i * 8 + c];
                ch[c] = idx == kEmpty ? kEmpty : prev[idx];
            }
            if (written[t]) {
                // Equal hashes from both sides must carry equal nodes.
                return lm.masks[t] == src.masks[i] &&
                       std::memcmp(&lm.children[(size_t)t * 8], ch, 32) == 0;
            }
            written[t] = 1;
            lm.masks[t] = src.masks[i];
            std::memcpy(&lm.children[(size_t)t * 8], ch, 32);
            return true;
        };
        for (size_t i = 0; i < la.size(); ++i)
            if (!put(la, i, cur_a, prev_a)) return ORACLE_ERR_HASH_COLLISION;
        for (size_t i = 0; i < lb.size(); ++i)
            if (!put(lb, i, cur_b, prev_b)) return ORACLE_ERR_HASH_COLLISION;
        prev_a.swap(cur_a);
        prev_b.swap(cur_b);
    }
    out = std::move(m);
    return ORACLE_OK;
}

// DAGCompression::MergeDAGs, src/DAGCompression.cu:1446-1548. Inputs are
// sub-DAGs in Morton order; their count must be 8^k (:1451, :1467).
int merge_dags(std::vector<Dag>& dags, Dag& out) {
    if (dags.empty()) return ORACLE_ERR_INVALID_ARGUMENT;
    uint64_t k = dags.size();
    while (k > 1) {
        if (k % 8) return ORACLE_ERR_INVALID_ARGUMENT;
        k /= 8;
    }
    const size_t num_levels = dags[0].levels.size();
    for (auto& d : dags)
        if (d.levels.size() != num_levels) return ORACLE_ERR_INVALID_ARGUMENT;
    while (dags.size() > 1) {
        std::vector<Dag> next(dags.size() / 8);
        for (size_t g = 0; g < next.size(); ++g) {
            uint64_t root_hashes[8];
            for (int i = 0; i < 8; ++i) {
                const Dag& d = dags[8 * g + i];
                root_hashes[i] = d.levels.empty() ? (d.leaves.empty() ? 0 : d.leaves[0])
                                 : (d.levels[0].hashes.empty() ? 0 : d.levels[0].hashes[0]);
            }
            Dag merged = std::move(dags[8 * g]);
            for (int i = 1; i < 8; ++i) {
                Dag m;
                int st = merge_pair(merged, dags[8 * g + i], m);
                if (st) return st;
                merged = std::move(m);
            }
            // New root over the 8 sub-roots (:1504-1533).
            Level top;
            uint8_t mask = 0;
            uint32_t ch[8];
            const std::vector<uint64_t>& top_hashes =
                merged.levels.empty() ? merged.leaves : merged.levels[0].hashes;
            for (int i = 0; i < 8; ++i) {
                if (root_hashes[i] == 0) { ch[i] = kEmpty; continue; }
                mask |= (uint8_t)(1u << i);
                auto it = std::lower_bound(top_hashes.begin(), top_hashes.end(), root_hashes[i]);
                if (it == top_hashes.end() || *it != root_hashes[i]) return ORACLE_ERR_BAD_INPUT;
                ch[i] = (uint32_t)(it - top_hashes.begin());
            }
            if (mask) {
                top.masks.push_back(mask);
                top.children.assign(ch, ch + 8);
                top.hashes.push_back(hash_children(root_hashes));
            }
            merged.levels.insert(merged.levels.begin(), std::move(top));
            next[g] = std::move(merged);
        }
        dags = std::move(next);
    }
    out = std::move(dags[0]);
    return ORACLE_OK;
}

// CreateFinalDAG, src/DAGCompression.cu:1550-1610, with ComputeChildPositions
// (:834-844), WriteTo (:845-861) and Utils::TotalSize / ChildOffset
// (src/Utils.h:68-75). An empty DAG yields 0 words (the reference asserts).
int final_dag(const Dag& d, std::vector<uint32_t>& words) {
    words.clear();
    if (d.leaves.empty()) return ORACLE_OK;
    const size_t nl = d.levels.size();
    std::vector<std::vector<uint32_t>> pos(nl);
    std::vector<uint64_t> start(nl + 1, 0);
    for (size_t l = 0; l < nl; ++l) {
        const Level& L = d.levels[l];
        pos[l].resize(L.size());
        uint64_t s = 0;
        for (size_t i = 0; i < L.size(); ++i) { pos[l][i] = (uint32_t)s; s += popc8(L.masks[i]) + 1; }
        start[l + 1] = start[l] + s;
    }
    const uint64_t total = start[nl] + 2 * (uint64_t)d.leaves.size();
    if (total >= (1ull << 32)) return ORACLE_ERR_TOO_LARGE;
    words.assign(total, 0xFFFFFFFFu);
    for (size_t l = 0; l < nl; ++l) {
        const Level& L = d.levels[l];
        const uint64_t next_start = start[l + 1];
        for (size_t i = 0; i < L.size(); ++i) {
            const uint64_t at = start[l] + pos[l][i];
            const uint32_t mask = L.masks[i];
            words[at] = mask;
            for (uint32_t c = 0; c < 8; ++c) {
                const uint32_t idx = L.children[i * 8 + c];
                if (idx == kEmpty) continue;
                const uint64_t ptr = (l + 1 == nl) ? next_start + 2ull * idx
                                                   : next_start + pos[l + 1][idx];
                words[at + child_offset(mask, c)] = (uint32_t)ptr;
            }
        }
    }
    const uint64_t leaf_at = start[nl];
    for (size_t i = 0; i < d.leaves.size(); ++i) {
        words[leaf_at + 2 * i + 0] = (uint32_t)(d.leaves[i] & 0xFFFFFFFFu);
        words[leaf_at + 2 * i + 1] = (uint32_t)(d.leaves[i] >> 32);
    }
    return ORACLE_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI for the Python test harness (ctypes).
// ---------------------------------------------------------------------------
extern "C" {

struct oracle_dag { Dag d; };

uint64_t oracle_hash_children(const uint64_t* h8) { return hash_children(h8); }

oracle_dag* oracle_create(const uint64_t* codes, uint64_t n, int depth, int threads, int* status) {
    auto* o = new oracle_dag;
    const int st = create_dag(codes, n, depth, threads, o->d);
    if (status) *status = st;
    if (st) { delete o; return nullptr; }
    return o;
}

oracle_dag* oracle_empty(int depth) {
    if (depth < 2) return nullptr;
    auto* o = new oracle_dag;
    o->d.levels.assign(depth - 2, Level{});
    return o;
}

// Builds a DAG from flat arrays: level l occupies nodes [offsets[l], offsets[l+1]).
oracle_dag* oracle_from_arrays(int num_levels, const uint64_t* offsets, const uint8_t* masks,
                               const uint32_t* children, const uint64_t* hashes,
                               const uint64_t* leaves, uint64_t num_leaves) {
    auto* o = new oracle_dag;
    o->d.levels.resize(num_levels);
    for (int l = 0; l < num_levels; ++l) {
        const uint64_t a = offsets[l], b = offsets[l + 1];
        Level& L = o->d.levels[l];
        L.masks.assign(masks + a, masks + b);
        L.children.assign(children + 8 * a, children + 8 * b);
        L.hashes.assign(hashes + a, hashes + b);
    }
    o->d.leaves.assign(leaves, leaves + num_leaves);
    return o;
}

// Merges k DAGs (8^k of them, Morton order). The inputs are left intact.
oracle_dag* oracle_merge(oracle_dag* const* dags, uint64_t k, int* status) {
    std::vector<Dag> v;
    v.reserve(k);
    for (uint64_t i = 0; i < k; ++i) v.push_back(dags[i]->d);
    auto* o = new oracle_dag;
    const int st = merge_dags(v, o->d);
    if (status) *status = st;
    if (st) { delete o; return nullptr; }
    return o;
}

void oracle_free(oracle_dag* o) { delete o; }

int oracle_num_levels(const oracle_dag* o) { return (int)o->d.levels.size(); }
uint64_t oracle_level_size(const oracle_dag* o, int l) { return o->d.levels[l].size(); }
uint64_t oracle_num_leaves(const oracle_dag* o) { return o->d.leaves.size(); }

void oracle_level_copy(const oracle_dag* o, int l, uint8_t* masks, uint32_t* children, uint64_t* hashes) {
    const Level& L = o->d.levels[l];
    if (masks) std::memcpy(masks, L.masks.data(), L.masks.size());
    if (children) std::memcpy(children, L.children.data(), L.children.size() * 4);
    if (hashes) std::memcpy(hashes, L.hashes.data(), L.hashes.size() * 8);
}

void oracle_leaves_copy(const oracle_dag* o, uint64_t* leaves) {
    std::memcpy(leaves, o->d.leaves.data(), o->d.leaves.size() * 8);
}

// Final layout. Call with out == nullptr to get the word count.
int oracle_final(const oracle_dag* o, uint32_t* out, uint64_t cap, uint64_t* n_words) {
    std::vector<uint32_t> w;
    const int st = final_dag(o->d, w);
    if (st) return st;
    if (n_words) *n_words = w.size();
    if (out) {
        if (cap < w.size()) return ORACLE_ERR_INVALID_ARGUMENT;
        std::memcpy(out, w.data(), w.size() * 4);
    }
    return ORACLE_OK;
}

// Sort helper exposed for tests of the baseline radix sort.
void oracle_radix_sort_keys(uint64_t* keys, uint64_t n, int lo_bit, int hi_bit, int threads) {
    std::vector<uint64_t> k(keys, keys + n);
    radix_sort(k, nullptr, lo_bit, hi_bit, threads);
    std::memcpy(keys, k.data(), n * 8);
}

}  // extern "C"
