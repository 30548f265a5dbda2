// dagc host orchestration and C ABI (include/dagc.h).
//
// Host code is C++ and reaches the GPU only through the kernel launchers of
// dagc_kernels.h. The pipelines keep every count on the device: a call
// enqueues its whole kernel sequence, then reads the counts back once.
//
// Reference mapping (src/DAGCompression.cu of Phyronnaz/DAG_Compression_Fast):
//   create_dag        <- DAGCompression::CreateDAG          :1003-1107
//   merge_dags        <- DAGCompression::MergeDAGs          :1446-1548 (+ :1109-1320)
//   final_dag         <- DAGCompression::CreateFinalDAG     :1550-1610
//   DevicePool        <- FPool :32-269 / FMemory (src/Memory.cpp:42-98)

#include "../../include/dagc.h"
#include "dagc_hash.h"
#include "dagc_kernels.h"
#include "dagc_launch.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <dlfcn.h>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

namespace dagc {
namespace {

constexpr int kMaxDepth = 21;
constexpr uint64_t kMaxFragments = (1ull << 31) - 2;  // digit counts + 1 in the sort's 31-bit status
constexpr int kMaxSorts = 48;
constexpr int kMaxTileCounters = 1024;

// Device-count slots of one call.
enum : int {
    kCntFragments = 0,
    kCntBricks = 1,
    kCntLeaves = 2,
    kCntNodes = 3,                 // + level
    kCntUnique = 3 + kMaxDepth,    // + level
    kCntSlots = 3 + 2 * kMaxDepth + 1,
    kCntOverflow = 63,             // fragments the grouping spilled past their partition's slab
};

struct CallHeader {
    uint32_t err;
    uint32_t pad;
    uint64_t counts[64];
    uint32_t tile_counters[kMaxTileCounters];
    uint32_t hist[kMaxSorts][kSortHistWords];
    DedupState dedup[kMaxDepth + 1];  // leaves + one per level
    uint32_t sketch[kGroupSketchRegs];  // distinct-brick sketch of the fragment grouping's probe
    uint32_t gover[kGroupMaxParts];     // its partitions that spilled past their slabs
    uint64_t gcursor[kGroupMaxParts];   // its partition starts, then ends
    uint32_t path[4];                   // [0] 1: fragments grouped by hash, 0: sorted; [1], [2] its shape
    uint32_t leaf_sorted;               // 1: the distinct leaf masks were sorted by one CTA in shared memory
    uint32_t pad1;
};
static_assert(kCntSlots <= kCntOverflow, "count slots");

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Device allocations of a context go through here: a test hook can make the
// next `inject` of them fail as cudaMalloc does when the device is full
// (cudaErrorMemoryAllocation), without touching the device.
struct AllocStats {
    int inject = 0;             // allocations still to fail (test hook)
    uint64_t failures = 0;      // failed attempts, injected or real
    uint64_t retries_ok = 0;    // allocations that succeeded on their retry
};
inline cudaError_t dev_malloc(void** p, size_t bytes, AllocStats* st) {
    if (st && st->inject > 0) {
        --st->inject;
        ++st->failures;
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    const cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess && st) ++st->failures;
    return e;
}

// Best-fit cache of device blocks (the reference's FPool): freed blocks are
// kept and reused; on cudaMalloc failure the cache is released and the
// allocation retried once (the OOM fallback of src/Memory.cpp:56-70).
class DevicePool {
public:
    AllocStats* stats = nullptr;
    ~DevicePool() {
        trim();
        for (cudaEvent_t e : spare_events_) cudaEventDestroy(e);
    }
    cudaError_t alloc(void** p, size_t bytes, const char* name = "block") {
        reclaim();
        bytes = align_up(std::max<size_t>(bytes, 1), 512);
        auto it = free_.lower_bound(bytes);
        if (it != free_.end() && it->first <= 2 * bytes + (4u << 20)) {
            *p = it->second;
            live_[*p] = {it->first, name};
            cached_ -= it->first;
            in_use_ += it->first;
            free_.erase(it);
            peak_ = std::max(peak_, in_use_);
            return cudaSuccess;
        }
        cudaError_t e = dev_malloc(p, bytes, stats);
        if (e == cudaErrorMemoryAllocation) {
            cudaGetLastError();
            trim();
            e = dev_malloc(p, bytes, stats);
            if (e == cudaSuccess && stats) ++stats->retries_ok;
        }
        if (e != cudaSuccess) { cudaGetLastError(); *p = nullptr; return e; }
        live_[*p] = {bytes, name};
        in_use_ += bytes;
        peak_ = std::max(peak_, in_use_);
        return cudaSuccess;
    }
    void release(void* p) {
        if (!p) return;
        auto it = live_.find(p);
        if (it == live_.end()) return;
        free_.emplace(it->second.first, p);
        cached_ += it->second.first;
        in_use_ -= it->second.first;
        live_.erase(it);
    }
    // Bytes and block count of the live blocks by name, and of the cache.
    void tally(std::map<std::string, std::pair<uint64_t, uint64_t>>& m) const {
        for (const auto& kv : live_) {
            auto& e = m[kv.second.second];
            e.first += kv.second.first;
            ++e.second;
        }
        for (const auto& kv : free_) {
            auto& e = m["cached for reuse"];
            e.first += kv.first;
            ++e.second;
        }
    }
    // Returns a block once the work queued on `s` so far has completed (work
    // that may still read it): an event is recorded on `s` and the block is
    // handed out again only after the event has completed.
    void release_after(void* p, cudaStream_t s) {
        if (!p || live_.find(p) == live_.end()) return;
        cudaEvent_t e = nullptr;
        if (!spare_events_.empty()) {
            e = spare_events_.back();
            spare_events_.pop_back();
        } else if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            e = nullptr;
        }
        if (!e || cudaEventRecord(e, s) != cudaSuccess) {
            cudaGetLastError();
            if (e) spare_events_.push_back(e);
            cudaStreamSynchronize(s);
            cudaGetLastError();
            release(p);
            return;
        }
        deferred_.push_back({p, e});
    }
    // Moves deferred blocks whose event has completed to the free cache.
    void reclaim() {
        for (size_t i = 0; i < deferred_.size();) {
            const cudaError_t q = cudaEventQuery(deferred_[i].e);
            if (q == cudaErrorNotReady) {
                cudaGetLastError();
                ++i;
                continue;
            }
            if (q != cudaSuccess) cudaGetLastError();
            release(deferred_[i].p);
            spare_events_.push_back(deferred_[i].e);
            deferred_[i] = deferred_.back();
            deferred_.pop_back();
        }
    }
    void trim() {
        for (const Deferred& d : deferred_) {
            cudaEventSynchronize(d.e);
            release(d.p);
            spare_events_.push_back(d.e);
        }
        cudaGetLastError();
        deferred_.clear();
        for (auto& kv : free_) cudaFree(kv.second);
        free_.clear();
        cached_ = 0;
    }
    size_t in_use() const { return in_use_; }
    size_t peak() const { return peak_; }
    size_t cached() const { return cached_; }

private:
    struct Deferred {
        void* p;
        cudaEvent_t e;
    };
    std::multimap<size_t, void*> free_;
    std::unordered_map<void*, std::pair<size_t, const char*>> live_;
    std::vector<Deferred> deferred_;
    std::vector<cudaEvent_t> spare_events_;
    size_t in_use_ = 0, cached_ = 0, peak_ = 0;
};

// One growable scratch block; every call lays its buffers out from offset 0.
struct Arena {
    void* base = nullptr;
    size_t cap = 0;
    AllocStats* stats = nullptr;
    // Grows to at least `bytes` (with 25% headroom; without it when that
    // does not fit).
    cudaError_t reserve(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (base) cudaFree(base);
        base = nullptr;
        cap = 0;
        const size_t want = align_up(bytes + bytes / 4, 1u << 21);
        cudaError_t e = dev_malloc(&base, want, stats);
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = dev_malloc(&base, align_up(bytes, 1u << 21), stats);
            if (e != cudaSuccess) { cudaGetLastError(); base = nullptr; return e; }
            if (stats) ++stats->retries_ok;
            cap = align_up(bytes, 1u << 21);
            return cudaSuccess;
        }
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (base) cudaFree(base);
        base = nullptr;
        cap = 0;
    }
};

struct Layout {
    size_t off = 0;
    template <typename T>
    size_t take(uint64_t count) {
        off = align_up(off, 256);
        const size_t o = off;
        off += (size_t)count * sizeof(T);
        return o;
    }
};

}  // namespace
}  // namespace dagc

using namespace dagc;

struct StageStats {
    double ms = 0;
    uint64_t launches = 0;
    uint64_t bytes = 0;
};

struct PendingTiming {
    int stage;
    cudaEvent_t a, b;
    uint64_t launches;
    uint64_t bytes;
};

// A digit-pass plan: kernel shape and widest digit.
struct SortChoice {
    int shape;
    int radix_bits;
};
// Class of a sort for the tuning table: keys-only or pairs, number of sorted
// bits, and the key count's power of two (counts within a factor of two
// share a plan).
inline uint32_t sort_class(bool with_values, int bits, uint64_t n) {
    int lg = 0;
    while (lg < 40 && (1ull << (lg + 1)) <= n) ++lg;
    return (with_values ? 1u << 24 : 0u) | (uint32_t)bits << 8 | (uint32_t)lg;
}

// A recorded CreateDAG pipeline: valid for one input pointer, size, depth,
// arena block and pass shapes.
struct GraphKey {
    const void* frag;
    uint64_t n;
    int depth;
    void* arena;
    uint32_t chunks;   // batched calls: number of chunks (0 otherwise)
    int chunk_depth;   // batched calls: chunk depth, which sets the composite key split (0 otherwise)
    bool chunk_path;   // batched calls: persistent per-chunk leaves
    bool dedup;        // hash-set dedup (else radix sort + unique) for the leaves and levels
    void* table;       // the dedup table block
    int group;         // fragment grouping mode
    bool operator==(const GraphKey& o) const {
        return frag == o.frag && n == o.n && depth == o.depth && arena == o.arena && chunks == o.chunks &&
               chunk_depth == o.chunk_depth && chunk_path == o.chunk_path && dedup == o.dedup && table == o.table &&
               group == o.group;
    }
};
struct GraphEntry {
    GraphKey key;
    uint32_t tune_version;
    cudaGraphExec_t exec;
    uint64_t launches;
};

struct dagc_context_t {
    int device = 0;
    bool profiling = false;
    bool use_graphs = true;
    cudaStream_t capture_stream = nullptr;
    std::vector<GraphEntry> graphs;
    std::vector<GraphKey> graph_seen;  // call shapes launched directly once; recorded when seen again
    // Digit-pass plans. A forced shape / width (dagc_set_option, >= 0)
    // applies to every sort of its kind; otherwise the tuning table picks per
    // sort class (SortClass), falling back to the defaults.
    int shape_keys = -1, shape_pairs = -1, radix_keys = -1;
    std::map<uint32_t, SortChoice> tune;  // sort_class key -> measured best plan
    std::map<uint32_t, std::pair<double, double>> tune_ms;  // its time and the default plan's (ms)
    const SortChoice* plan_override = nullptr;  // the autotuner's candidate while it is timed
    uint32_t* sort_err = nullptr;               // error word of the last standalone sort
    std::string tune_file;                      // the file the table was loaded from at creation
    uint32_t tune_version = 0;            // bumped on every change of the table or a forced plan
    int occ_keys[kNumKeyShapes][kMaxRadixBits - kRadixBits + 1] = {}, occ_pairs[kNumPairShapes] = {};
    StageStats stages[DAGC_NUM_STAGES];
    std::vector<cudaEvent_t> free_events;
    std::vector<PendingTiming> pending;
    uint64_t launches = 0;
    int sms = 152;
    int grid_hist = 0, grid_pass_kv = 0, grid_pass_k = 0;
    int grid_leaf = 0, grid_extract = 0, grid_unique = 0, grid_scan = 0, grid_write = 0;
    AllocStats alloc_stats;
    DevicePool pool;
    Arena arena;
    uint32_t test_spin_limit = 0;  // DAGC_OPT_TEST_SPIN_LIMIT (0: kSpinLimit)
    int test_stall = 0;            // DAGC_OPT_TEST_STALL_LOOKBACK
    // Dedup table: keys (0 = empty), then aux words; every level leaves its
    // keys zero; after a call that stopped early it is cleared. Grouping
    // scratch (kGroupScratchBytes): the brick masks.
    bool use_dedup = true;
    int group_mode = 1;  // DAGC_OPT_GROUP
    int batch_path = 1;  // DAGC_OPT_BATCH_PATH
    std::vector<uint32_t> ck_tile_host;  // chunk path: first tile of each chunk (host copy for the upload)
    bool pdl = false;    // DAGC_OPT_PDL
    uint64_t dedup_unique_limit = kDedupMaxUnique;  // lowered only to exercise the rerun
    void* table = nullptr;
    void* gtable = nullptr;  // fragment grouping scratch
    uint64_t table_cap = 0;  // slots (table_size_for of the largest item count so far)
    bool table_dirty = true;
    uint64_t fallbacks = 0;  // calls rerun with the radix form
    uint32_t* trace_err = nullptr;  // tracer error word
    void* vox_scratch = nullptr;    // voxelizer counters and look-back status
    size_t vox_scratch_bytes = 0;
    std::string last_error;
    std::vector<uint64_t> last_counts;
    uint64_t* h_stage = nullptr;  // pinned: counts + error word read back
    // CreateDAG returns while its DAG is still being copied out of the arena:
    // the next call that writes the arena waits for this event first.
    cudaEvent_t arena_copy = nullptr;
    bool arena_copy_pending = false;
    std::vector<cudaEvent_t> free_sync_events;  // DAG readiness events, reused
    std::mutex mu;
};

struct dagc_dag_t {
    dagc_context ctx = nullptr;
    int num_levels = 0;
    std::vector<uint64_t> level_offset;  // num_levels + 1 (nodes, concatenated, root level first)
    uint64_t num_leaves = 0;
    void* block = nullptr;
    uint64_t* hashes = nullptr;
    uint32_t* children = nullptr;
    uint8_t* masks = nullptr;
    uint64_t* leaves = nullptr;
    uint64_t* d_level_offset = nullptr;
    // Recorded after the kernel that fills the block, when the call that made
    // the DAG returned before that kernel finished (CreateDAG); null when the
    // block was complete on return.
    cudaEvent_t ready = nullptr;
    uint64_t num_nodes() const { return level_offset.empty() ? 0 : level_offset.back(); }
};

namespace {

int set_error(dagc_context ctx, int status, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return status;
}

int cuda_status(cudaError_t e) {
    return e == cudaErrorMemoryAllocation ? DAGC_ERR_OUT_OF_MEMORY : DAGC_ERR_CUDA;
}

#define DAGC_CUDA(ctx, expr)                                                                      \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            cudaGetLastError();                                                                   \
            return set_error(ctx, cuda_status(e_), std::string(#expr) + ": " + cudaGetErrorString(e_)); \
        }                                                                                         \
    } while (0)

#define DAGC_LAUNCHED(ctx) DAGC_CUDA(ctx, cudaGetLastError())

cudaEvent_t take_event(dagc_context ctx) {
    if (!ctx->free_events.empty()) {
        cudaEvent_t e = ctx->free_events.back();
        ctx->free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return e;
}

cudaEvent_t take_sync_event(dagc_context ctx) {
    if (!ctx->free_sync_events.empty()) {
        cudaEvent_t e = ctx->free_sync_events.back();
        ctx->free_sync_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return e;
}

// Work on stream `s` that reads DAG `d` waits until its block is complete.
void dag_ready_wait(dagc_dag d, cudaStream_t s) {
    if (d && d->ready) cudaStreamWaitEvent(s, d->ready, 0);
}
// The host waits until DAG `d`'s block is complete.
void dag_ready_sync(dagc_dag d) {
    if (d && d->ready) cudaEventSynchronize(d->ready);
}
// Work on stream `s` that writes the context's arena waits for the last copy
// out of it.
void arena_wait(dagc_context ctx, cudaStream_t s) {
    if (ctx->arena_copy_pending) cudaStreamWaitEvent(s, ctx->arena_copy, 0);
}

// Brackets the launches of one stage with events on the call's stream when
// profiling is on; bytes may be filled in later (see settle_bytes).
struct StageTimer {
    dagc_context ctx;
    int stage;
    cudaStream_t s;
    cudaEvent_t a = nullptr;
    uint64_t launches0 = 0;
    // stage < 0 disables the timer.
    StageTimer(dagc_context c, int st, cudaStream_t stream) : ctx(c), stage(st), s(stream) {
        launches0 = ctx->launches;
        if (st >= 0 && ctx->profiling && (a = take_event(ctx))) cudaEventRecord(a, s);
    }
    void stop(uint64_t bytes = 0) {
        if (!a) return;
        cudaEvent_t b = take_event(ctx);
        if (!b) { ctx->free_events.push_back(a); a = nullptr; return; }
        cudaEventRecord(b, s);
        ctx->pending.push_back({stage, a, b, ctx->launches - launches0, bytes});
        a = nullptr;
    }
};

// Fills in the algorithmic bytes of pending timings of `stage` recorded
// without them (their sizes were only known on the device at launch time).
void set_pending_bytes(dagc_context ctx, int stage, uint64_t bytes) {
    for (PendingTiming& p : ctx->pending)
        if (p.stage == stage && p.bytes == 0) p.bytes = bytes;
}

// Sets the algorithmic bytes of every pending timing of `stage` (used for the
// kernels of the path the device did not take: they ran and returned at once,
// so they moved nothing).
void override_pending_bytes(dagc_context ctx, int stage, uint64_t bytes) {
    for (PendingTiming& p : ctx->pending)
        if (p.stage == stage) p.bytes = bytes;
}

// Called after a stream synchronisation: folds the finished event pairs into
// the per-stage totals.
void settle_profile(dagc_context ctx) {
    for (const PendingTiming& p : ctx->pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            StageStats& st = ctx->stages[p.stage];
            st.ms += ms;
            st.launches += p.launches;
            st.bytes += p.bytes;
        } else {
            cudaGetLastError();
        }
        ctx->free_events.push_back(p.a);
        ctx->free_events.push_back(p.b);
    }
    ctx->pending.clear();
}

int grid_for(int per_sm, int sms, uint64_t tiles) {
    const uint64_t g = (uint64_t)std::max(per_sm, 1) * (uint64_t)sms;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, std::max<uint64_t>(tiles, 1)));
}

int device_error_status(uint32_t err, std::string& msg) {
    if (err & kErrTimeout) { msg = "a bounded device wait ran out"; return DAGC_ERR_DEVICE_TIMEOUT; }
    if (err & kErrBadInput) { msg = "fragment code out of range for the depth, or malformed DAG"; return DAGC_ERR_BAD_INPUT; }
    if (err & kErrCollision) { msg = "64-bit node hash collision between different nodes"; return DAGC_ERR_HASH_COLLISION; }
    if (err & kErrCapacity) { msg = "internal capacity bound exceeded"; return DAGC_ERR_CUDA; }
    if (err & kErrNotRooted) { msg = "level 0 does not hold exactly one node"; return DAGC_ERR_BAD_INPUT; }
    if (err & kErrMergeRoot) { msg = "sub-DAG root missing from merged level"; return DAGC_ERR_BAD_INPUT; }
    return DAGC_OK;
}

// Per-call scratch slots inside the zeroed header.
// Each single-value look-back launch gets its own zeroed status region sized
// for its tile bound; the regions are carved in launch order.
struct CallSlots {
    CallHeader* h;
    int next_counter = 0, next_hist = 0, next_dedup = 0;
    uint64_t* sv_next = nullptr;
    uint64_t* sv_end = nullptr;
    uint32_t* counter() { return &h->tile_counters[next_counter++]; }
    uint32_t* counters(int k) { uint32_t* p = &h->tile_counters[next_counter]; next_counter += k; return p; }
    uint32_t* hist() { return h->hist[next_hist++]; }
    DedupState* dedup() { return &h->dedup[next_dedup++]; }
    uint64_t* sv(uint64_t n_bound) {
        uint64_t* p = sv_next;
        sv_next += scan_tiles(n_bound) + 1;
        return sv_next <= sv_end ? p : nullptr;
    }
    uint64_t* count(int slot) { return &h->counts[slot]; }
};
inline uint64_t sv_words(uint64_t n_bound) { return scan_tiles(n_bound) + 1; }

struct SortBuffers {
    uint32_t* status[2];
};

struct SegmentSpec {
    const uint64_t* d_offsets;
    uint32_t count;
    int shift;
};

// Default plans, measured on GB300: keys-only sorts take 16 keys per thread,
// 3 CTAs per SM, alternating matchers; key/value sorts 8 items, 4 CTAs, ballots.
constexpr SortChoice kDefaultKeys{0, kRadixBits};
constexpr SortChoice kDefaultPairs{3, kRadixBits};

// The plan of one sort: forced options first, then the tuning table, then
// the defaults; a plan that cannot take the bit range falls back to 8-bit
// digits.
SortChoice sort_plan_for(dagc_context ctx, bool with_values, int lo, int hi, uint64_t n) {
    if (ctx->plan_override) return *ctx->plan_override;
    SortChoice c = with_values ? kDefaultPairs : kDefaultKeys;
    auto it = ctx->tune.find(sort_class(with_values, hi - lo, n));
    if (it != ctx->tune.end()) c = it->second;
    const int forced_shape = with_values ? ctx->shape_pairs : ctx->shape_keys;
    if (forced_shape >= 0) c.shape = forced_shape;
    if (!with_values && ctx->radix_keys >= 0) c.radix_bits = ctx->radix_keys;
    if (!sort_plan_valid(c.shape, with_values, c.radix_bits, lo, hi)) c.radix_bits = kRadixBits;
    if (!sort_plan_valid(c.shape, with_values, c.radix_bits, lo, hi)) c = with_values ? kDefaultPairs : kDefaultKeys;
    return c;
}

// pass_stage >= 0: time the histogram under hist_stage and every digit pass
// separately under pass_stage (host-known n only, for the byte counts).
int run_sort(dagc_context ctx, CallSlots& cs, const SortBuffers& sb, const uint64_t* keys_in,
             uint64_t* keys_out, uint64_t* keys_alt, const uint32_t* vals_in, uint32_t* vals_out,
             uint32_t* vals_alt, bool with_values, uint64_t n_bound, const uint64_t* d_n, int lo, int hi,
             int validate_bits, cudaStream_t s, int hist_stage = -1, int pass_stage = -1,
             const SegmentSpec* seg = nullptr, const uint32_t* gate = nullptr, uint32_t gate_run = 0) {
    t_pdl = ctx->pdl;
    if (cs.next_hist >= kMaxSorts || cs.next_counter + kMaxPasses > kMaxTileCounters)
        return set_error(ctx, DAGC_ERR_TOO_LARGE, "too many sorts in one call");
    SortArgs a{};
    a.keys_in = keys_in;
    a.keys_out = keys_out;
    a.keys_alt = keys_alt;
    a.vals_in = vals_in;
    a.vals_out = vals_out;
    a.vals_alt = vals_alt;
    a.with_values = with_values;
    a.n = n_bound;
    a.d_n = d_n;
    a.lo_bit = lo;
    a.hi_bit = hi;
    a.validate_bits = validate_bits;
    a.hist = cs.hist();
    a.status[0] = sb.status[0];
    a.status[1] = sb.status[1];
    a.tile_counters = cs.counters(kMaxPasses);
    a.err = &cs.h->err;
    a.spin_limit = ctx->test_spin_limit;
    a.stall_first_tile = ctx->test_stall;
    const uint64_t tiles = sort_tiles(n_bound);
    a.grid_hist = grid_for(ctx->grid_hist / std::max(ctx->sms, 1), ctx->sms, (n_bound + 4095) / 4096);
    const SortChoice plan = sort_plan_for(ctx, with_values, lo, hi, n_bound);
    a.shape = plan.shape;
    a.radix_bits = plan.radix_bits;
    a.gate = gate;
    a.gate_run = gate_run;
    if (seg && seg->d_offsets) {
        a.seg_offsets = seg->d_offsets;
        a.seg_count = seg->count;
        a.seg_shift = seg->shift;
    }
    // Grid: resident CTAs of the widest pass kernel (the narrower ones of
    // the same shape fit at least as many).
    const int occ = with_values ? ctx->occ_pairs[a.shape] : ctx->occ_keys[a.shape][a.radix_bits - kRadixBits];
    const uint64_t tile = 256ull * sort_shape_items(a.shape, with_values);
    const uint64_t shape_tiles = (n_bound + tile - 1) / tile;
    a.grid_pass = grid_for(occ, ctx->sms, std::min<uint64_t>(tiles, shape_tiles));
    const int passes = sort_plan_passes(a);
    const uint64_t kv = with_values ? 12 : 8;
    {
        StageTimer t(ctx, hist_stage, s);
        launch_sort_histogram(a, s);
        ctx->launches += passes == 0 ? 2 : 1;
        t.stop(d_n ? 0 : n_bound * 8);
    }
    DAGC_LAUNCHED(ctx);
    for (int i = 0; i < passes; ++i) {
        StageTimer t(ctx, pass_stage, s);
        launch_sort_pass(a, i, s);
        ++ctx->launches;
        t.stop(d_n ? 0 : 2 * kv * n_bound);
    }
    DAGC_LAUNCHED(ctx);
    return DAGC_OK;
}

int alloc_dag(dagc_context ctx, int num_levels, const std::vector<uint64_t>& level_sizes,
              uint64_t num_leaves, dagc_dag* out) {
    std::unique_ptr<dagc_dag_t> d(new dagc_dag_t);
    d->ctx = ctx;
    d->num_levels = num_levels;
    d->level_offset.assign(num_levels + 1, 0);
    for (int l = 0; l < num_levels; ++l) d->level_offset[l + 1] = d->level_offset[l] + level_sizes[l];
    d->num_leaves = num_leaves;
    const uint64_t nn = d->num_nodes();
    Layout L;
    const size_t o_h = L.take<uint64_t>(nn);
    const size_t o_c = L.take<uint32_t>(nn * 8);
    const size_t o_l = L.take<uint64_t>(num_leaves);
    const size_t o_o = L.take<uint64_t>(num_levels + 1);
    const size_t o_m = L.take<uint8_t>(nn);
    void* block = nullptr;
    DAGC_CUDA(ctx, ctx->pool.alloc(&block, L.off, "DAG (levels + leaves)"));
    char* b = static_cast<char*>(block);
    d->block = block;
    d->hashes = reinterpret_cast<uint64_t*>(b + o_h);
    d->children = reinterpret_cast<uint32_t*>(b + o_c);
    d->leaves = reinterpret_cast<uint64_t*>(b + o_l);
    d->d_level_offset = reinterpret_cast<uint64_t*>(b + o_o);
    d->masks = reinterpret_cast<uint8_t*>(b + o_m);
    *out = d.release();
    return DAGC_OK;
}

void free_dag(dagc_dag d) {
    if (!d) return;
    dag_ready_sync(d);  // the block returns to the pool only once nothing writes it
    if (d->ctx) {
        if (d->ready) d->ctx->free_sync_events.push_back(d->ready);
        d->ctx->pool.release(d->block);
    } else if (d->ready) {
        cudaEventDestroy(d->ready);
    }
    delete d;
}

uint64_t level_cap(int level, uint64_t n) {
    // A level-l node is identified by the top 3*l code bits: at most 8^l of them.
    if (3 * level >= 62) return n;
    return std::min<uint64_t>(n, 1ull << (3 * level));
}

void drop_graphs(dagc_context ctx) {
    for (GraphEntry& g : ctx->graphs) cudaGraphExecDestroy(g.exec);
    ctx->graphs.clear();
    ctx->graph_seen.clear();
}

// Runs `enqueue` (which puts one call's whole kernel sequence on a stream).
// With graphs on, a call shape's second call records the sequence on the
// context's own capture stream and later calls replay it on `s`, which removes
// the per-launch host cost (a shape's first call launches directly); with
// profiling on (events per stage) it is launched directly.
template <typename F>
int run_enqueue(dagc_context ctx, const GraphKey& key, cudaStream_t s, F&& enqueue) {
    if (!ctx->use_graphs || ctx->profiling || !ctx->capture_stream) return enqueue(s);
    for (GraphEntry& g : ctx->graphs) {
        if (g.key == key && g.tune_version == ctx->tune_version) {
            DAGC_CUDA(ctx, cudaGraphLaunch(g.exec, s));
            ctx->launches += g.launches;
            return DAGC_OK;
        }
    }
    // A call shape seen for the first time launches directly: recording and
    // instantiating a graph costs more than one direct launch sequence, and a
    // stream of requests of ever new sizes would pay that on every call. The
    // shape's second call records it.
    bool seen = false;
    for (size_t i = 0; i < ctx->graph_seen.size(); ++i) {
        if (ctx->graph_seen[i] == key) {
            ctx->graph_seen.erase(ctx->graph_seen.begin() + i);
            seen = true;
            break;
        }
    }
    if (!seen) {
        if (ctx->graph_seen.size() >= 16) ctx->graph_seen.erase(ctx->graph_seen.begin());
        ctx->graph_seen.push_back(key);
        return enqueue(s);
    }
    // Entries made for an arena block that has since been replaced are dead.
    for (size_t i = 0; i < ctx->graphs.size();) {
        if (ctx->graphs[i].key.arena != key.arena) {
            cudaGraphExecDestroy(ctx->graphs[i].exec);
            ctx->graphs.erase(ctx->graphs.begin() + i);
        } else {
            ++i;
        }
    }
    const uint64_t l0 = ctx->launches;
    DAGC_CUDA(ctx, cudaStreamBeginCapture(ctx->capture_stream, cudaStreamCaptureModeThreadLocal));
    const int st = enqueue(ctx->capture_stream);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->capture_stream, &graph);
    const uint64_t recorded = ctx->launches - l0;
    ctx->launches = l0;
    if (st != DAGC_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (st != DAGC_OK) return st;
        return enqueue(s);  // recording failed: launch directly
    }
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        cudaGetLastError();
        return enqueue(s);
    }
    if (ctx->graphs.size() >= 8) {
        cudaGraphExecDestroy(ctx->graphs.front().exec);
        ctx->graphs.erase(ctx->graphs.begin());
    }
    ctx->graphs.push_back({key, ctx->tune_version, exec, recorded});
    DAGC_CUDA(ctx, cudaGraphLaunch(exec, s));
    ctx->launches += recorded;
    return DAGC_OK;
}

// -------------------------------------------------------------- CreateDAG --
// Output of the device pipeline before materialisation: per-level unique
// arrays in the scratch pools (upper-bound strides) and the counts.
struct CreatePools {
    std::vector<uint64_t*> hashes;
    std::vector<uint32_t*> children;
    std::vector<uint8_t*> masks;
    uint64_t* leaves = nullptr;
    std::vector<uint64_t> unique;  // u_l
    uint64_t num_leaves = 0;
};

// Batched input (see dagc_create_batched): chunk offsets into the fragment
// array and each chunk's Morton index in the grid of chunks, host arrays.
struct BatchSpec {
    const uint64_t* h_offsets;  // k + 1
    const uint64_t* h_morton;   // k, ascending
    uint32_t k;
    int chunk_depth;
};

int bits_for(uint64_t values) {  // bits to tell `values` values apart
    int b = 0;
    while (b < 64 && (values - 1) >> b) ++b;
    return b;
}

// Scratch layout of one CreateDAG call (also used to report its footprint).
struct CreateLayout {
    std::vector<uint64_t> cap;  // node bound per level
    uint64_t capmax = 1, p0cap = 0, sv_total = 0;
    size_t zero_bytes = 0, total = 0;
    size_t o_hdr, o_sv, o_ss0, o_ss1, o_A, o_B, o_P, o_LM, o_SK, o_SKa, o_V, o_Va, o_M0, o_M1;
    size_t o_NC0, o_NC1, o_NM, o_NCH, o_NH, o_PL, o_lead_or, o_lead_run, o_seg_off, o_seg_code;
    // Fragment grouping (when `grouping`): the partition slabs.
    uint64_t group_slab_total = 0;
    float group_probe_max = 0.0f;
    size_t o_slab = 0, o_over = 0;
    std::vector<size_t> o_ph, o_pc, o_pm;
    // Hash-set dedup (when `dedup`): per-item slots, the unique list, buckets.
    bool dedup = false;
    uint64_t item_cap = 0, uniq_cap = 0, bucket_area = 0, table_slots = 0;
    size_t o_islot = 0, o_ukey = 0, o_ukey_alt = 0;
    size_t o_bcnt = 0, o_bent = 0;
    // Persistent per-chunk leaves (batched form): zeroed chunk state
    // (histograms, cursors, done counters, item counter), tile offsets, the
    // mask stage and per-item brick counts / offsets.
    uint32_t ck_bins = 0, ck_groups = 0;
    size_t o_ck_state = 0, ck_state_bytes = 0, o_ck_hist = 0, o_ck_cursor = 0, o_ck_done = 0, o_ck_work = 0;
    size_t o_ck_tile = 0, o_ck_mask = 0, o_ck_gb = 0, o_ck_gs = 0, o_ck_gd = 0;
    CreateLayout(uint64_t n, int depth, uint32_t k_batch, bool use_dedup, uint64_t unique_limit = kDedupMaxUnique,
                 bool grouping = false, int chunk_depth = 0) {
        const int nl = depth - 2;
        cap.resize(nl);
        for (int l = 0; l < nl; ++l) { cap[l] = level_cap(l, n); capmax = std::max(capmax, cap[l]); }
        p0cap = level_cap(depth - 2, n);
        sv_total = sv_words(n) + sv_words(p0cap);
        for (int l = nl - 1; l >= 0; --l) sv_total += sv_words(l == nl - 1 ? p0cap : cap[l + 1]) + sv_words(cap[l]);
        Layout L;
        o_hdr = L.take<CallHeader>(1);
        o_sv = L.take<uint64_t>(sv_total);
        zero_bytes = L.off;
        o_ss0 = L.take<uint32_t>(sort_status_words(n));
        o_ss1 = L.take<uint32_t>(sort_status_words(n));
        o_A = L.take<uint64_t>(n);
        o_B = L.take<uint64_t>(n);
        if (grouping) {
            group_shape(n, &group_slab_total, &group_probe_max);
            o_slab = L.take<uint64_t>(group_slab_total);
            o_over = L.take<uint64_t>(n);
        }
        o_P = L.take<uint64_t>(p0cap);
        o_LM = L.take<uint64_t>(p0cap);
        dedup = use_dedup;
        const uint64_t sort_cap = dedup ? 0 : p0cap;  // hash sorts of the radix form only
        o_SK = L.take<uint64_t>(sort_cap);
        o_SKa = L.take<uint64_t>(sort_cap);
        o_V = L.take<uint32_t>(sort_cap);
        o_Va = L.take<uint32_t>(sort_cap);
        if (dedup) {
            // Items per level are at most p0cap (leaves) or cap[l] <= p0cap.
            item_cap = std::min<uint64_t>(p0cap, kDedupMaxItems);
            uniq_cap = std::min<uint64_t>(p0cap, std::min<uint64_t>(unique_limit, kDedupMaxUnique));
            bucket_area = dedup_bucket_area(uniq_cap);
            table_slots = std::max(table_size_for(item_cap, true), table_size_for(item_cap, false));
            o_islot = L.take<uint32_t>(item_cap);
            o_ukey = L.take<uint64_t>(uniq_cap);
            // The other key buffer of the unique leaf masks' sort (the sorted
            // keys go out to the leaf array).
            o_ukey_alt = L.take<uint64_t>(uniq_cap);
            o_bcnt = L.take<uint32_t>(kDedupMaxBuckets);
            o_bent = L.take<uint4>(bucket_area);
        }
        o_M0 = L.take<uint32_t>(p0cap);
        o_M1 = L.take<uint32_t>(p0cap);
        o_NC0 = L.take<uint64_t>(capmax);
        o_NC1 = L.take<uint64_t>(capmax);
        o_NM = L.take<uint8_t>(capmax);
        o_NCH = L.take<uint32_t>(std::max<uint64_t>(capmax, kTailCap) * 8);
        o_NH = L.take<uint64_t>(capmax);
        o_PL = L.take<uint64_t>(p0cap);
        o_ph.resize(nl); o_pc.resize(nl); o_pm.resize(nl);
        for (int l = 0; l < nl; ++l) {
            o_ph[l] = L.take<uint64_t>(cap[l]);
            o_pc[l] = L.take<uint32_t>(cap[l] * 8);
            o_pm[l] = L.take<uint8_t>(cap[l]);
        }
        o_lead_or = L.take<uint64_t>(scan_tiles(n) + 1);
        o_lead_run = L.take<uint64_t>(scan_tiles(n) + 1);
        o_seg_off = L.take<uint64_t>(k_batch ? k_batch + 1 : 0);
        o_seg_code = L.take<uint64_t>(k_batch);
        if (chunk_depth > 0 && k_batch) {
            ck_bins = 1u << chunk_bin_bits(chunk_depth);
            ck_groups = (ck_bins + kChunkGroupBins - 1) / kChunkGroupBins;
            o_ck_hist = L.take<uint32_t>((uint64_t)k_batch * ck_bins);
            o_ck_state = o_ck_hist;
            o_ck_cursor = L.take<uint32_t>((uint64_t)k_batch * ck_bins);
            o_ck_done = L.take<uint32_t>(2ull * k_batch);
            o_ck_work = L.take<uint32_t>(1);
            ck_state_bytes = L.off - o_ck_state;
            o_ck_tile = L.take<uint32_t>(k_batch + 1ull);
            o_ck_mask = L.take<uint64_t>(n);
            o_ck_gb = L.take<uint32_t>((uint64_t)k_batch * ck_groups);
            o_ck_gs = L.take<uint64_t>((uint64_t)k_batch * ck_groups);
            o_ck_gd = L.take<uint32_t>((uint64_t)k_batch * ck_groups);
        }
        total = L.off;
    }
};

// Grows the context's dedup table to `slots` (zeroed); clears it after a call
// that may have stopped between an insert and its map.
int reserve_table(dagc_context ctx, uint64_t slots, cudaStream_t s) {
    if (slots > ctx->table_cap) {
        if (ctx->table) cudaFree(ctx->table);
        ctx->table = nullptr;
        ctx->table_cap = 0;
        DAGC_CUDA(ctx, cudaMalloc(&ctx->table, slots * 16));  // per slot: key u64, aux u64
        ctx->table_cap = slots;
        ctx->table_dirty = true;
    }
    if (ctx->table_dirty) {
        DAGC_CUDA(ctx, cudaMemsetAsync(ctx->table, 0, ctx->table_cap * 16, s));
        ctx->table_dirty = false;
    }
    if (!ctx->gtable && ctx->group_mode != 0) DAGC_CUDA(ctx, cudaMalloc(&ctx->gtable, kGroupScratchBytes));
    return DAGC_OK;
}

int load_tune_file(dagc_context ctx, const char* path);

// Internal status: the hash-set dedup could not hold this input; the caller
// reruns the call with the radix form.
constexpr int kStatusFallback = -1000;

int create_pipeline(dagc_context ctx, const uint64_t* d_frag, uint64_t n, int depth, cudaStream_t s,
                    CreatePools& out, const BatchSpec* batch, bool use_dedup) {
    t_pdl = ctx->pdl;
    const int group_mode = ctx->group_mode;
    const int nl = depth - 2;
    const int bits = 3 * depth;
    // Batched calls take the persistent per-chunk leaf build (chunks.cu) when
    // the chunk's bins fit its limits; otherwise the composite-key path.
    const bool chunk_path = batch && ctx->batch_path == 1 && chunk_bin_bits(batch->chunk_depth) <= kChunkMaxBinBits;
    const CreateLayout Lo(n, depth, batch ? batch->k : 0u, use_dedup, ctx->dedup_unique_limit,
                          group_mode != 0 && use_dedup && !chunk_path, chunk_path ? batch->chunk_depth : 0);
    const std::vector<uint64_t>& cap = Lo.cap;
    const uint64_t capmax = Lo.capmax, p0cap = Lo.p0cap, sv_total = Lo.sv_total;
    const size_t zero_bytes = Lo.zero_bytes;
    (void)capmax;
    DAGC_CUDA(ctx, ctx->arena.reserve(Lo.total));
    arena_wait(ctx, s);
    if (use_dedup) {
        const int st = reserve_table(ctx, Lo.table_slots, s);
        if (st) return st;
    }
    char* b = static_cast<char*>(ctx->arena.base);
    auto P64 = [&](size_t o) { return reinterpret_cast<uint64_t*>(b + o); };
    auto P32 = [&](size_t o) { return reinterpret_cast<uint32_t*>(b + o); };
    auto P8 = [&](size_t o) { return reinterpret_cast<uint8_t*>(b + o); };
    // Fragment sort bits: the brick key [6, 3*depth); batched input sorts the
    // composite (chunk rank << 3*chunk_depth) | local code instead, whose
    // chunk rank needs only bits_for(k) bits (the chunks are in Morton order).
    int sort_hi = std::max(6, bits), validate = bits < 64 ? bits : 0, seg_shift = 0;
    if (batch) {
        seg_shift = 3 * batch->chunk_depth;
        sort_hi = std::max(6, seg_shift + bits_for(batch->k));
        validate = seg_shift;
        DAGC_CUDA(ctx, cudaMemcpyAsync(P64(Lo.o_seg_off), batch->h_offsets, (batch->k + 1) * 8,
                                       cudaMemcpyHostToDevice, s));
        DAGC_CUDA(ctx, cudaMemcpyAsync(P64(Lo.o_seg_code), batch->h_morton, batch->k * 8, cudaMemcpyHostToDevice, s));
    }
    // Chunk path: the first COUNT/SCATTER tile of every chunk (none when a
    // chunk is a single bin).
    uint32_t ck_tiles = 0;
    if (chunk_path) {
        ctx->ck_tile_host.assign(batch->k + 1, 0);
        for (uint32_t c = 0; c < batch->k; ++c) {
            const uint64_t nc = batch->h_offsets[c + 1] - batch->h_offsets[c];
            const uint64_t t = Lo.ck_bins > 1 ? (nc + kChunkTile - 1) / kChunkTile : 0;
            ctx->ck_tile_host[c + 1] = ctx->ck_tile_host[c] + (uint32_t)t;
        }
        ck_tiles = ctx->ck_tile_host[batch->k];
        DAGC_CUDA(ctx, cudaMemcpyAsync(P32(Lo.o_ck_tile), ctx->ck_tile_host.data(), (batch->k + 1) * 4,
                                       cudaMemcpyHostToDevice, s));
    }

    // Everything from here to the last kernel is enqueued by one function, so
    // that it can be recorded once as a CUDA graph and replayed.
    auto enqueue = [&](cudaStream_t s) -> int {
        CallSlots cs;
        cs.h = reinterpret_cast<CallHeader*>(b + Lo.o_hdr);
        cs.sv_next = P64(Lo.o_sv);
        cs.sv_end = P64(Lo.o_sv) + sv_total;
        SortBuffers sb{{P32(Lo.o_ss0), P32(Lo.o_ss1)}};
        DAGC_CUDA(ctx, cudaMemsetAsync(b, 0, zero_bytes, s));
        uint32_t* err = &cs.h->err;

        int st = DAGC_OK;
        // 1a. Fragment grouping by hash (group.cu): a sketch of the distinct
        //     bricks picks, on the device, this path or the sort path 1b-2;
        //     the kernels of the path not taken do nothing. Either path leaves
        //     the sorted bricks in P, their leaf masks in LM and their count.
        const uint32_t* gate = nullptr;
        if (chunk_path) {
            // 1. Every chunk's leaves in one persistent launch (+ scan, pack).
            StageTimer t(ctx, DAGC_STAGE_CHUNK_LEAVES, s);
            DAGC_CUDA(ctx, cudaMemsetAsync(b + Lo.o_ck_state, 0, Lo.ck_state_bytes, s));
            ChunkArgs ca{};
            ca.frags = d_frag;
            ca.seg_offsets = P64(Lo.o_seg_off);
            ca.seg_code = P64(Lo.o_seg_code);
            ca.k = batch->k;
            ca.chunk_depth = batch->chunk_depth;
            ca.seg_shift = seg_shift;
            ca.bin_bits = chunk_bin_bits(batch->chunk_depth);
            ca.tile_off = P32(Lo.o_ck_tile);
            ca.tiles = ck_tiles;
            ca.groups_per_chunk = Lo.ck_groups;
            ca.hist = P32(Lo.o_ck_hist);
            ca.cursor = P32(Lo.o_ck_cursor);
            ca.done = P32(Lo.o_ck_done);
            ca.work = P32(Lo.o_ck_work);
            ca.scratch = P64(Lo.o_B);
            ca.stage_parent = P64(Lo.o_A);
            ca.stage_mask = P64(Lo.o_ck_mask);
            ca.group_bricks = P32(Lo.o_ck_gb);
            ca.group_src = P64(Lo.o_ck_gs);
            ca.group_dst = P32(Lo.o_ck_gd);
            ca.parents = P64(Lo.o_P);
            ca.leaves = P64(Lo.o_LM);
            ca.out_capacity = p0cap;
            ca.d_out_n = cs.count(kCntBricks);
            ca.err = err;
            launch_chunk_leaves(ca, s);
            ctx->launches += 3;
            DAGC_LAUNCHED(ctx);
            t.stop();
        }
        if (!chunk_path && group_mode != 0 && use_dedup && ctx->gtable) {
            GroupArgs g{};
            g.frags = d_frag;
            g.n = n;
            g.seg_offsets = batch ? P64(Lo.o_seg_off) : nullptr;
            g.seg_count = batch ? batch->k : 0u;
            g.seg_shift = seg_shift;
            g.seg_code = batch ? P64(Lo.o_seg_code) : nullptr;
            g.validate_bits = validate;
            g.mode = group_mode;
            g.narrow = sort_hi <= 37 ? 1 : 0;
            g.chunks = group_chunks(n);
            g.sketch = cs.h->sketch;
            g.probe_max_distinct = Lo.group_probe_max;
            g.cursor = cs.h->gcursor;
            g.path = cs.h->path;
            g.parts = P64(Lo.o_slab);
            g.overflow = P64(Lo.o_over);
            g.overflow_cap = n;
            g.overflow_count = cs.count(kCntOverflow);
            g.part_over = cs.h->gover;
            g.bricks = P64(Lo.o_A);
            g.idx = P32(Lo.o_M0);
            g.masks = static_cast<uint64_t*>(ctx->gtable);
            g.cap = std::min<uint64_t>(p0cap, kGroupMaxBricks);
            g.d_count = cs.count(kCntBricks);
            g.sorted_bricks = P64(Lo.o_P);
            g.sorted_idx = P32(Lo.o_M1);
            g.parents = P64(Lo.o_P);
            g.leaves = P64(Lo.o_LM);
            g.err = err;
            {
                StageTimer t1(ctx, DAGC_STAGE_GROUP_SKETCH, s);
                launch_group_probe(g, s);
                launch_group_plan(g, s);
                ctx->launches += 2;
                t1.stop();
                StageTimer t2(ctx, DAGC_STAGE_GROUP_SCATTER, s);
                launch_group_scatter(g, s);
                ++ctx->launches;
                t2.stop();
                StageTimer t3(ctx, DAGC_STAGE_GROUP_AGGREGATE, s);
                launch_group_aggregate(g, s);
                ++ctx->launches;
                t3.stop();
            }
            DAGC_LAUNCHED(ctx);
            StageTimer tg(ctx, DAGC_STAGE_GROUP, s);
            // The bricks (B of them instead of N fragments), sorted with their indices.
            st = run_sort(ctx, cs, sb, P64(Lo.o_A), P64(Lo.o_P), P64(Lo.o_B), P32(Lo.o_M0), P32(Lo.o_M1),
                          P32(Lo.o_LM), true, g.cap, cs.count(kCntBricks), 0, sort_hi - 6, 0, s, -1, -1, nullptr,
                          cs.h->path, 1u);
            if (st) return st;
            launch_group_gather(g, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);
            tg.stop();
            gate = cs.h->path;
        }

        // 1b. Fragment sort on the brick key bits [6, 3*depth): only the order of
        //     code >> 6 matters downstream (the leaf mask ORs the low 6 bits).
        const SegmentSpec seg{batch ? P64(Lo.o_seg_off) : nullptr, batch ? batch->k : 0u, seg_shift};
        if (!chunk_path)
            st = run_sort(ctx, cs, sb, d_frag, P64(Lo.o_A), P64(Lo.o_B), nullptr, nullptr, nullptr, false, n, nullptr, 6,
                          sort_hi, validate, s, DAGC_STAGE_FRAGMENT_HIST, DAGC_STAGE_FRAGMENT_PASS, &seg, gate, 0u);
        if (st) return st;

        // 2. Fused unique + leaf build.
        if (!chunk_path) {
            StageTimer t(ctx, DAGC_STAGE_LEAF_BUILD, s);
            LeafBuildArgs a{};
            a.sorted = P64(Lo.o_A);
            a.d_n = nullptr;
            a.n_bound = n;
            a.parents = P64(Lo.o_P);
            a.leaves = P64(Lo.o_LM);
            a.out_capacity = p0cap;
            a.lead_or = P64(Lo.o_lead_or);
            a.lead_run = P64(Lo.o_lead_run);
            a.seg_code = batch ? P64(Lo.o_seg_code) : nullptr;
            a.seg_shift = seg_shift;
            a.d_out_n = cs.count(kCntBricks);
            a.status = cs.sv(n);
            a.tile_counter = cs.counter();
            a.err = err;
            a.grid = grid_for(ctx->grid_leaf / ctx->sms, ctx->sms, leaf_tiles(n));
            a.gate = gate;
            a.gate_run = 0u;
            launch_leaf_build(a, s);
            ctx->launches += 2;
            DAGC_LAUNCHED(ctx);
            t.stop();
        }
        // 3. Leaf dedup: SortLevel on the leaf masks (the mask is its own hash).
        StageTimer t_dedup(ctx, DAGC_STAGE_LEAF_DEDUP, s);
        // Hash-set dedup arguments shared by the leaves and every level.
        auto dedup_args = [&](const uint64_t* keys, uint64_t* d_n, const uint8_t* masks, const uint32_t* children,
                              uint64_t* out_keys, uint8_t* out_masks, uint32_t* out_children, uint64_t out_cap,
                              uint64_t* d_out_n, uint32_t* map) {
            DedupArgs d{};
            d.keys = keys;
            d.d_n = d_n;
            d.masks = masks;
            d.children = children;
            d.to_list = masks == nullptr;  // leaf masks are not uniformly distributed; node hashes are
            d.item_cap = Lo.item_cap;
            d.table_key = static_cast<uint64_t*>(ctx->table);
            d.table_aux = static_cast<uint64_t*>(ctx->table) + 1;
            d.table_cap = ctx->table_cap;
            d.item_slot = P32(Lo.o_islot);
            d.uniq_key = P64(Lo.o_ukey);
            d.uniq_cap = Lo.uniq_cap;
            d.bucket_count = P32(Lo.o_bcnt);
            d.bucket = reinterpret_cast<uint4*>(b + Lo.o_bent);
            d.bucket_area = Lo.bucket_area;
            d.state = cs.dedup();
            d.out_keys = out_keys;
            d.out_masks = out_masks;
            d.out_children = out_children;
            d.out_capacity = out_cap;
            d.d_out_n = d_out_n;
            d.map = map;
            d.err = err;
            return d;
        };
        if (use_dedup) {
            // Distinct masks into the table and the unique list; the list
            // sorted (keys only) straight into the leaf array; each mask's
            // slot gets the mask's rank as unique id; every brick its id.
            const DedupArgs d = dedup_args(P64(Lo.o_LM), cs.count(kCntBricks), nullptr, nullptr, P64(Lo.o_PL), nullptr,
                                           nullptr, p0cap, cs.count(kCntLeaves), P32(Lo.o_M0));
            launch_dedup_insert(d, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);
            // Up to kSmallSortMax distinct masks: one CTA sorts them in shared
            // memory and the grid-wide sort's kernels return at once.
            const uint64_t* d_u = reinterpret_cast<const uint64_t*>(&d.state->u);
            launch_small_sort(P64(Lo.o_ukey), P64(Lo.o_PL), d_u, Lo.uniq_cap, &cs.h->leaf_sorted, s);
            ++ctx->launches;
            st = run_sort(ctx, cs, sb, P64(Lo.o_ukey), P64(Lo.o_PL), P64(Lo.o_ukey_alt), nullptr, nullptr, nullptr,
                          false, Lo.uniq_cap, d_u, 0, 64, 0, s, -1, -1, nullptr, &cs.h->leaf_sorted, 0u);
            if (st) return st;
            launch_dedup_assign(d, P64(Lo.o_PL), s);
            launch_dedup_map(d, s);
            ctx->launches += 2;
            DAGC_LAUNCHED(ctx);
        } else {
        st = run_sort(ctx, cs, sb, P64(Lo.o_LM), P64(Lo.o_SK), P64(Lo.o_SKa), nullptr, P32(Lo.o_V), P32(Lo.o_Va), true, p0cap,
                      cs.count(kCntBricks), 0, 64, 0, s);
        if (st) return st;
        {
            UniqueArgs a{};
            a.keys = P64(Lo.o_SK);
            a.perm = P32(Lo.o_V);
            a.d_n = cs.count(kCntBricks);
            a.n_bound = p0cap;
            a.map = P32(Lo.o_M0);
            a.out_keys = P64(Lo.o_PL);
            a.out_capacity = p0cap;
            a.d_out_n = cs.count(kCntLeaves);
            a.status = cs.sv(p0cap);
            a.tile_counter = cs.counter();
            a.err = err;
            a.grid = grid_for(ctx->grid_unique / ctx->sms, ctx->sms, scan_tiles(p0cap));
            launch_unique(a, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);
        }
        }
        t_dedup.stop();
        // 4. Level loop, bottom-up.
        StageTimer t_levels(ctx, DAGC_STAGE_LEVELS, s);
        const uint64_t* child_codes = P64(Lo.o_P);
        const uint32_t* child_map = P32(Lo.o_M0);
        const uint64_t* child_hashes = P64(Lo.o_PL);
        const uint64_t* d_child_n = cs.count(kCntBricks);
        uint64_t child_bound = p0cap;
        uint64_t* node_codes[2] = {P64(Lo.o_NC0), P64(Lo.o_NC1)};
        uint32_t* maps[2] = {P32(Lo.o_M1), P32(Lo.o_M0)};
        // Levels whose node bound fits one CTA's shared memory go to the tail
        // kernel; the bound only grows with the level index, so they are the top
        // tail_first + 1 levels.
        int tail_first = -1;
        while (tail_first + 1 < nl && tail_first + 1 < kMaxTailLevels && cap[tail_first + 1] <= (uint64_t)kTailCap)
            ++tail_first;
        // The tail's first level reads all of its children in one CTA: a level
        // that may have many (8^5 bound at depth >= 8 with dense top levels)
        // goes to the multi-CTA path instead.
        while (tail_first >= 0 && (tail_first + 1 < nl ? cap[tail_first + 1] : p0cap) > (uint64_t)kTailChildCap)
            --tail_first;
        for (int l = nl - 1, it = 0; l > tail_first; --l, ++it) {
            ExtractArgs e{};
            e.child_codes = child_codes;
            e.child_map = child_map;
            e.d_n = d_child_n;
            e.n_bound = child_bound;
            e.child_hashes = child_hashes;
            e.node_codes = node_codes[it & 1];
            e.node_masks = P8(Lo.o_NM);
            e.node_children = P32(Lo.o_NCH);
            e.node_hashes = P64(Lo.o_NH);
            e.out_capacity = cap[l];
            e.d_out_n = cs.count(kCntNodes + l);
            e.status = cs.sv(child_bound);
            e.tile_counter = cs.counter();
            e.err = err;
            e.grid = grid_for(ctx->grid_extract / ctx->sms, ctx->sms, scan_tiles(child_bound));
            DedupArgs d{};
            if (use_dedup) {
                // The node hashes go into the dedup table inside extract_level.
                d = dedup_args(P64(Lo.o_NH), cs.count(kCntNodes + l), P8(Lo.o_NM), P32(Lo.o_NCH), P64(Lo.o_ph[l]),
                               P8(Lo.o_pm[l]), P32(Lo.o_pc[l]), cap[l], cs.count(kCntUnique + l), maps[it & 1]);
                e.fuse_insert = 1;
                e.dedup = d;
            }
            launch_extract(e, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);

            if (use_dedup) {
                ctx->launches += launch_dedup(d, s);
                DAGC_LAUNCHED(ctx);
                child_codes = node_codes[it & 1];
                child_map = maps[it & 1];
                child_hashes = P64(Lo.o_ph[l]);
                d_child_n = cs.count(kCntNodes + l);
                child_bound = cap[l];
                continue;
            }
            st = run_sort(ctx, cs, sb, P64(Lo.o_NH), P64(Lo.o_SK), P64(Lo.o_SKa), nullptr, P32(Lo.o_V), P32(Lo.o_Va), true,
                          cap[l], cs.count(kCntNodes + l), 0, 64, 0, s);
            if (st) return st;

            UniqueArgs u{};
            u.keys = P64(Lo.o_SK);
            u.perm = P32(Lo.o_V);
            u.d_n = cs.count(kCntNodes + l);
            u.n_bound = cap[l];
            u.masks = P8(Lo.o_NM);
            u.children = P32(Lo.o_NCH);
            u.map = maps[it & 1];
            u.out_keys = P64(Lo.o_ph[l]);
            u.out_masks = P8(Lo.o_pm[l]);
            u.out_children = P32(Lo.o_pc[l]);
            u.out_capacity = cap[l];
            u.d_out_n = cs.count(kCntUnique + l);
            u.status = cs.sv(cap[l]);
            u.tile_counter = cs.counter();
            u.err = err;
            u.grid = grid_for(ctx->grid_unique / ctx->sms, ctx->sms, scan_tiles(cap[l]));
            launch_unique(u, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);

            child_codes = node_codes[it & 1];
            child_map = maps[it & 1];
            child_hashes = P64(Lo.o_ph[l]);
            d_child_n = cs.count(kCntNodes + l);
            child_bound = cap[l];
        }
        if (tail_first >= 0) {
            TailArgs ta{};
            ta.first_level = tail_first;
            ta.child_codes = child_codes;
            ta.child_map = child_map;
            ta.child_hashes = child_hashes;
            ta.d_child_n = d_child_n;
            for (int l = 0; l <= tail_first; ++l) {
                ta.lv[l].hashes = P64(Lo.o_ph[l]);
                ta.lv[l].masks = P8(Lo.o_pm[l]);
                ta.lv[l].children = P32(Lo.o_pc[l]);
                ta.lv[l].capacity = cap[l];
                ta.lv[l].d_nodes = cs.count(kCntNodes + l);
                ta.lv[l].d_unique = cs.count(kCntUnique + l);
            }
            ta.err = err;
            launch_tail(ta, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);
        }

        t_levels.stop();
        if (cs.sv_next > cs.sv_end) return set_error(ctx, DAGC_ERR_CUDA, "look-back status regions miscounted");
    return DAGC_OK;
    };
    int st = run_enqueue(ctx, GraphKey{d_frag, n, depth, ctx->arena.base, batch ? batch->k : 0u,
                                       batch ? batch->chunk_depth : 0, chunk_path, use_dedup,
                                       use_dedup ? ctx->table : nullptr, use_dedup ? group_mode : 0},
                         s, enqueue);
    if (st) { ctx->table_dirty = true; return st; }
    CallHeader* hdr = reinterpret_cast<CallHeader*>(b + Lo.o_hdr);
    // 5. One read-back of every count and the error word.
    static_assert(sizeof(CallHeader) >= 8 * 65, "header");
    DAGC_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage, hdr, 8 + 8 * 64, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaStreamSynchronize(s));
    const uint32_t e32 = (uint32_t)(ctx->h_stage[0] & 0xFFFFFFFFu);
    const uint64_t* counts = ctx->h_stage + 1;
    ctx->last_counts.assign(3 + nl, 0);
    ctx->last_counts[0] = n;
    ctx->last_counts[1] = counts[kCntBricks];
    ctx->last_counts[2] = counts[kCntLeaves];
    for (int l = 0; l < nl; ++l) ctx->last_counts[3 + l] = counts[kCntNodes + l];
    if (ctx->profiling) {
        // Algorithmic bytes: the minimum each stage must read and write.
        const uint64_t p0 = counts[kCntBricks], lv = counts[kCntLeaves];
        set_pending_bytes(ctx, DAGC_STAGE_LEAF_BUILD, 8 * n + 16 * p0);
        // Grouping: the probe reads a sixteenth of the fragments; the scatter
        // reads 8 bytes per fragment and writes its slab entry (4 bytes in the
        // narrow form, else 8), which the aggregation reads; the brick sort
        // and the gather move ~60 bytes per brick.
        const uint64_t entry = sort_hi <= 37 ? 4 : 8;
        set_pending_bytes(ctx, DAGC_STAGE_GROUP_SKETCH, n / 2);
        set_pending_bytes(ctx, DAGC_STAGE_GROUP_SCATTER, (8 + entry) * n);
        set_pending_bytes(ctx, DAGC_STAGE_GROUP_AGGREGATE, entry * n + 20 * p0);
        set_pending_bytes(ctx, DAGC_STAGE_GROUP, 60 * p0);
        // Chunk leaves: COUNT reads the fragments, SCATTER reads and writes
        // them, LEAVES reads them and writes 16 bytes per brick, the pack
        // moves those bricks once more.
        set_pending_bytes(ctx, DAGC_STAGE_CHUNK_LEAVES, (Lo.ck_bins > 1 ? 32 : 8) * n + 48 * p0);
        set_pending_bytes(ctx, DAGC_STAGE_LEAF_DEDUP, 216 * p0 + 8 * lv);
        uint64_t lb = 0;
        for (int l = 0; l < nl; ++l) {
            const uint64_t child = l + 1 < nl ? counts[kCntNodes + l + 1] : p0;
            lb += 20 * child + 293 * counts[kCntNodes + l] + 41 * counts[kCntUnique + l];
        }
        set_pending_bytes(ctx, DAGC_STAGE_LEVELS, lb);
        // The kernels of the path the device did not take returned at once.
        if (group_mode != 0 && use_dedup && ctx->gtable) {
            uint32_t path = 0;
            DAGC_CUDA(ctx, cudaMemcpy(&path, &hdr->path[0], 4, cudaMemcpyDeviceToHost));
            if (path == 1) {
                override_pending_bytes(ctx, DAGC_STAGE_FRAGMENT_HIST, 0);
                override_pending_bytes(ctx, DAGC_STAGE_FRAGMENT_PASS, 0);
                override_pending_bytes(ctx, DAGC_STAGE_LEAF_BUILD, 0);
            } else {
                override_pending_bytes(ctx, DAGC_STAGE_GROUP_SCATTER, 0);
                override_pending_bytes(ctx, DAGC_STAGE_GROUP_AGGREGATE, 0);
                override_pending_bytes(ctx, DAGC_STAGE_GROUP, 0);
            }
        }
        settle_profile(ctx);
    }
    if (e32) ctx->table_dirty = true;  // a level may have stopped before clearing its slots
    if ((e32 & kErrFallback) && !(e32 & (kErrBadInput | kErrTimeout))) return kStatusFallback;
    std::string msg;
    st = device_error_status(e32, msg);
    if (st) return set_error(ctx, st, msg);
    if (nl > 0 && counts[kCntUnique + 0] != 1) return set_error(ctx, DAGC_ERR_BAD_INPUT, "root level must hold one node");
    if (nl == 0 && counts[kCntLeaves] != 1) return set_error(ctx, DAGC_ERR_BAD_INPUT, "depth-2 volume must hold one leaf");

    out.hashes.resize(nl);
    out.children.resize(nl);
    out.masks.resize(nl);
    out.unique.resize(nl);
    for (int l = 0; l < nl; ++l) {
        out.hashes[l] = P64(Lo.o_ph[l]);
        out.children[l] = P32(Lo.o_pc[l]);
        out.masks[l] = P8(Lo.o_pm[l]);
        out.unique[l] = counts[kCntUnique + l];
    }
    out.leaves = P64(Lo.o_PL);
    out.num_leaves = counts[kCntLeaves];
    return DAGC_OK;
}

int materialise(dagc_context ctx, const CreatePools& p, int nl, cudaStream_t s, dagc_dag* out) {
    t_pdl = ctx->pdl;
    dagc_dag d = nullptr;
    int st = alloc_dag(ctx, nl, p.unique, p.num_leaves, &d);
    if (st) return st;
    uint64_t total_u = 0;
    for (int l = 0; l < nl; ++l) total_u += p.unique[l];
    StageTimer t(ctx, DAGC_STAGE_MATERIALISE, s);
    // Every level's arrays and the leaves in one copy kernel; the level
    // offsets from the host. No wait: the words (CreateFinalDAG) or any read
    // of the DAG follow on the same stream.
    CopyTable ct{};
    auto add = [&](const void* src, void* dst, uint64_t bytes) {
        if (bytes) ct.seg[ct.count++] = CopySeg{src, dst, bytes};
    };
    for (int l = 0; l < nl; ++l) {
        const uint64_t o = d->level_offset[l], u = p.unique[l];
        add(p.hashes[l], d->hashes + o, u * 8);
        add(p.children[l], d->children + o * 8, u * 32);
        add(p.masks[l], d->masks + o, u);
    }
    add(p.leaves, d->leaves, p.num_leaves * 8);
    static_assert(3 * (kMaxDepth - 2) + 1 <= kMaxCopySegs && kMaxDepth - 1 <= 24, "copy table");
    ct.lit_dst = d->d_level_offset;
    ct.lit_count = nl + 1;
    for (int l = 0; l <= nl; ++l) ct.lit[l] = d->level_offset[l];
    launch_copy_segments(ct, s);
    ++ctx->launches;
    t.stop(2 * (41 * total_u + 8 * p.num_leaves));
    cudaError_t e = cudaGetLastError();
    d->ready = take_sync_event(ctx);
    if (!ctx->arena_copy && cudaEventCreateWithFlags(&ctx->arena_copy, cudaEventDisableTiming) != cudaSuccess)
        ctx->arena_copy = nullptr;
    if (e == cudaSuccess && d->ready) e = cudaEventRecord(d->ready, s);
    if (e == cudaSuccess && ctx->arena_copy) e = cudaEventRecord(ctx->arena_copy, s);
    if (e == cudaSuccess && (!d->ready || !ctx->arena_copy)) e = cudaStreamSynchronize(s);  // no events: wait here
    ctx->arena_copy_pending = ctx->arena_copy != nullptr;
    if (ctx->profiling && e == cudaSuccess) e = cudaStreamSynchronize(s);
    settle_profile(ctx);
    if (e != cudaSuccess) {
        free_dag(d);
        cudaGetLastError();
        return set_error(ctx, cuda_status(e), std::string("materialise: ") + cudaGetErrorString(e));
    }
    *out = d;
    return DAGC_OK;
}

int empty_dag(dagc_context ctx, int nl, dagc_dag* out) {
    return alloc_dag(ctx, nl, std::vector<uint64_t>(nl, 0), 0, out);
}

// --------------------------------------------------------- CreateFinalDAG --
// The node levels (root first) and leaves that CreateFinalDAG lays out.
struct FinalSource {
    std::vector<const uint8_t*> masks;     // per level
    std::vector<const uint32_t*> children;  // per level, 8 per node
    std::vector<uint64_t> off;              // num_levels + 1 node offsets
    const uint64_t* leaves = nullptr;
    uint64_t num_leaves = 0;
};

// Bytes of arena scratch the final layout of nn nodes takes (from offset 0).
size_t final_scratch_bytes(uint64_t nn) {
    Layout L;
    L.take<CallHeader>(1);
    L.take<uint64_t>(scan_tiles(nn) + 1);
    L.take<uint32_t>(nn + 1);
    return L.off;
}

// Positions and words of `src`, their scratch at the start of the arena,
// which the caller has reserved and made safe to write.
int final_words(dagc_context ctx, const FinalSource& src, cudaStream_t s, uint32_t** d_words, uint64_t* n_words) {
    t_pdl = ctx->pdl;
    *d_words = nullptr;
    *n_words = 0;
    const int nlv = (int)src.masks.size();
    if (nlv > kFinalMaxLevels) return set_error(ctx, DAGC_ERR_TOO_LARGE, "too many levels");
    const uint64_t nn = src.off[nlv];
    Layout L;
    const size_t o_hdr = L.take<CallHeader>(1);
    const uint64_t svt = scan_tiles(nn) + 1;
    const size_t o_sv = L.take<uint64_t>(svt);
    const size_t zero_bytes = L.off;
    const size_t o_pos = L.take<uint32_t>(nn + 1);
    char* b = static_cast<char*>(ctx->arena.base);
    CallHeader* h = reinterpret_cast<CallHeader*>(b + o_hdr);
    uint32_t* pos = reinterpret_cast<uint32_t*>(b + o_pos);
    DAGC_CUDA(ctx, cudaMemsetAsync(b, 0, zero_bytes, s));
    FinalArgs a{};
    for (int l = 0; l < nlv; ++l) {
        a.lv_masks[l] = src.masks[l];
        a.lv_children[l] = src.children[l];
    }
    for (int l = 0; l <= nlv; ++l) a.lv_off[l] = src.off[l];
    a.num_levels = nlv;
    a.num_nodes = nn;
    a.leaves = src.leaves;
    a.num_leaves = src.num_leaves;
    a.word_pos = pos;
    a.d_total = &h->counts[0];
    a.status = reinterpret_cast<uint64_t*>(b + o_sv);
    a.tile_counter = &h->tile_counters[0];
    a.err = &h->err;
    a.grid_scan = grid_for(ctx->grid_scan / ctx->sms, ctx->sms, scan_tiles(nn));
    a.grid_write = grid_for(ctx->grid_write / ctx->sms, ctx->sms, (nn + src.num_leaves + 255) / 256);
    // Words: at most 1 + 8 per node and 2 per leaf. Allocating that bound
    // lets the positions and the write run back to back; the exact count
    // comes back with the error word in the call's one read-back.
    const uint64_t bound = 9 * nn + 2 * src.num_leaves;
    const bool by_bound = bound < (1ull << 32);
    uint64_t node_words = 0;
    void* w = nullptr;
    StageTimer t(ctx, DAGC_STAGE_FINAL, s);
    if (nn) {
        launch_final_positions(a, s);
        ++ctx->launches;
        DAGC_LAUNCHED(ctx);
        if (!by_bound) {
            DAGC_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage, &h->counts[0], 8, cudaMemcpyDeviceToHost, s));
            DAGC_CUDA(ctx, cudaStreamSynchronize(s));
            node_words = ctx->h_stage[0];
            if (node_words + 2 * src.num_leaves >= (1ull << 32))
                return set_error(ctx, DAGC_ERR_TOO_LARGE, "final DAG exceeds 2^32 words");
        }
    } else {
        DAGC_CUDA(ctx, cudaMemsetAsync(pos, 0, 4, s));
    }
    DAGC_CUDA(ctx, ctx->pool.alloc(&w, (by_bound ? bound : node_words + 2 * src.num_leaves) * 4, "final DAG words"));
    a.words = static_cast<uint32_t*>(w);
    launch_final_write(a, s);
    ++ctx->launches;
    t.stop();
    cudaError_t le = cudaGetLastError();
    if (le == cudaSuccess) le = cudaMemcpyAsync(ctx->h_stage, h, 16, cudaMemcpyDeviceToHost, s);  // err, counts[0]
    if (le == cudaSuccess) le = cudaStreamSynchronize(s);
    if (le != cudaSuccess) {
        ctx->pool.release(w);
        return set_error(ctx, cuda_status(le), std::string("final: ") + cudaGetErrorString(le));
    }
    if (nn) node_words = ctx->h_stage[1];
    const uint64_t total = node_words + 2 * src.num_leaves;
    set_pending_bytes(ctx, DAGC_STAGE_FINAL, nn * 2 + (41 * nn + 8 * src.num_leaves) + 4 * total);
    settle_profile(ctx);
    std::string msg;
    const int st = device_error_status((uint32_t)ctx->h_stage[0], msg);
    if (st) { ctx->pool.release(w); return set_error(ctx, st, msg); }
    *d_words = a.words;
    *n_words = total;
    return DAGC_OK;
}

int final_dag(dagc_context ctx, dagc_dag d, cudaStream_t s, uint32_t** d_words, uint64_t* n_words) {
    *d_words = nullptr;
    *n_words = 0;
    if (d->num_leaves == 0) return DAGC_OK;
    FinalSource src;
    for (int l = 0; l < d->num_levels; ++l) {
        src.masks.push_back(d->masks + d->level_offset[l]);
        src.children.push_back(d->children + 8 * d->level_offset[l]);
    }
    src.off.assign(d->level_offset.begin(), d->level_offset.begin() + d->num_levels + 1);
    src.leaves = d->leaves;
    src.num_leaves = d->num_leaves;
    DAGC_CUDA(ctx, ctx->arena.reserve(final_scratch_bytes(d->num_nodes())));
    arena_wait(ctx, s);
    dag_ready_wait(d, s);
    return final_words(ctx, src, s, d_words, n_words);
}

// CreateDAG + CreateFinalDAG in one call: the words straight from the call's
// per-level pools, with no copy of the DAG out of the arena, when the final
// layout's scratch lies below every pool in the arena.
int compress_from_pools(dagc_context ctx, const CreatePools& p, int nl, cudaStream_t s, uint32_t** d_words,
                        uint64_t* n_words, bool* done) {
    *done = false;
    if (p.num_leaves == 0) { *done = true; *d_words = nullptr; *n_words = 0; return DAGC_OK; }
    FinalSource src;
    src.off.push_back(0);
    const char* base = static_cast<const char*>(ctx->arena.base);
    size_t lowest = reinterpret_cast<const char*>(p.leaves) - base;
    for (int l = 0; l < nl; ++l) {
        src.masks.push_back(p.masks[l]);
        src.children.push_back(p.children[l]);
        src.off.push_back(src.off.back() + p.unique[l]);
        lowest = std::min<size_t>(lowest, reinterpret_cast<const char*>(p.masks[l]) - base);
        lowest = std::min<size_t>(lowest, reinterpret_cast<const char*>(p.children[l]) - base);
        lowest = std::min<size_t>(lowest, reinterpret_cast<const char*>(p.hashes[l]) - base);
    }
    src.leaves = p.leaves;
    src.num_leaves = p.num_leaves;
    if (final_scratch_bytes(src.off[nl]) > lowest) return DAGC_OK;  // would overlap a pool
    *done = true;
    return final_words(ctx, src, s, d_words, n_words);
}

// -------------------------------------------------------------- MergeDAGs --
struct HostNode {
    uint64_t hash;
    uint8_t mask;
    uint32_t ch[8];
};

// union_only: the per-level union of any number k >= 1 of DAGs of equal depth
// (no levels added; the result's top level holds every input's root), and
// each input's root hash in root_hash_out (0 for an empty input). Otherwise
// MergeDAGs: k = 8^m inputs in Morton order, m levels built above them.
int merge_dags(dagc_context ctx, dagc_dag* in, uint64_t k, cudaStream_t s, dagc_dag* out, bool union_only = false,
               std::vector<uint64_t>* root_hash_out = nullptr) {
    t_pdl = ctx->pdl;
    const int nl = in[0]->num_levels;
    int m = 0;
    if (!union_only)
        for (uint64_t x = k; x > 1; x /= 8) ++m;
    uint64_t total_leaves = 0;
    std::vector<uint64_t> level_total(nl, 0);
    for (uint64_t i = 0; i < k; ++i) {
        total_leaves += in[i]->num_leaves;
        for (int l = 0; l < nl; ++l) level_total[l] += in[i]->level_offset[l + 1] - in[i]->level_offset[l];
    }
    const int out_levels = nl + m;
    if (total_leaves == 0) {
        if (root_hash_out) root_hash_out->assign(k, 0);
        return empty_dag(ctx, out_levels, out);
    }
    uint64_t capmax = total_leaves;
    for (int l = 0; l < nl; ++l) capmax = std::max(capmax, level_total[l]);
    if (capmax > kMaxFragments) return set_error(ctx, DAGC_ERR_TOO_LARGE, "merged level too large");

    Layout L;
    const size_t o_hdr = L.take<CallHeader>(1);
    uint64_t sv_total = sv_words(total_leaves);
    for (int l = 0; l < nl; ++l) sv_total += sv_words(level_total[l]);
    const size_t o_sv = L.take<uint64_t>(sv_total);
    const size_t zero_bytes = L.off;
    const size_t o_ss0 = L.take<uint32_t>(sort_status_words(capmax));
    const size_t o_ss1 = L.take<uint32_t>(sort_status_words(capmax));
    const size_t o_KC = L.take<uint64_t>(capmax);
    const size_t o_MC = L.take<uint8_t>(capmax);
    const size_t o_CC = L.take<uint32_t>(capmax * 8);
    const size_t o_SK = L.take<uint64_t>(capmax);
    const size_t o_SKa = L.take<uint64_t>(capmax);
    const size_t o_V = L.take<uint32_t>(capmax);
    const size_t o_Va = L.take<uint32_t>(capmax);
    const size_t o_M0 = L.take<uint32_t>(capmax);
    const size_t o_M1 = L.take<uint32_t>(capmax);
    const size_t o_PL = L.take<uint64_t>(total_leaves);
    std::vector<size_t> o_ph(nl), o_pc(nl), o_pm(nl);
    for (int l = 0; l < nl; ++l) {
        o_ph[l] = L.take<uint64_t>(level_total[l]);
        o_pc[l] = L.take<uint32_t>(level_total[l] * 8);
        o_pm[l] = L.take<uint8_t>(level_total[l]);
    }
    const size_t o_root_hash = L.take<uint64_t>(k);
    const size_t o_root_uid = L.take<uint32_t>(k);
    DAGC_CUDA(ctx, ctx->arena.reserve(L.off));
    arena_wait(ctx, s);
    for (uint64_t i = 0; i < k; ++i) dag_ready_wait(in[i], s);
    char* b = static_cast<char*>(ctx->arena.base);
    auto P64 = [&](size_t o) { return reinterpret_cast<uint64_t*>(b + o); };
    auto P32 = [&](size_t o) { return reinterpret_cast<uint32_t*>(b + o); };
    auto P8 = [&](size_t o) { return reinterpret_cast<uint8_t*>(b + o); };
    CallSlots cs;
    cs.h = reinterpret_cast<CallHeader*>(b + o_hdr);
    cs.sv_next = P64(o_sv);
    cs.sv_end = P64(o_sv) + sv_total;
    SortBuffers sb{{P32(o_ss0), P32(o_ss1)}};
    DAGC_CUDA(ctx, cudaMemsetAsync(b, 0, zero_bytes, s));
    uint32_t* err = &cs.h->err;

    StageTimer t_merge(ctx, DAGC_STAGE_MERGE, s);
    // Leaves: sorted union of all inputs' leaves.
    std::vector<uint64_t> prev_off(k + 1, 0);
    for (uint64_t i = 0; i < k; ++i) {
        prev_off[i + 1] = prev_off[i] + in[i]->num_leaves;
        if (in[i]->num_leaves)
            DAGC_CUDA(ctx, cudaMemcpyAsync(P64(o_KC) + prev_off[i], in[i]->leaves, in[i]->num_leaves * 8,
                                           cudaMemcpyDeviceToDevice, s));
    }
    int st = run_sort(ctx, cs, sb, P64(o_KC), P64(o_SK), P64(o_SKa), nullptr, P32(o_V), P32(o_Va), true,
                      total_leaves, nullptr, 0, 64, 0, s);
    if (st) return st;
    {
        UniqueArgs a{};
        a.keys = P64(o_SK);
        a.perm = P32(o_V);
        a.n_bound = total_leaves;
        a.map = P32(o_M0);
        a.out_keys = P64(o_PL);
        a.out_capacity = total_leaves;
        a.d_out_n = cs.count(kCntLeaves);
        a.status = cs.sv(total_leaves);
        a.tile_counter = cs.counter();
        a.err = err;
        a.grid = grid_for(ctx->grid_unique / ctx->sms, ctx->sms, scan_tiles(total_leaves));
        launch_unique(a, s);
        ++ctx->launches;
        DAGC_LAUNCHED(ctx);
    }
    uint32_t* maps[2] = {P32(o_M0), P32(o_M1)};
    int cur = 0;
    for (int l = nl - 1; l >= 0; --l) {
        std::vector<uint64_t> off(k + 1, 0);
        for (uint64_t i = 0; i < k; ++i) {
            const dagc_dag d = in[i];
            const uint64_t a0 = d->level_offset[l], u = d->level_offset[l + 1] - a0;
            off[i + 1] = off[i] + u;
            if (!u) continue;
            DAGC_CUDA(ctx, cudaMemcpyAsync(P64(o_KC) + off[i], d->hashes + a0, u * 8, cudaMemcpyDeviceToDevice, s));
            DAGC_CUDA(ctx, cudaMemcpyAsync(P8(o_MC) + off[i], d->masks + a0, u, cudaMemcpyDeviceToDevice, s));
            launch_remap_children(d->children + a0 * 8, maps[cur] + prev_off[i], P32(o_CC) + off[i] * 8, u, s);
            ++ctx->launches;
            DAGC_LAUNCHED(ctx);
        }
        const uint64_t nlev = off[k];
        st = run_sort(ctx, cs, sb, P64(o_KC), P64(o_SK), P64(o_SKa), nullptr, P32(o_V), P32(o_Va), true, nlev,
                      nullptr, 0, 64, 0, s);
        if (st) return st;
        UniqueArgs u{};
        u.keys = P64(o_SK);
        u.perm = P32(o_V);
        u.n_bound = nlev;
        u.masks = P8(o_MC);
        u.children = P32(o_CC);
        u.map = maps[cur ^ 1];
        u.out_keys = P64(o_ph[l]);
        u.out_masks = P8(o_pm[l]);
        u.out_children = P32(o_pc[l]);
        u.out_capacity = level_total[l];
        u.d_out_n = cs.count(kCntUnique + l);
        u.status = cs.sv(level_total[l]);
        u.tile_counter = cs.counter();
        u.err = err;
        u.grid = grid_for(ctx->grid_unique / ctx->sms, ctx->sms, scan_tiles(nlev));
        launch_unique(u, s);
        ++ctx->launches;
        DAGC_LAUNCHED(ctx);
        cur ^= 1;
        prev_off = off;
    }
    // Root ids of every input in the merged top level (or the leaves when
    // the inputs have no inner level), and their hashes.
    std::vector<uint64_t> root_hash(k, 0);
    std::vector<uint32_t> root_uid(k, kEmptyChild);
    auto input_empty = [&](uint64_t i) { return nl > 0 ? in[i]->level_offset[1] == 0 : in[i]->num_leaves == 0; };
    for (uint64_t i = 0; i < k; ++i) {
        if (input_empty(i)) continue;
        DAGC_CUDA(ctx, cudaMemcpyAsync(P32(o_root_uid) + i, maps[cur] + prev_off[i], 4, cudaMemcpyDeviceToDevice, s));
        DAGC_CUDA(ctx, cudaMemcpyAsync(P64(o_root_hash) + i, nl > 0 ? in[i]->hashes : in[i]->leaves, 8,
                                       cudaMemcpyDeviceToDevice, s));
    }
    t_merge.stop();
    std::vector<uint64_t> stage_hash(k, 0);
    std::vector<uint32_t> stage_uid(k, 0);
    DAGC_CUDA(ctx, cudaMemcpyAsync(stage_hash.data(), P64(o_root_hash), k * 8, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaMemcpyAsync(stage_uid.data(), P32(o_root_uid), k * 4, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage, cs.h, 8 + 8 * 64, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaStreamSynchronize(s));
    {
        std::string msg;
        st = device_error_status((uint32_t)(ctx->h_stage[0] & 0xFFFFFFFFu), msg);
        if (st) return set_error(ctx, st, msg);
    }
    if (cs.sv_next > cs.sv_end) return set_error(ctx, DAGC_ERR_CUDA, "look-back status regions miscounted");
    settle_profile(ctx);
    const uint64_t* counts = ctx->h_stage + 1;
    for (uint64_t i = 0; i < k; ++i) {
        if (input_empty(i)) continue;
        root_uid[i] = stage_uid[i];
        root_hash[i] = stage_hash[i];
    }
    if (root_hash_out) *root_hash_out = root_hash;

    // Top levels: groups of 8 consecutive roots, built on the host like the
    // reference (src/DAGCompression.cu:1504-1533), deduplicated by hash.
    std::vector<std::vector<HostNode>> top;  // top[0] = just above the inputs
    uint64_t groups = union_only ? 1 : k;
    while (groups > 1) {
        const uint64_t ng = groups / 8;
        std::vector<HostNode> cand;
        std::vector<int64_t> cand_of(ng, -1);
        for (uint64_t g = 0; g < ng; ++g) {
            HostNode nd{};
            uint64_t hs[8];
            for (int c = 0; c < 8; ++c) {
                hs[c] = root_hash[8 * g + c];
                nd.ch[c] = root_uid[8 * g + c];
                if (hs[c]) nd.mask |= (uint8_t)(1u << c);
            }
            nd.hash = hash_children(hs);
            if (nd.mask) { cand_of[g] = (int64_t)cand.size(); cand.push_back(nd); }
        }
        std::vector<uint32_t> order(cand.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (uint32_t)i;
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return cand[a].hash < cand[c].hash; });
        std::vector<HostNode> lvl;
        std::vector<uint32_t> uid_of(cand.size());
        for (size_t i = 0; i < order.size(); ++i) {
            const HostNode& nd = cand[order[i]];
            if (lvl.empty() || lvl.back().hash != nd.hash) lvl.push_back(nd);
            else if (lvl.back().mask != nd.mask || std::memcmp(lvl.back().ch, nd.ch, 32) != 0)
                return set_error(ctx, DAGC_ERR_HASH_COLLISION, "64-bit node hash collision between different nodes");
            uid_of[order[i]] = (uint32_t)(lvl.size() - 1);
        }
        std::vector<uint64_t> nh(ng, 0);
        std::vector<uint32_t> nu(ng, kEmptyChild);
        for (uint64_t g = 0; g < ng; ++g)
            if (cand_of[g] >= 0) { nh[g] = cand[cand_of[g]].hash; nu[g] = uid_of[cand_of[g]]; }
        root_hash = nh;
        root_uid = nu;
        top.push_back(std::move(lvl));
        groups = ng;
    }

    // Materialise: top levels (root first), then the merged input levels.
    std::vector<uint64_t> sizes(out_levels);
    for (int t = 0; t < m; ++t) sizes[t] = top[m - 1 - t].size();
    for (int l = 0; l < nl; ++l) sizes[m + l] = counts[kCntUnique + l];
    dagc_dag d = nullptr;
    st = alloc_dag(ctx, out_levels, sizes, counts[kCntLeaves], &d);
    if (st) return st;
    std::vector<uint64_t> th, tm8;
    std::vector<uint32_t> tc;
    for (int t = 0; t < m; ++t) {
        for (const HostNode& nd : top[m - 1 - t]) {
            th.push_back(nd.hash);
            tm8.push_back(nd.mask);
            tc.insert(tc.end(), nd.ch, nd.ch + 8);
        }
    }
    std::vector<uint8_t> tm(tm8.begin(), tm8.end());
    const uint64_t ntop = th.size();
    cudaError_t ce = cudaSuccess;
    if (ntop) {
        ce = cudaMemcpyAsync(d->hashes, th.data(), ntop * 8, cudaMemcpyHostToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->children, tc.data(), ntop * 32, cudaMemcpyHostToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->masks, tm.data(), ntop, cudaMemcpyHostToDevice, s);
    }
    for (int l = 0; l < nl && !ce; ++l) {
        const uint64_t o = d->level_offset[m + l], u = sizes[m + l];
        if (!u) continue;
        ce = cudaMemcpyAsync(d->hashes + o, P64(o_ph[l]), u * 8, cudaMemcpyDeviceToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->children + o * 8, P32(o_pc[l]), u * 32, cudaMemcpyDeviceToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->masks + o, P8(o_pm[l]), u, cudaMemcpyDeviceToDevice, s);
    }
    if (!ce && d->num_leaves) ce = cudaMemcpyAsync(d->leaves, P64(o_PL), d->num_leaves * 8, cudaMemcpyDeviceToDevice, s);
    if (!ce) ce = cudaMemcpyAsync(d->d_level_offset, d->level_offset.data(), (out_levels + 1) * 8, cudaMemcpyHostToDevice, s);
    if (!ce) ce = cudaStreamSynchronize(s);
    if (ce) {
        free_dag(d);
        cudaGetLastError();
        return set_error(ctx, cuda_status(ce), std::string("merge: ") + cudaGetErrorString(ce));
    }
    *out = d;
    return DAGC_OK;
}

// The DAG of a grid of 8^top chunk slots over a union `body` of chunk DAGs
// (its top level holds the chunk roots): slot i holds the chunk whose root
// hash is slot_hash[i] (0: empty). The top levels are built on the host by
// groups of 8 slots in Morton order, as MergeDAGs does
// (src/DAGCompression.cu:1504-1533); the body's levels are copied below them.
int lift_dag(dagc_context ctx, dagc_dag body, const uint64_t* slot_hash, uint64_t slots, cudaStream_t s,
             dagc_dag* out) {
    int m = 0;
    for (uint64_t x = slots; x > 1; x /= 8) ++m;
    const int nl = body->num_levels;
    // The roots in the body: their hashes, ascending (level 0 of a union).
    std::vector<uint64_t> roots;
    const uint64_t nroot = nl > 0 ? body->level_offset[1] : body->num_leaves;
    if (nroot) {
        roots.resize(nroot);
        dag_ready_sync(body);
        DAGC_CUDA(ctx, cudaMemcpy(roots.data(), nl > 0 ? body->hashes : body->leaves, nroot * 8, cudaMemcpyDeviceToHost));
    }
    std::vector<uint64_t> root_hash(slot_hash, slot_hash + slots);
    std::vector<uint32_t> root_uid(slots, kEmptyChild);
    bool any = false;
    for (uint64_t i = 0; i < slots; ++i) {
        if (!root_hash[i]) continue;
        auto it = std::lower_bound(roots.begin(), roots.end(), root_hash[i]);
        if (it == roots.end() || *it != root_hash[i]) return set_error(ctx, DAGC_ERR_BAD_INPUT, "chunk root missing from the body");
        root_uid[i] = (uint32_t)(it - roots.begin());
        any = true;
    }
    const int out_levels = nl + m;
    if (!any) return empty_dag(ctx, out_levels, out);
    std::vector<std::vector<HostNode>> top;
    uint64_t groups = slots;
    while (groups > 1) {
        const uint64_t ng = groups / 8;
        std::vector<HostNode> cand;
        std::vector<int64_t> cand_of(ng, -1);
        for (uint64_t g = 0; g < ng; ++g) {
            HostNode nd{};
            uint64_t hs[8];
            for (int c = 0; c < 8; ++c) {
                hs[c] = root_hash[8 * g + c];
                nd.ch[c] = root_uid[8 * g + c];
                if (hs[c]) nd.mask |= (uint8_t)(1u << c);
            }
            nd.hash = hash_children(hs);
            if (nd.mask) { cand_of[g] = (int64_t)cand.size(); cand.push_back(nd); }
        }
        std::vector<uint32_t> order(cand.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (uint32_t)i;
        std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return cand[a].hash < cand[c].hash; });
        std::vector<HostNode> lvl;
        std::vector<uint32_t> uid_of(cand.size());
        for (size_t i = 0; i < order.size(); ++i) {
            const HostNode& nd = cand[order[i]];
            if (lvl.empty() || lvl.back().hash != nd.hash) lvl.push_back(nd);
            else if (lvl.back().mask != nd.mask || std::memcmp(lvl.back().ch, nd.ch, 32) != 0)
                return set_error(ctx, DAGC_ERR_HASH_COLLISION, "64-bit node hash collision between different nodes");
            uid_of[order[i]] = (uint32_t)(lvl.size() - 1);
        }
        std::vector<uint64_t> nh(ng, 0);
        std::vector<uint32_t> nu(ng, kEmptyChild);
        for (uint64_t g = 0; g < ng; ++g)
            if (cand_of[g] >= 0) { nh[g] = cand[cand_of[g]].hash; nu[g] = uid_of[cand_of[g]]; }
        root_hash = nh;
        root_uid = nu;
        top.push_back(std::move(lvl));
        groups = ng;
    }
    // Nodes of the body no slot reaches stay in it (a union of exactly the
    // slots' chunks has none).
    std::vector<uint64_t> sizes(out_levels);
    for (int t = 0; t < m; ++t) sizes[t] = top[m - 1 - t].size();
    for (int l = 0; l < nl; ++l) sizes[m + l] = body->level_offset[l + 1] - body->level_offset[l];
    dagc_dag d = nullptr;
    int st = alloc_dag(ctx, out_levels, sizes, body->num_leaves, &d);
    if (st) return st;
    std::vector<uint64_t> th;
    std::vector<uint8_t> tm;
    std::vector<uint32_t> tc;
    for (int t = 0; t < m; ++t) {
        for (const HostNode& nd : top[m - 1 - t]) {
            th.push_back(nd.hash);
            tm.push_back(nd.mask);
            tc.insert(tc.end(), nd.ch, nd.ch + 8);
        }
    }
    const uint64_t ntop = th.size(), nbody = body->num_nodes();
    cudaError_t ce = cudaSuccess;
    if (ntop) {
        ce = cudaMemcpyAsync(d->hashes, th.data(), ntop * 8, cudaMemcpyHostToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->children, tc.data(), ntop * 32, cudaMemcpyHostToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->masks, tm.data(), ntop, cudaMemcpyHostToDevice, s);
    }
    if (!ce && nbody) ce = cudaMemcpyAsync(d->hashes + ntop, body->hashes, nbody * 8, cudaMemcpyDeviceToDevice, s);
    if (!ce && nbody) ce = cudaMemcpyAsync(d->children + ntop * 8, body->children, nbody * 32, cudaMemcpyDeviceToDevice, s);
    if (!ce && nbody) ce = cudaMemcpyAsync(d->masks + ntop, body->masks, nbody, cudaMemcpyDeviceToDevice, s);
    if (!ce && d->num_leaves) ce = cudaMemcpyAsync(d->leaves, body->leaves, d->num_leaves * 8, cudaMemcpyDeviceToDevice, s);
    if (!ce) ce = cudaMemcpyAsync(d->d_level_offset, d->level_offset.data(), (out_levels + 1) * 8, cudaMemcpyHostToDevice, s);
    if (!ce) ce = cudaStreamSynchronize(s);
    if (ce) {
        free_dag(d);
        cudaGetLastError();
        return set_error(ctx, cuda_status(ce), std::string("lift: ") + cudaGetErrorString(ce));
    }
    *out = d;
    return DAGC_OK;
}

bool valid_ctx(dagc_context ctx) { return ctx != nullptr; }

}  // namespace

// ===================================================================== C ABI
extern "C" {

int dagc_version(void) { return 1; }

uint64_t dagc_hash_children(const uint64_t* h8) { return h8 ? hash_children(h8) : 0; }

const char* dagc_status_string(int status) {
    switch (status) {
        case DAGC_OK: return "ok";
        case DAGC_ERR_INVALID_ARGUMENT: return "invalid argument";
        case DAGC_ERR_OUT_OF_MEMORY: return "out of device memory";
        case DAGC_ERR_BAD_INPUT: return "bad input";
        case DAGC_ERR_HASH_COLLISION: return "hash collision";
        case DAGC_ERR_DEVICE_TIMEOUT: return "device timeout";
        case DAGC_ERR_CUDA: return "cuda error";
        case DAGC_ERR_TOO_LARGE: return "too large";
        default: return "unknown status";
    }
}

int dagc_context_create(int device, dagc_context* out) {
    if (!out) return DAGC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { cudaGetLastError(); return cuda_status(e); }
    std::unique_ptr<dagc_context_t> c(new dagc_context_t);
    c->device = device;
    c->pool.stats = &c->alloc_stats;
    c->arena.stats = &c->alloc_stats;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    sort_configure();
    kernels_configure();
    e = cudaMallocHost(&c->h_stage, 4096);
    if (e != cudaSuccess) { cudaGetLastError(); return cuda_status(e); }
    if (cudaStreamCreateWithFlags(&c->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        c->capture_stream = nullptr;  // graphs off; calls launch directly
    }
    if (const char* g = std::getenv("DAGC_GRAPHS")) c->use_graphs = std::atoi(g) != 0;
    if (const char* d = std::getenv("DAGC_DEDUP")) c->use_dedup = std::atoi(d) != 0;
    if (const char* gm = std::getenv("DAGC_GROUP")) c->group_mode = std::min(2, std::max(0, std::atoi(gm)));
    if (const char* pd = std::getenv("DAGC_PDL")) c->pdl = std::atoi(pd) != 0;
    if (const char* bp = std::getenv("DAGC_BATCH_PATH")) c->batch_path = std::atoi(bp) != 0;
    // Persistent grid sizes: resident CTAs per SM x SMs.
    for (int sh = 0; sh < kNumKeyShapes; ++sh)
        for (int b = kRadixBits; b <= kMaxRadixBits; ++b)
            c->occ_keys[sh][b - kRadixBits] = std::max(1, occupancy_sort_shape(sh, false, b));
    for (int sh = 0; sh < kNumPairShapes; ++sh) c->occ_pairs[sh] = std::max(1, occupancy_sort_shape(sh, true));
    if (const char* e = std::getenv("DAGC_SORT_SHAPE_KEYS")) c->shape_keys = std::atoi(e) % kNumKeyShapes;
    if (const char* e = std::getenv("DAGC_SORT_SHAPE_PAIRS")) c->shape_pairs = std::atoi(e) % kNumPairShapes;
    if (const char* e = std::getenv("DAGC_SORT_RADIX_BITS")) {
        const int r = std::atoi(e);
        if (r >= kRadixBits && r <= kMaxRadixBits) c->radix_keys = r;
    }
    // The tuning table: the file DAGC_TUNE_FILE names (empty: none), else
    // sort_plans.json of the package (one directory above this library); a
    // missing file leaves the defaults.
    std::string tune_path;
    if (const char* t = std::getenv("DAGC_TUNE_FILE")) {
        tune_path = t;
    } else {
        Dl_info info{};
        if (dladdr(reinterpret_cast<void*>(&dagc_context_create), &info) && info.dli_fname) {
            const std::string lib = info.dli_fname;
            const size_t slash = lib.rfind('/');
            if (slash != std::string::npos) tune_path = lib.substr(0, slash) + "/../sort_plans.json";
        }
    }
    if (!tune_path.empty()) {
        if (FILE* f = std::fopen(tune_path.c_str(), "r")) {
            std::fclose(f);
            if (load_tune_file(c.get(), tune_path.c_str()) == DAGC_OK) c->tune_file = tune_path;
        }
    }
    c->grid_hist = std::max(1, occupancy_sort_histogram()) * c->sms;
    c->grid_leaf = std::max(1, occupancy_kernel(0)) * c->sms;
    if (const char* e = std::getenv("DAGC_SCAN_CTAS_PER_SM"))
        c->grid_leaf = std::min(c->grid_leaf, std::max(1, std::atoi(e)) * c->sms);
    c->grid_extract = std::max(1, occupancy_kernel(1)) * c->sms;
    c->grid_unique = std::max(1, occupancy_kernel(2)) * c->sms;
    c->grid_scan = std::max(1, occupancy_kernel(3)) * c->sms;
    // Grid-stride kernels get the resident CTA count: a second, partial wave
    // of CTAs with full shares would run at a fraction of the occupancy.
    c->grid_write = std::max(1, occupancy_kernel(kKernelFinalWrite)) * c->sms;
    dedup_configure(c->sms);
    group_configure(c->sms);
    chunk_configure(c->sms);
    *out = c.release();
    return DAGC_OK;
}

void dagc_context_destroy(dagc_context ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    settle_profile(ctx);
    for (cudaEvent_t e : ctx->free_events) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->free_sync_events) cudaEventDestroy(e);
    if (ctx->arena_copy) cudaEventDestroy(ctx->arena_copy);
    drop_graphs(ctx);
    if (ctx->capture_stream) cudaStreamDestroy(ctx->capture_stream);
    ctx->arena.release();
    if (ctx->table) cudaFree(ctx->table);
    if (ctx->gtable) cudaFree(ctx->gtable);
    if (ctx->trace_err) cudaFree(ctx->trace_err);
    if (ctx->vox_scratch) cudaFree(ctx->vox_scratch);
    ctx->pool.trim();
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    delete ctx;
}

const char* dagc_last_error(dagc_context ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int dagc_create(dagc_context ctx, const uint64_t* d_fragments, uint64_t n, int depth, void* stream,
                dagc_dag* out) {
    if (!valid_ctx(ctx) || !out) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    if (depth < 2 || depth > kMaxDepth) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "depth must be in [2, 21]");
    if (n > kMaxFragments) return set_error(ctx, DAGC_ERR_TOO_LARGE, "more than 2^31 - 2 fragments");
    if (n && !d_fragments) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null fragments");
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    const int nl = depth - 2;
    if (n == 0) {  // src/DAGCompression.cu:1010-1013
        ctx->last_counts.assign(3 + nl, 0);
        return empty_dag(ctx, nl, out);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    CreatePools p;
    int st = create_pipeline(ctx, d_fragments, n, depth, s, p, nullptr, ctx->use_dedup);
    if (st == kStatusFallback) {
        ++ctx->fallbacks;
        st = create_pipeline(ctx, d_fragments, n, depth, s, p, nullptr, false);
    }
    if (st) return st;
    return materialise(ctx, p, nl, s, out);
}

int dagc_create_batched(dagc_context ctx, const uint64_t* d_fragments, const uint64_t* h_chunk_offsets,
                        const uint64_t* h_chunk_morton, uint64_t k, int chunk_depth, int top_levels, void* stream,
                        dagc_dag* out) {
    if (!valid_ctx(ctx) || !out || !h_chunk_offsets || (k && !h_chunk_morton)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    const int depth = chunk_depth + top_levels;
    if (chunk_depth < 2 || top_levels < 0 || depth > kMaxDepth)
        return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "need chunk_depth >= 2 and chunk_depth + top_levels <= 21");
    if (k == 0 || k > (1ull << (3 * top_levels)) || k > (1u << 20))
        return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "chunk count must be in [1, 8^top_levels]");
    if (h_chunk_offsets[0] != 0) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "chunk offsets must start at 0");
    for (uint64_t i = 0; i < k; ++i) {
        if (h_chunk_offsets[i + 1] < h_chunk_offsets[i])
            return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "chunk offsets must not decrease");
        if (h_chunk_morton[i] >> (3 * top_levels) || (i && h_chunk_morton[i] <= h_chunk_morton[i - 1]))
            return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "chunk Morton indices must ascend inside the grid");
    }
    const uint64_t n = h_chunk_offsets[k];
    if (n > kMaxFragments) return set_error(ctx, DAGC_ERR_TOO_LARGE, "more than 2^31 - 2 fragments");
    if (n && !d_fragments) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null fragments");
    if (3 * chunk_depth + bits_for(k) > 64) return set_error(ctx, DAGC_ERR_TOO_LARGE, "composite key exceeds 64 bits");
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    const int nl = depth - 2;
    if (n == 0) {
        ctx->last_counts.assign(3 + nl, 0);
        return empty_dag(ctx, nl, out);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const BatchSpec batch{h_chunk_offsets, h_chunk_morton, (uint32_t)k, chunk_depth};
    CreatePools p;
    int st = create_pipeline(ctx, d_fragments, n, depth, s, p, &batch, ctx->use_dedup);
    if (st == kStatusFallback) {
        ++ctx->fallbacks;
        st = create_pipeline(ctx, d_fragments, n, depth, s, p, &batch, false);
    }
    if (st) return st;
    return materialise(ctx, p, nl, s, out);
}

uint64_t dagc_create_footprint(uint64_t n, int depth) {
    if (depth < 2 || depth > kMaxDepth || n == 0) return 0;
    const CreateLayout L(n, depth, 0, true, kDedupMaxUnique, true);
    return L.total + L.table_slots * 16 + kGroupScratchBytes;
}

int dagc_dag_num_levels(dagc_dag d, int* num_levels) {
    if (!d || !num_levels) return DAGC_ERR_INVALID_ARGUMENT;
    *num_levels = d->num_levels;
    return DAGC_OK;
}

int dagc_dag_level_size(dagc_dag d, int level, uint64_t* n) {
    if (!d || !n || level < 0 || level >= d->num_levels) return DAGC_ERR_INVALID_ARGUMENT;
    *n = d->level_offset[level + 1] - d->level_offset[level];
    return DAGC_OK;
}

int dagc_dag_num_leaves(dagc_dag d, uint64_t* n) {
    if (!d || !n) return DAGC_ERR_INVALID_ARGUMENT;
    *n = d->num_leaves;
    return DAGC_OK;
}

int dagc_dag_level_device(dagc_dag d, int level, const uint8_t** m, const uint32_t** c, const uint64_t** h) {
    if (!d || level < 0 || level >= d->num_levels) return DAGC_ERR_INVALID_ARGUMENT;
    dag_ready_sync(d);
    const uint64_t o = d->level_offset[level];
    if (m) *m = d->masks + o;
    if (c) *c = d->children + o * 8;
    if (h) *h = d->hashes + o;
    return DAGC_OK;
}

int dagc_dag_leaves_device(dagc_dag d, const uint64_t** leaves) {
    if (!d || !leaves) return DAGC_ERR_INVALID_ARGUMENT;
    dag_ready_sync(d);
    *leaves = d->leaves;
    return DAGC_OK;
}

int dagc_dag_download_level(dagc_dag d, int level, uint8_t* m, uint32_t* c, uint64_t* h) {
    if (!d || level < 0 || level >= d->num_levels) return DAGC_ERR_INVALID_ARGUMENT;
    dagc_context ctx = d->ctx;
    const uint64_t o = d->level_offset[level], u = d->level_offset[level + 1] - o;
    if (!u) return DAGC_OK;
    dag_ready_sync(d);
    if (m) DAGC_CUDA(ctx, cudaMemcpy(m, d->masks + o, u, cudaMemcpyDeviceToHost));
    if (c) DAGC_CUDA(ctx, cudaMemcpy(c, d->children + o * 8, u * 32, cudaMemcpyDeviceToHost));
    if (h) DAGC_CUDA(ctx, cudaMemcpy(h, d->hashes + o, u * 8, cudaMemcpyDeviceToHost));
    return DAGC_OK;
}

int dagc_dag_download_leaves(dagc_dag d, uint64_t* leaves) {
    if (!d || (!leaves && d->num_leaves)) return DAGC_ERR_INVALID_ARGUMENT;
    dag_ready_sync(d);
    if (d->num_leaves) DAGC_CUDA(d->ctx, cudaMemcpy(leaves, d->leaves, d->num_leaves * 8, cudaMemcpyDeviceToHost));
    return DAGC_OK;
}

int dagc_dag_upload(dagc_context ctx, int num_levels, const uint64_t* sizes, const uint8_t* const* m,
                    const uint32_t* const* c, const uint64_t* const* h, const uint64_t* leaves,
                    uint64_t num_leaves, void* stream, dagc_dag* out) {
    if (!valid_ctx(ctx) || !out || num_levels < 0 || num_levels > kMaxDepth - 2 || (num_levels && !sizes))
        return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<uint64_t> sz(sizes, sizes + num_levels);
    // Structural validation on the host, so that no kernel ever indexes out of
    // bounds: children in range of the next level (or the leaves), the mask
    // bit set exactly for the present children, hashes ascending and unique.
    for (int l = 0; l < num_levels; ++l) {
        if (sz[l] && (!m[l] || !c[l] || !h[l])) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null level array");
        const uint64_t next = l + 1 < num_levels ? sz[l + 1] : num_leaves;
        for (uint64_t i = 0; i < sz[l]; ++i) {
            for (int k = 0; k < 8; ++k) {
                const uint32_t ch = c[l][i * 8 + k];
                const bool has = (m[l][i] >> k) & 1;
                if (has != (ch != kEmptyChild) || (has && ch >= next))
                    return set_error(ctx, DAGC_ERR_BAD_INPUT, "malformed DAG level " + std::to_string(l));
            }
            if (i && h[l][i] <= h[l][i - 1]) return set_error(ctx, DAGC_ERR_BAD_INPUT, "level hashes not ascending");
        }
    }
    for (uint64_t i = 1; i < num_leaves; ++i)
        if (leaves[i] <= leaves[i - 1]) return set_error(ctx, DAGC_ERR_BAD_INPUT, "leaves not ascending");
    dagc_dag d = nullptr;
    int st = alloc_dag(ctx, num_levels, sz, num_leaves, &d);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t ce = cudaSuccess;
    for (int l = 0; l < num_levels && !ce; ++l) {
        const uint64_t o = d->level_offset[l], u = sz[l];
        if (!u) continue;
        ce = cudaMemcpyAsync(d->masks + o, m[l], u, cudaMemcpyHostToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->children + o * 8, c[l], u * 32, cudaMemcpyHostToDevice, s);
        if (!ce) ce = cudaMemcpyAsync(d->hashes + o, h[l], u * 8, cudaMemcpyHostToDevice, s);
    }
    if (!ce && num_leaves) ce = cudaMemcpyAsync(d->leaves, leaves, num_leaves * 8, cudaMemcpyHostToDevice, s);
    if (!ce) ce = cudaMemcpyAsync(d->d_level_offset, d->level_offset.data(), (num_levels + 1) * 8, cudaMemcpyHostToDevice, s);
    if (!ce) ce = cudaStreamSynchronize(s);
    if (ce) {
        free_dag(d);
        cudaGetLastError();
        return set_error(ctx, cuda_status(ce), std::string("upload: ") + cudaGetErrorString(ce));
    }
    *out = d;
    return DAGC_OK;
}

int dagc_dag_copy(dagc_context ctx, dagc_dag src, void* stream, dagc_dag* out) {
    if (!valid_ctx(ctx) || !src || !out) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<uint64_t> sizes(src->num_levels);
    for (int l = 0; l < src->num_levels; ++l) sizes[l] = src->level_offset[l + 1] - src->level_offset[l];
    dagc_dag d = nullptr;
    const int st = alloc_dag(ctx, src->num_levels, sizes, src->num_leaves, &d);
    if (st) return st;
    // Same layout: one copy of the whole block.
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t bytes = reinterpret_cast<char*>(d->masks + d->num_nodes()) - reinterpret_cast<char*>(d->block);
    dag_ready_wait(src, s);
    cudaError_t e = cudaMemcpyAsync(d->block, src->block, bytes, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        free_dag(d);
        cudaGetLastError();
        return set_error(ctx, cuda_status(e), std::string("copy: ") + cudaGetErrorString(e));
    }
    *out = d;
    return DAGC_OK;
}

void dagc_dag_free(dagc_dag d) {
    if (!d) return;
    if (d->ctx) {
        std::lock_guard<std::mutex> lock(d->ctx->mu);
        free_dag(d);
    } else {
        delete d;
    }
}

int dagc_merge(dagc_context ctx, dagc_dag* dags, uint64_t k, void* stream, dagc_dag* out) {
    if (!valid_ctx(ctx) || !out || !dags || k == 0) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    uint64_t x = k;
    while (x > 1) {  // src/DAGCompression.cu:1451, :1467
        if (x % 8) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "MergeDAGs needs 8^m inputs");
        x /= 8;
    }
    for (uint64_t i = 0; i < k; ++i) {
        if (!dags[i] || dags[i]->ctx != ctx) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "bad DAG handle");
        if (dags[i]->num_levels != dags[0]->num_levels)
            return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "sub-DAGs of different depths");
    }
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    if (k == 1) { *out = dags[0]; dags[0] = nullptr; return DAGC_OK; }
    const int st = merge_dags(ctx, dags, k, static_cast<cudaStream_t>(stream), out);
    if (st) return st;
    for (uint64_t i = 0; i < k; ++i) { free_dag(dags[i]); dags[i] = nullptr; }
    return DAGC_OK;
}

int dagc_union(dagc_context ctx, dagc_dag* dags, uint64_t k, void* stream, dagc_dag* out, uint64_t* root_hashes) {
    if (!valid_ctx(ctx) || !dags || !out || k == 0) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    for (uint64_t i = 0; i < k; ++i) {
        if (!dags[i]) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null DAG");
        if (dags[i]->num_levels != dags[0]->num_levels) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "depths differ");
    }
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<uint64_t> rh;
    const int st = merge_dags(ctx, dags, k, static_cast<cudaStream_t>(stream), out, true, &rh);
    if (st) return st;
    if (root_hashes)
        for (uint64_t i = 0; i < k; ++i) root_hashes[i] = i < rh.size() ? rh[i] : 0;
    return DAGC_OK;
}

int dagc_dag_lift(dagc_context ctx, dagc_dag body, const uint64_t* slot_root_hashes, uint64_t slots, void* stream,
                  dagc_dag* out) {
    if (!valid_ctx(ctx) || !body || !out || !slot_root_hashes || slots == 0) return DAGC_ERR_INVALID_ARGUMENT;
    uint64_t x = slots;
    while (x % 8 == 0) x /= 8;
    if (x != 1) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "slot count must be a power of 8");
    std::lock_guard<std::mutex> lock(ctx->mu);
    *out = nullptr;
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    int m = 0;
    for (uint64_t y = slots; y > 1; y /= 8) ++m;
    if (body->num_levels + m + 2 > kMaxDepth) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "result deeper than 21");
    return lift_dag(ctx, body, slot_root_hashes, slots, static_cast<cudaStream_t>(stream), out);
}

int dagc_final(dagc_context ctx, dagc_dag dag, void* stream, uint32_t** d_words, uint64_t* n_words) {
    if (!valid_ctx(ctx) || !dag || !d_words || !n_words || dag->ctx != ctx) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    const int st = final_dag(ctx, dag, static_cast<cudaStream_t>(stream), d_words, n_words);
    if (st) return st;
    free_dag(dag);
    return DAGC_OK;
}

int dagc_free_words(dagc_context ctx, uint32_t* d_words, void* stream) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (!d_words) return DAGC_OK;
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    // Work already queued on `stream` (a copy of the words, a kernel reading
    // them) finishes before the block can be handed out again.
    ctx->pool.release_after(d_words, static_cast<cudaStream_t>(stream));
    return DAGC_OK;
}

int dagc_words_download(dagc_context ctx, const uint32_t* d_words, uint64_t n, uint32_t* h_words) {
    if (!valid_ctx(ctx) || (n && (!d_words || !h_words))) return DAGC_ERR_INVALID_ARGUMENT;
    if (n) DAGC_CUDA(ctx, cudaMemcpy(h_words, d_words, n * 4, cudaMemcpyDeviceToHost));
    return DAGC_OK;
}

int dagc_free_all(dagc_context ctx) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    DAGC_CUDA(ctx, cudaDeviceSynchronize());
    drop_graphs(ctx);
    ctx->arena.release();
    if (ctx->table) cudaFree(ctx->table);
    if (ctx->gtable) cudaFree(ctx->gtable);
    ctx->table = nullptr;
    ctx->gtable = nullptr;
    ctx->table_cap = 0;
    ctx->table_dirty = true;
    ctx->pool.trim();
    return DAGC_OK;
}

int dagc_compress(dagc_context ctx, const uint64_t* d_fragments, uint64_t n, int depth, void* stream,
                  uint32_t** d_words, uint64_t* n_words) {
    if (!valid_ctx(ctx) || !d_words || !n_words) return DAGC_ERR_INVALID_ARGUMENT;
    *d_words = nullptr;
    *n_words = 0;
    {
        // The pipeline, then the words from its pools (no DAG in between).
        std::lock_guard<std::mutex> lock(ctx->mu);
        if (depth < 2 || depth > kMaxDepth) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "depth must be in [2, 21]");
        if (n > kMaxFragments) return set_error(ctx, DAGC_ERR_TOO_LARGE, "more than 2^31 - 2 fragments");
        if (n && !d_fragments) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null fragments");
        if (n) {
            DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
            cudaStream_t s = static_cast<cudaStream_t>(stream);
            CreatePools p;
            int st = create_pipeline(ctx, d_fragments, n, depth, s, p, nullptr, ctx->use_dedup);
            if (st == kStatusFallback) {
                ++ctx->fallbacks;
                st = create_pipeline(ctx, d_fragments, n, depth, s, p, nullptr, false);
            }
            if (st) return st;
            bool done = false;
            st = compress_from_pools(ctx, p, depth - 2, s, d_words, n_words, &done);
            if (st || done) return st;
            // The layout's scratch would overlap the pools: copy the DAG out.
            dagc_dag d = nullptr;
            st = materialise(ctx, p, depth - 2, s, &d);
            if (st) return st;
            st = final_dag(ctx, d, s, d_words, n_words);
            free_dag(d);
            return st;
        }
    }
    dagc_dag d = nullptr;
    int st = dagc_create(ctx, d_fragments, n, depth, stream, &d);
    if (st) return st;
    st = dagc_final(ctx, d, stream, d_words, n_words);
    if (st) dagc_dag_free(d);
    return st;
}

int dagc_compress_host(dagc_context ctx, const uint64_t* h_fragments, uint64_t n, int depth, void* stream,
                       uint32_t* h_words, uint64_t capacity, uint64_t* n_words) {
    if (!valid_ctx(ctx) || !n_words || (n && !h_fragments)) return DAGC_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void* d_in = nullptr;
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
        if (n) {
            DAGC_CUDA(ctx, ctx->pool.alloc(&d_in, n * 8, "staged fragments"));
            const cudaError_t e = cudaMemcpyAsync(d_in, h_fragments, n * 8, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) { ctx->pool.release(d_in); DAGC_CUDA(ctx, e); }
        }
    }
    uint32_t* w = nullptr;
    uint64_t nw = 0;
    int st = dagc_compress(ctx, static_cast<const uint64_t*>(d_in), n, depth, stream, &w, &nw);
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        ctx->pool.release(d_in);
    }
    if (st) return st;
    *n_words = nw;
    if (h_words && capacity >= nw && nw) {
        const cudaError_t e = cudaMemcpyAsync(h_words, w, nw * 4, cudaMemcpyDeviceToHost, s);
        const cudaError_t e2 = e == cudaSuccess ? cudaStreamSynchronize(s) : e;
        dagc_free_words(ctx, w, stream);
        if (e2 != cudaSuccess) { cudaGetLastError(); return set_error(ctx, cuda_status(e2), cudaGetErrorString(e2)); }
        return DAGC_OK;
    }
    dagc_free_words(ctx, w, stream);
    return h_words && capacity < nw ? set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "word buffer too small") : DAGC_OK;
}

int dagc_set_option(dagc_context ctx, int option, int value) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    switch (option) {
        case DAGC_OPT_SORT_SHAPE_KEYS:
            if (value < -1 || value >= kNumKeyShapes) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "bad shape");
            ctx->shape_keys = value;
            ++ctx->tune_version;
            return DAGC_OK;
        case DAGC_OPT_SORT_SHAPE_PAIRS:
            if (value < -1 || value >= kNumPairShapes) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "bad shape");
            ctx->shape_pairs = value;
            ++ctx->tune_version;
            return DAGC_OK;
        case DAGC_OPT_SORT_RADIX_BITS:
            if (value != -1 && (value < kRadixBits || value > kMaxRadixBits))
                return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "digit width must be -1 or 8..11");
            ctx->radix_keys = value;
            ++ctx->tune_version;
            return DAGC_OK;
        case DAGC_OPT_GRAPHS:
            ctx->use_graphs = value != 0;
            if (!ctx->use_graphs) drop_graphs(ctx);
            return DAGC_OK;
        case DAGC_OPT_DEDUP:
            ctx->use_dedup = value != 0;
            return DAGC_OK;
        case DAGC_OPT_PDL:
            if (ctx->pdl != (value != 0)) drop_graphs(ctx);  // recorded graphs keep their launch attributes
            ctx->pdl = value != 0;
            return DAGC_OK;
        case DAGC_OPT_GROUP:
            if (value < 0 || value > 2) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "group mode must be 0, 1 or 2");
            ctx->group_mode = value;
            return DAGC_OK;
        case DAGC_OPT_BATCH_PATH:
            if (value < 0 || value > 1) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "batch path must be 0 or 1");
            ctx->batch_path = value;
            return DAGC_OK;
        case DAGC_OPT_TEST_SPIN_LIMIT:
            if (value < 0) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "spin limit must be >= 0");
            ctx->test_spin_limit = (uint32_t)value;
            ++ctx->tune_version;  // recorded graphs carry the old value
            return DAGC_OK;
        case DAGC_OPT_TEST_STALL_LOOKBACK:
            ctx->test_stall = value != 0;
            ++ctx->tune_version;
            return DAGC_OK;
        case DAGC_OPT_TEST_FAIL_ALLOCS:
            if (value < 0) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "count must be >= 0");
            ctx->alloc_stats.inject = value;
            return DAGC_OK;
        case DAGC_OPT_DEDUP_UNIQUE_LIMIT:
            if (value < 1) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "limit must be positive");
            ctx->dedup_unique_limit = (uint64_t)value;
            drop_graphs(ctx);
            return DAGC_OK;
        default:
            return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "unknown option");
    }
}

int dagc_profile_enable(dagc_context ctx, int enable) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->profiling = enable != 0;
    return DAGC_OK;
}

int dagc_profile_reset(dagc_context ctx) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    for (auto& st : ctx->stages) st = StageStats{};
    return DAGC_OK;
}

int dagc_profile_read(dagc_context ctx, int stage, double* ms, uint64_t* launches, uint64_t* bytes) {
    if (!valid_ctx(ctx) || stage < 0 || stage >= DAGC_NUM_STAGES) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    const StageStats& st = ctx->stages[stage];
    if (ms) *ms = st.ms;
    if (launches) *launches = st.launches;
    if (bytes) *bytes = st.bytes;
    return DAGC_OK;
}

int dagc_memory_report(dagc_context ctx, char* buf, uint64_t capacity, uint64_t* needed) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::string out;
    {
        std::lock_guard<std::mutex> lock(ctx->mu);
        std::map<std::string, std::pair<uint64_t, uint64_t>> m;
        ctx->pool.tally(m);
        if (ctx->arena.cap) m["scratch arena"] = {ctx->arena.cap, 1};
        if (ctx->table_cap) m["dedup table"] = {ctx->table_cap * 16, 1};
        if (ctx->gtable) m["grouping table"] = {kGroupScratchBytes, 1};
        uint64_t total = 0;
        for (const auto& kv : m) total += kv.second.first;
        std::vector<std::pair<std::string, std::pair<uint64_t, uint64_t>>> list(m.begin(), m.end());
        std::sort(list.begin(), list.end(), [](const auto& a, const auto& b) { return a.second.first > b.second.first; });
        char line[256];
        std::snprintf(line, sizeof(line), "GPU memory: %.3f MB\nPeak of DAG and word blocks: %.3f MB\n\nAllocations overview:\n",
                      total / 1048576.0, ctx->pool.peak() / 1048576.0);
        out += line;
        for (const auto& kv : list) {
            std::snprintf(line, sizeof(line), "\t%24s: %12.3f MB (%llu allocs)\n", kv.first.c_str(),
                          kv.second.first / 1048576.0, (unsigned long long)kv.second.second);
            out += line;
        }
    }
    if (needed) *needed = out.size() + 1;
    if (buf && capacity) {
        const size_t k = std::min<size_t>(capacity - 1, out.size());
        std::memcpy(buf, out.data(), k);
        buf[k] = 0;
    }
    return DAGC_OK;
}

int dagc_memory_events(dagc_context ctx, uint64_t* alloc_failures, uint64_t* retries_ok) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (alloc_failures) *alloc_failures = ctx->alloc_stats.failures;
    if (retries_ok) *retries_ok = ctx->alloc_stats.retries_ok;
    return DAGC_OK;
}

int dagc_memory_stats(dagc_context ctx, uint64_t* in_use, uint64_t* peak, uint64_t* cached, uint64_t* arena) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (in_use) *in_use = ctx->pool.in_use();
    if (peak) *peak = ctx->pool.peak();
    if (cached) *cached = ctx->pool.cached();
    if (arena) *arena = ctx->arena.cap;
    return DAGC_OK;
}

int dagc_trace_camera(const double position[3], const double right[3], const double up[3], const double forward[3],
                      double fov_degrees, uint32_t width, uint32_t height, const double aabb_min[3],
                      const double aabb_max[3], int depth, uint32_t debug_level, dagc_trace_params* out) {
    if (!position || !right || !up || !forward || !aabb_min || !aabb_max || !out || !width || !height ||
        depth < 3 || depth > kMaxDepth)
        return DAGC_ERR_INVALID_ARGUMENT;
    const double fov = fov_degrees / 2.0 * (3.14159265358979323846 / 180.);
    const double aspect = double(width) / double(height);
    const double sf = std::sin(fov), cf = std::cos(fov);
    double bl[3], br[3], tl[3], cam[3];
    for (int i = 0; i < 3; ++i) {
        const double x = right[i] * sf * aspect, y = up[i] * sf, z = forward[i] * cf;
        bl[i] = position[i] + z - y - x;
        br[i] = position[i] + z - y + x;
        tl[i] = position[i] + z + y - x;
        const double scale = double(1u << depth) / (aabb_max[i] - aabb_min[i]);
        const double t = -aabb_min[i];
        cam[i] = (position[i] + t) * scale;
        bl[i] = (bl[i] + t) * scale;
        br[i] = (br[i] + t) * scale;
        tl[i] = (tl[i] + t) * scale;
    }
    dagc_trace_params p{};
    p.debug_level = debug_level;
    p.width = width;
    p.height = height;
    for (int i = 0; i < 3; ++i) {
        p.camera[i] = cam[i];
        p.ray_min[i] = bl[i];
        p.ray_ddx[i] = (br[i] - bl[i]) * (1.0 / width);
        p.ray_ddy[i] = (tl[i] - bl[i]) * (1.0 / height);
    }
    *out = p;
    return DAGC_OK;
}

int dagc_trace(dagc_context ctx, const uint32_t* d_words, uint64_t n_words, int depth,
               const dagc_trace_params* params, uint32_t* d_colors, uint64_t* d_hits, void* stream) {
    if (!valid_ctx(ctx) || !params) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (depth < 3 || depth > kMaxDepth) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "depth must be in [3, 21]");
    const uint64_t pixels = (uint64_t)params->width * params->height;
    if (pixels == 0) return DAGC_OK;
    if (!d_colors || !d_words || n_words == 0) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null buffers");
    if (params->width > 65535u * 8u || params->height > 65535u * 16u)
        return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "image too large");
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!ctx->trace_err) DAGC_CUDA(ctx, cudaMalloc(&ctx->trace_err, 256));
    DAGC_CUDA(ctx, cudaMemsetAsync(ctx->trace_err, 0, 4, s));
    TraceArgs a{};
    a.words = d_words;
    a.n_words = n_words;
    a.depth = depth;
    a.debug_level = params->debug_level;
    a.width = params->width;
    a.height = params->height;
    for (int i = 0; i < 3; ++i) {
        a.camera[i] = params->camera[i];
        a.ray_min[i] = params->ray_min[i];
        a.ray_ddx[i] = params->ray_ddx[i];
        a.ray_ddy[i] = params->ray_ddy[i];
    }
    a.colors = d_colors;
    a.hits = d_hits;
    a.err = ctx->trace_err;
    launch_trace(a, s);
    ++ctx->launches;
    DAGC_LAUNCHED(ctx);
    uint32_t err = 0;
    DAGC_CUDA(ctx, cudaMemcpyAsync(&err, ctx->trace_err, 4, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaStreamSynchronize(s));
    if (err) return set_error(ctx, DAGC_ERR_BAD_INPUT, "the word array is not a valid final DAG of this depth");
    return DAGC_OK;
}

int dagc_voxelize(dagc_context ctx, const double* d_vertices, uint64_t n_triangles, const double aabb[6], int depth,
                  int mode, uint64_t* d_codes, uint64_t capacity, uint64_t* n_codes, void* stream) {
    if (!valid_ctx(ctx) || !aabb || !n_codes) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *n_codes = 0;
    if (depth < 1 || depth > kMaxDepth) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "depth must be in [1, 21]");
    if (mode != DAGC_VOXELIZE_GL && mode != DAGC_VOXELIZE_SAT)
        return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "unknown voxelization mode");
    for (int a = 0; a < 3; ++a)
        if (!(aabb[3 + a] > aabb[a])) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "empty box");
    if (n_triangles == 0) return DAGC_OK;
    if (!d_vertices || (capacity && !d_codes)) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "null buffers");
    if (n_triangles > (1ull << 36)) return set_error(ctx, DAGC_ERR_TOO_LARGE, "too many triangles");
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Scratch: total, tile counter, error word, look-back status per tile.
    const uint64_t tiles = voxelize_tiles(n_triangles);
    const size_t bytes = 64 + (tiles + 1) * 8;
    if (bytes > ctx->vox_scratch_bytes) {
        if (ctx->vox_scratch) cudaFree(ctx->vox_scratch);
        ctx->vox_scratch = nullptr;
        ctx->vox_scratch_bytes = 0;
        DAGC_CUDA(ctx, cudaMalloc(&ctx->vox_scratch, bytes));
        ctx->vox_scratch_bytes = bytes;
    }
    char* b = static_cast<char*>(ctx->vox_scratch);
    DAGC_CUDA(ctx, cudaMemsetAsync(b, 0, bytes, s));
    VoxArgs a{};
    a.vertices = d_vertices;
    a.n_tri = n_triangles;
    for (int i = 0; i < 6; ++i) a.aabb[i] = aabb[i];
    a.depth = depth;
    a.mode = mode;
    a.codes = d_codes;
    a.capacity = capacity;
    a.d_total = reinterpret_cast<uint64_t*>(b);
    a.tile_counter = reinterpret_cast<uint32_t*>(b + 8);
    a.err = reinterpret_cast<uint32_t*>(b + 16);
    a.status = reinterpret_cast<uint64_t*>(b + 64);
    const int grid = (int)std::min<uint64_t>(tiles, (uint64_t)ctx->sms * 8);
    launch_voxelize(a, grid, s);
    ++ctx->launches;
    DAGC_LAUNCHED(ctx);
    uint64_t h[3] = {0, 0, 0};
    DAGC_CUDA(ctx, cudaMemcpyAsync(h, b, 24, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaStreamSynchronize(s));
    if ((uint32_t)h[2]) return set_error(ctx, DAGC_ERR_DEVICE_TIMEOUT, "a bounded device wait ran out");
    *n_codes = h[0];
    if (h[0] > capacity) return set_error(ctx, DAGC_ERR_TOO_LARGE, "fragment buffer too small (see n_codes)");
    return DAGC_OK;
}

int dagc_dedup_fallbacks(dagc_context ctx, uint64_t* count) {
    if (!valid_ctx(ctx) || !count) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    *count = ctx->fallbacks;
    return DAGC_OK;
}

int dagc_kernel_launches(dagc_context ctx, uint64_t* launches) {
    if (!valid_ctx(ctx) || !launches) return DAGC_ERR_INVALID_ARGUMENT;
    *launches = ctx->launches;
    return DAGC_OK;
}

int dagc_last_counts(dagc_context ctx, uint64_t* out, int cap) {
    if (!valid_ctx(ctx) || (!out && cap > 0)) return 0;
    const int k = std::min<int>(cap, (int)ctx->last_counts.size());
    for (int i = 0; i < k; ++i) out[i] = ctx->last_counts[i];
    return k;
}

}  // extern "C"

namespace {

// One standalone sort enqueued on `s` through the context's arena (no wait).
int enqueue_sort(dagc_context ctx, const uint64_t* d_keys_in, uint64_t* d_keys_out, const uint32_t* d_vals_in,
                 uint32_t* d_vals_out, uint64_t n, int lo, int hi, cudaStream_t s) {
    const bool with_values = d_vals_out != nullptr;
    Layout L;
    const size_t o_hdr = L.take<CallHeader>(1);
    const size_t zero_bytes = L.off;
    const size_t o_ss0 = L.take<uint32_t>(sort_status_words(n));
    const size_t o_ss1 = L.take<uint32_t>(sort_status_words(n));
    const size_t o_ka = L.take<uint64_t>(n);
    const size_t o_va = L.take<uint32_t>(with_values ? n : 0);
    DAGC_CUDA(ctx, ctx->arena.reserve(L.off));
    arena_wait(ctx, s);
    char* b = static_cast<char*>(ctx->arena.base);
    CallSlots cs;
    cs.h = reinterpret_cast<CallHeader*>(b + o_hdr);
    SortBuffers sb{{reinterpret_cast<uint32_t*>(b + o_ss0), reinterpret_cast<uint32_t*>(b + o_ss1)}};
    DAGC_CUDA(ctx, cudaMemsetAsync(b, 0, zero_bytes, s));
    ctx->sort_err = &cs.h->err;
    return run_sort(ctx, cs, sb, d_keys_in, d_keys_out, reinterpret_cast<uint64_t*>(b + o_ka), d_vals_in, d_vals_out,
                    with_values ? reinterpret_cast<uint32_t*>(b + o_va) : nullptr, with_values, n, nullptr, lo, hi, 0,
                    s);
}

// Waits for the sorts enqueued on `s` and maps their error word to a status.
int finish_sort(dagc_context ctx, cudaStream_t s) {
    DAGC_CUDA(ctx, cudaMemcpyAsync(ctx->h_stage, ctx->sort_err, 8, cudaMemcpyDeviceToHost, s));
    DAGC_CUDA(ctx, cudaStreamSynchronize(s));
    std::string msg;
    const int st = device_error_status((uint32_t)ctx->h_stage[0], msg);
    return st ? set_error(ctx, st, msg) : DAGC_OK;
}

// Tuning table file: JSON, one object per sort class.
int save_tune_file(dagc_context ctx, const char* path) {
    FILE* f = std::fopen(path, "w");
    if (!f) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, ctx->device);
    cudaGetLastError();
    std::fprintf(f, "{\n  \"format\": \"dagc digit-pass plans\",\n  \"version\": 1,\n  \"device\": \"%s\",\n"
                    "  \"sm\": %d,\n  \"entries\": [",
                 prop.name, prop.major * 10 + prop.minor);
    bool first = true;
    for (const auto& kv : ctx->tune) {
        const uint32_t cls = kv.first;
        auto m = ctx->tune_ms.find(cls);
        const double ms = m == ctx->tune_ms.end() ? 0.0 : m->second.first;
        const double dms = m == ctx->tune_ms.end() ? 0.0 : m->second.second;
        std::fprintf(f,
                     "%s\n    {\"values\": %u, \"bits\": %u, \"log2n\": %u, \"shape\": %d, \"radix_bits\": %d, "
                     "\"ms\": %.6f, \"default_ms\": %.6f}",
                     first ? "" : ",", cls >> 24, (cls >> 8) & 0xFFu, cls & 0xFFu, kv.second.shape,
                     kv.second.radix_bits, ms, dms);
        first = false;
    }
    std::fprintf(f, "\n  ]\n}\n");
    const bool ok = std::fclose(f) == 0;
    return ok ? DAGC_OK : set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, std::string("cannot write ") + path);
}

// Number after `"key":` inside [b, e), or `fallback`.
double json_number(const char* b, const char* e, const char* key, double fallback) {
    const std::string pat = std::string("\"") + key + "\":";
    const char* p = std::search(b, e, pat.begin(), pat.end());
    if (p == e) return fallback;
    return std::strtod(p + pat.size(), nullptr);
}

int load_tune_file(dagc_context ctx, const char* path) {
    FILE* f = std::fopen(path, "r");
    if (!f) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, std::string("cannot read ") + path);
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    std::fclose(f);
    const size_t ent = text.find("\"entries\"");
    if (ent == std::string::npos) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "no entries in tuning file");
    std::map<uint32_t, SortChoice> table;
    std::map<uint32_t, std::pair<double, double>> times;
    size_t pos = ent;
    while ((pos = text.find('{', pos)) != std::string::npos) {
        const size_t close = text.find('}', pos);
        if (close == std::string::npos) break;
        const char* b = text.data() + pos;
        const char* e = text.data() + close;
        const int values = (int)json_number(b, e, "values", -1), bits = (int)json_number(b, e, "bits", -1);
        const int lg = (int)json_number(b, e, "log2n", -1), shape = (int)json_number(b, e, "shape", -1);
        const int rb = (int)json_number(b, e, "radix_bits", -1);
        pos = close + 1;
        if (values < 0 || values > 1 || bits < 1 || bits > 64 || lg < 0 || lg > 40) continue;
        if (!sort_plan_valid(shape, values != 0, rb, 0, bits)) continue;  // not a plan of this build: skipped
        const uint32_t cls = (values ? 1u << 24 : 0u) | (uint32_t)bits << 8 | (uint32_t)lg;
        table[cls] = SortChoice{shape, rb};
        times[cls] = {json_number(b, e, "ms", 0), json_number(b, e, "default_ms", 0)};
    }
    ctx->tune.swap(table);
    ctx->tune_ms.swap(times);
    ++ctx->tune_version;
    return DAGC_OK;
}

}  // namespace

extern "C" {

int dagc_sort_keys(dagc_context ctx, const uint64_t* d_in, uint64_t* d_out, uint64_t n, int lo, int hi, void* stream) {
    return dagc_sort_pairs(ctx, d_in, d_out, nullptr, nullptr, n, lo, hi, stream);
}

int dagc_sort_pairs(dagc_context ctx, const uint64_t* d_keys_in, uint64_t* d_keys_out, const uint32_t* d_vals_in,
                    uint32_t* d_vals_out, uint64_t n, int lo, int hi, void* stream) {
    if (!valid_ctx(ctx) || lo < 0 || hi > 64 || lo > hi) return DAGC_ERR_INVALID_ARGUMENT;
    if (n > kMaxFragments) return set_error(ctx, DAGC_ERR_TOO_LARGE, "more than 2^31 - 2 keys");
    if (n == 0) return DAGC_OK;
    if (!d_keys_in || !d_keys_out || d_keys_in == d_keys_out) return set_error(ctx, DAGC_ERR_INVALID_ARGUMENT, "bad key buffers");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int st = enqueue_sort(ctx, d_keys_in, d_keys_out, d_vals_in, d_vals_out, n, lo, hi, s);
    if (st) return st;
    return finish_sort(ctx, s);
}

int dagc_sort_plan(dagc_context ctx, uint64_t n, int lo_bit, int hi_bit, int with_values, int* shape,
                   int* radix_bits) {
    if (!valid_ctx(ctx) || lo_bit < 0 || hi_bit > 64 || lo_bit > hi_bit || !shape || !radix_bits)
        return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    const SortChoice c = sort_plan_for(ctx, with_values != 0, lo_bit, hi_bit, n);
    *shape = c.shape;
    *radix_bits = c.radix_bits;
    return DAGC_OK;
}

int dagc_tune_sort(dagc_context ctx, uint64_t n, int lo_bit, int hi_bit, int with_values, int reps, int* best_shape,
                   int* best_radix_bits, double* best_ms, double* default_ms) {
    if (!valid_ctx(ctx) || lo_bit < 0 || hi_bit > 64 || lo_bit >= hi_bit || n == 0 || reps < 1)
        return DAGC_ERR_INVALID_ARGUMENT;
    if (n > kMaxFragments) return set_error(ctx, DAGC_ERR_TOO_LARGE, "more than 2^31 - 2 keys");
    std::lock_guard<std::mutex> lock(ctx->mu);
    DAGC_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool values = with_values != 0;
    cudaStream_t s = ctx->capture_stream;  // a stream of the context's own, idle between calls
    void *kin = nullptr, *kout = nullptr, *vout = nullptr;
    DAGC_CUDA(ctx, ctx->pool.alloc(&kin, n * 8, "tuning keys"));
    int st = DAGC_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(s);
        ctx->pool.release(kin);
        ctx->pool.release(kout);
        ctx->pool.release(vout);
        ctx->plan_override = nullptr;
    };
    if (ctx->pool.alloc(&kout, n * 8, "tuning keys") != cudaSuccess ||
        (values && ctx->pool.alloc(&vout, n * 4, "tuning keys") != cudaSuccess)) {
        cudaGetLastError();
        cleanup();
        return set_error(ctx, DAGC_ERR_OUT_OF_MEMORY, "tuning buffers");
    }
    launch_fill_tune_keys(static_cast<uint64_t*>(kin), n, lo_bit, hi_bit, 0x7E57C0DEull + n, s);
    cudaEvent_t e0 = take_event(ctx), e1 = take_event(ctx);
    if (!e0 || !e1) { cleanup(); return set_error(ctx, DAGC_ERR_CUDA, "events"); }
    // Times one plan: one untimed sort, then `reps` sorts between two events.
    auto time_plan = [&](SortChoice c, double* ms) -> int {
        ctx->plan_override = &c;
        for (int r = 0; r <= reps; ++r) {
            if (r == 1) cudaEventRecord(e0, s);
            const int e = enqueue_sort(ctx, static_cast<uint64_t*>(kin), static_cast<uint64_t*>(kout), nullptr,
                                       static_cast<uint32_t*>(vout), n, lo_bit, hi_bit, s);
            if (e) { ctx->plan_override = nullptr; return e; }
        }
        cudaEventRecord(e1, s);
        ctx->plan_override = nullptr;
        const int e = finish_sort(ctx, s);
        if (e) return e;
        float f = 0;
        DAGC_CUDA(ctx, cudaEventElapsedTime(&f, e0, e1));
        *ms = f / reps;
        return DAGC_OK;
    };
    const SortChoice def = values ? kDefaultPairs : kDefaultKeys;
    double dms = 0;
    st = time_plan(def, &dms);
    SortChoice best = def;
    double bms = dms;
    const int shapes = values ? kNumPairShapes : kNumKeyShapes;
    const int max_bits = values ? kRadixBits : kMaxRadixBits;
    for (int sh = 0; sh < shapes && !st; ++sh) {
        for (int b = kRadixBits; b <= max_bits && !st; ++b) {
            if (!sort_plan_valid(sh, values, b, lo_bit, hi_bit)) continue;
            // Wider digits only where they save a pass.
            if (b > kRadixBits && sort_passes_r(lo_bit, hi_bit, b) == sort_passes_r(lo_bit, hi_bit, b - 1)) continue;
            double ms = 0;
            st = time_plan(SortChoice{sh, b}, &ms);
            if (!st && ms < bms) { bms = ms; best = SortChoice{sh, b}; }
        }
    }
    ctx->free_events.push_back(e0);
    ctx->free_events.push_back(e1);
    cleanup();
    if (st) return st;
    const uint32_t cls = sort_class(values, hi_bit - lo_bit, n);
    ctx->tune[cls] = best;
    ctx->tune_ms[cls] = {bms, dms};
    ++ctx->tune_version;
    if (best_shape) *best_shape = best.shape;
    if (best_radix_bits) *best_radix_bits = best.radix_bits;
    if (best_ms) *best_ms = bms;
    if (default_ms) *default_ms = dms;
    return DAGC_OK;
}

int dagc_tune_save(dagc_context ctx, const char* path) {
    if (!valid_ctx(ctx) || !path) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    return save_tune_file(ctx, path);
}

int dagc_tune_load(dagc_context ctx, const char* path) {
    if (!valid_ctx(ctx) || !path) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    return load_tune_file(ctx, path);
}

int dagc_tune_clear(dagc_context ctx) {
    if (!valid_ctx(ctx)) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    ctx->tune.clear();
    ctx->tune_ms.clear();
    ++ctx->tune_version;
    return DAGC_OK;
}

}  // extern "C"
