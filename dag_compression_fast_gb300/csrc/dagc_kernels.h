// Host-side declarations of the dagc kernel launchers (implemented in the .cu
// files). Plain C++: the orchestrator (dagc.cpp) includes this header only.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dagc_hash.h"  // DAGC_HD

namespace dagc {

// ------------------------------------------------------------ error bits ----
// Kernels never trap: they OR one of these into the call's error word and
// carry on with a defined (if meaningless) value so that every wait still ends.
enum : uint32_t {
    kErrBadInput = 1u,      // fragment code >= 2^(3*depth)
    kErrCollision = 2u,     // equal 64-bit hash, different node
    kErrTimeout = 4u,       // a bounded wait ran out
    kErrCapacity = 8u,      // an upper bound on a buffer was exceeded
    kErrNotRooted = 16u,    // level 0 does not hold exactly one node
    kErrMergeRoot = 32u,    // a sub-DAG root hash missing from the merged level
    kErrFallback = 64u,     // the hash-set dedup could not hold a level: rerun with the radix form
};

constexpr uint32_t kEmptyChild = 0xFFFFFFFFu;


// ---------------------------------------------------------------- sort ----
constexpr int kSortThreads = 256;
// Digit-pass tiles hold 256 threads x (8..16) keys.
constexpr int kSortTile = 2048;
constexpr int kRadixBits = 8;       // default digit width
constexpr int kMaxRadixBits = 11;   // widest digit a keys-only pass takes
constexpr int kMaxPasses = 8;
constexpr int kSortHistWords = 8192;  // one sort's histograms: passes x 2^(widest digit)

DAGC_HD uint32_t sort_tiles(uint64_t n) { return (uint32_t)((n + kSortTile - 1) / kSortTile); }
// Look-back status words of one digit pass for n keys, enough for every pass
// shape: tiles of at least 2048 keys with 256 digits, or of at least 4096
// keys with up to 2048 digits.
DAGC_HD uint64_t sort_status_words(uint64_t n) { return ((n + 4095) / 4096 + 1) * 2048; }

// Digits of a sort over bits [lo, hi) in `passes` passes: widths differ by at
// most one, the wider ones first; pass i covers bits [shift, shift + bits).
DAGC_HD int sort_passes_r(int lo_bit, int hi_bit, int radix_bits) {
    return hi_bit > lo_bit ? (hi_bit - lo_bit + radix_bits - 1) / radix_bits : 0;
}
DAGC_HD void pass_digit(int lo_bit, int hi_bit, int passes, int i, int* shift, int* bits) {
    const int b = hi_bit - lo_bit, w = b / passes, extra = b % passes;
    *bits = w + (i < extra ? 1 : 0);
    *shift = lo_bit + i * w + (i < extra ? i : extra);
}
// Histogram words between consecutive passes: 2^(widest digit).
DAGC_HD int pass_hist_stride(int lo_bit, int hi_bit, int passes) {
    const int b = hi_bit - lo_bit;
    return passes > 0 ? 1 << ((b + passes - 1) / passes) : 0;
}
// Number of digit passes for a bit range at the default width.
DAGC_HD int sort_passes(int lo_bit, int hi_bit) { return sort_passes_r(lo_bit, hi_bit, kRadixBits); }

// Device count pointer convention: when d_n is non-null the kernels read the
// element count from device memory (written by an earlier kernel) and n is an
// upper bound used only to size the grid; otherwise n is the count.
struct SortArgs {
    const uint64_t* keys_in;
    uint64_t* keys_out;
    uint64_t* keys_alt;       // ping-pong buffer (n elements)
    const uint32_t* vals_in;  // null with with_values -> values are 0..n-1
    uint32_t* vals_out;
    uint32_t* vals_alt;
    bool with_values;
    uint64_t n;               // count or upper bound (see d_n)
    const uint64_t* d_n;
    int lo_bit, hi_bit;
    int radix_bits;           // widest digit (8..11; keys only above 8); 0 = 8
    int validate_bits;        // > 0: flag keys with bits >= validate_bits set
    uint32_t* hist;           // kSortHistWords words, zeroed
    uint32_t* status[2];      // 2 x sort_status_words(n) words; status[0] zeroed on entry
    uint32_t* tile_counters;  // kMaxPasses words, zeroed
    uint32_t* err;
    int grid_hist, grid_pass; // persistent grid sizes
    int shape;                // digit-pass kernel shape (a key shape or a pair shape)
    // Gate: when non-null, every kernel of the sort does nothing unless
    // *gate == gate_run (a path chosen on the device, see GroupArgs).
    const uint32_t* gate; uint32_t gate_run;
    // Segmented input (batched chunks): when seg_offsets is non-null, the key at
    // position i of keys_in belongs to segment s with seg_offsets[s] <= i <
    // seg_offsets[s+1] (seg_count + 1 ascending entries) and is sorted as the
    // composite (s << seg_shift) | key. Only the histogram and the first pass
    // read keys_in; they build the composite, later passes move it.
    const uint64_t* seg_offsets;
    uint32_t seg_count;
    int seg_shift;
    // Failure-path test hooks (zero in production): a lower limit on the
    // look-back waits (0 = kSpinLimit), and a first digit pass whose tile 0
    // never publishes its counts, so that the waits of the tiles after it run
    // out and the sort reports kErrTimeout.
    uint32_t spin_limit;
    int stall_first_tile;
};

// Digit-pass kernel shapes. Keys-only sorts: (items per thread, minimum
// resident CTAs per SM, which caps registers, equal-digit matching: ballots,
// match.any, alternating, shared-memory atomicOr); each is
// built for every digit width 8..kMaxRadixBits. Key/value sorts: 8-bit
// digits. The autotuner and dagc options pick a shape and a width per sort.
constexpr int kNumKeyShapes = 9;
constexpr int kNumPairShapes = 10;
constexpr int kNumSortShapes = kNumPairShapes;
int sort_shape_items(int shape, bool with_values);
// Resident CTAs per SM of a shape at a digit width (occupancy query) for grid sizing.
int occupancy_sort_shape(int shape, bool with_values, int radix_bits = kRadixBits);
int occupancy_sort_histogram();
// One-CTA sort of up to kSmallSortMax 64-bit keys (all 64 bits) held in
// shared memory, keys_in -> keys_out, when the device count *d_n fits; sets
// *done to 1 then (a grid-wide sort gated on *done == 0 then does nothing).
constexpr uint32_t kSmallSortMax = 12288;
void launch_small_sort(const uint64_t* keys_in, uint64_t* keys_out, const uint64_t* d_n, uint64_t n_bound,
                       uint32_t* done, cudaStream_t s);
// Whether a (shape, width) plan can sort bits [lo, hi): histogram room and
// look-back status room.
bool sort_plan_valid(int shape, bool with_values, int radix_bits, int lo_bit, int hi_bit);

// Where the result lands: keys_out always (the pass sequence is arranged so).
void launch_sort(const SortArgs& a, cudaStream_t s);
// The same, one launch at a time: histogram (+ copy when there is no digit),
// then digit pass i for i in [0, sort_plan_passes(a)).
int sort_plan_passes(const SortArgs& a);
void launch_sort_histogram(const SortArgs& a, cudaStream_t s);
void launch_sort_pass(const SortArgs& a, int i, cudaStream_t s);
void sort_configure();  // sets shared-memory attributes once per device
// Autotuner input: n pseudo-random keys with bits only in [lo_bit, hi_bit).
void launch_fill_tune_keys(uint64_t* out, uint64_t n, int lo_bit, int hi_bit, uint64_t seed, cudaStream_t s);

// ---------------------------------------------------------- DAG kernels ----
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
DAGC_HD uint32_t scan_tiles(uint64_t n) { return (uint32_t)((n + kScanTile - 1) / kScanTile); }
// leaf_build takes 8192 sorted keys per tile (its per-tile arrays, sized by
// scan_tiles, are large enough).
constexpr int kLeafTile = 8192;
DAGC_HD uint32_t leaf_tiles(uint64_t n) { return (uint32_t)((n + kLeafTile - 1) / kLeafTile); }

// Fused unique + 4x4x4 leaf build over fragments sorted by (code >> 6):
// parents[p] = code >> 6 and leaves[p] = OR of 1 << (code & 63) per distinct
// parent; *d_out_n = number of parents.
struct LeafBuildArgs {
    const uint64_t* sorted; const uint64_t* d_n; uint64_t n_bound;
    // Batched input: sorted keys are (segment << seg_shift) | local code; the
    // global code is (seg_code[segment] << seg_shift) | local code.
    const uint64_t* seg_code; int seg_shift;
    uint64_t* parents; uint64_t* leaves; uint64_t out_capacity; uint64_t* d_out_n;
    uint64_t* lead_or; uint64_t* lead_run;  // per tile: OR of keys continuing an earlier run, its run id
    uint64_t* status; uint32_t* tile_counter; uint32_t* err; int grid;
    const uint32_t* gate; uint32_t gate_run;  // as in SortArgs
};
void launch_leaf_build(const LeafBuildArgs& a, cudaStream_t s);  // two launches (build + fix-up)

// Fragment grouping by hash (group.cu): the same parents and leaf masks as
// the fragment sort + leaf build, for inputs with many fragments per brick.
constexpr double kGroupMinRedundancy = 8.0;  // fragments per distinct brick that make grouping pay
constexpr int kGroupSketchRegs = 4096;
constexpr int kGroupPartLog = 11;                        // fine partitions counted by the sketch pass
constexpr int kGroupMaxParts = 1 << kGroupPartLog;
constexpr int kGroupPartSlotsLog = 12;                   // shared-memory table of one partition
constexpr int kGroupPartSlots = 1 << kGroupPartSlotsLog;
constexpr double kGroupMaxBricksPerPart = 0.45 * kGroupPartSlots;  // most bricks per table (load 0.45)
constexpr float kGroupTargetBricksPerPart = 1536.0f;     // partitions chosen for ~this many (load ~0.3)
constexpr uint64_t kGroupMaxBricks = (uint64_t)kGroupMaxParts * kGroupPartSlots;
constexpr int kGroupMaxChunks = 512;                     // CTAs of the sketch and scatter passes
constexpr uint64_t kGroupScratchBytes = kGroupMaxBricks * 8;  // the brick masks
struct GroupArgs {
    const uint64_t* frags; uint64_t n;
    const uint64_t* seg_offsets; uint32_t seg_count; int seg_shift;  // batched input (as in SortArgs)
    const uint64_t* seg_code;                                         // chunk Morton index per segment
    int validate_bits;
    int mode;                  // 1: choose by the sketch, 2: always group (tests)
    int narrow;                // every key below 2^37 (bricks below 2^31): 32-bit hashes and table keys
    int chunks;                // CTAs of the scatter: chunk c = [c*L, (c+1)*L), L = ceil(n / chunks)
    uint32_t* sketch;          // kGroupSketchRegs words, zero: the probe's distinct-brick sketch
    float probe_max_distinct;  // grouping when the probe's sample shows at most this many distinct bricks
    uint64_t* cursor;          // kGroupMaxParts: partition p's next free position in its slab
    uint32_t* path;            // [0] 1 grouping, 0 sort path; [1] log2 partitions; [2] log2 table slots; [3] slab size
    uint64_t* parts;           // partition slabs (group_shape's slab_total fragment keys)
    uint64_t* overflow; uint64_t overflow_cap;  // fragments past their slab's end, any partition
    uint64_t* overflow_count;  // zero on entry
    uint32_t* part_over;       // kGroupMaxParts flags, zero on entry: the partition spilled
    uint64_t* bricks; uint32_t* idx; uint64_t* masks; uint64_t cap;  // brick list (unsorted), masks[idx]
    uint64_t* d_count;         // bricks found
    const uint64_t* sorted_bricks; const uint32_t* sorted_idx;      // after the brick sort
    uint64_t* parents; uint64_t* leaves;
    uint32_t* err;
};
void group_configure(int sms);
int group_chunks(uint64_t n);                                      // `chunks` for n fragments
// Room for the partition slabs of n fragments, and the probe's limit (host
// side, before the call).
void group_shape(uint64_t n, uint64_t* slab_total, float* probe_max_distinct);
void launch_group_probe(const GroupArgs& a, cudaStream_t s);
void launch_group_plan(const GroupArgs& a, cudaStream_t s);      // picks the path
void launch_group_scatter(const GroupArgs& a, cudaStream_t s);
void launch_group_aggregate(const GroupArgs& a, cudaStream_t s);
void launch_group_gather(const GroupArgs& a, cudaStream_t s);

// Batched form: every chunk's leaves in one persistent launch (chunks.cu).
// A chunk's local bricks (local code >> 6) fall in 2^bin_bits bins of at most
// 2^kChunkDirectBits bricks, direct-mapped in shared memory.
constexpr int kChunkThreads = 512;
constexpr int kChunkTile = 8192;       // fragments per COUNT / SCATTER item
constexpr int kChunkDirectBits = 13;   // bricks of one bin
constexpr int kChunkMaxBinBits = 12;   // bins per chunk (chunk depth <= 10)
constexpr int kChunkGroupBins = 32;    // bins per LEAVES item
struct ChunkArgs {
    const uint64_t* frags;                          // chunk-local codes, chunks back to back
    const uint64_t* seg_offsets; const uint64_t* seg_code;  // k + 1 offsets, k Morton indices (device)
    uint32_t k; int chunk_depth; int seg_shift;     // seg_shift = 3 * chunk_depth
    int bin_bits;                                   // chunk_bin_bits(chunk_depth)
    const uint32_t* tile_off;                       // k + 1: first COUNT/SCATTER tile of each chunk (device)
    uint32_t tiles;                                 // tile_off[k] (host copy, for the grid only)
    uint32_t groups_per_chunk;                      // LEAVES items per chunk
    uint32_t* hist; uint32_t* cursor;               // k << bin_bits each, zero
    uint32_t* done;                                 // 2k: COUNT tiles done, SCATTER tiles done (zero)
    uint32_t* work;                                 // item counter (zero)
    uint64_t* scratch;                              // fragments by bin (n)
    uint64_t* stage_parent; uint64_t* stage_mask;   // n each: each item's bricks at its fragment offset
    uint32_t* group_bricks; uint64_t* group_src; uint32_t* group_dst;  // per LEAVES item
    uint64_t* parents; uint64_t* leaves; uint64_t out_capacity; uint64_t* d_out_n;
    uint32_t* err;
};
void chunk_configure(int sms);
int chunk_bin_bits(int chunk_depth);  // -> bins of at most 2^kChunkDirectBits bricks
void launch_chunk_leaves(const ChunkArgs& a, cudaStream_t s);  // three launches

// Unique over (key, perm) sorted by key: uid = rank of the key among distinct
// keys; map[perm[i]] = uid; for the first of each run, out_keys[uid] = key and
// payloads are gathered from perm. With node payloads (masks/children) the
// run members are compared in full (collision check).
//
// Every kernel that produces a count is given the capacity of its outputs: it
// never writes past it, clamps the count (and ids) it publishes to it and
// flags kErrCapacity, so that later kernels stay inside their buffers even on
// rejected input.
struct UniqueArgs {
    const uint64_t* keys; const uint32_t* perm; const uint64_t* d_n; uint64_t n_bound;
    const uint8_t* masks; const uint32_t* children;  // null for leaves
    uint32_t* map;
    uint64_t* out_keys; uint8_t* out_masks; uint32_t* out_children;
    uint64_t out_capacity;
    uint64_t* d_out_n;
    uint64_t* status; uint32_t* tile_counter; uint32_t* err; int grid;
};
void launch_unique(const UniqueArgs& a, cudaStream_t s);

// ExtractLevel + ComputeHashes: from the sorted unique codes of the child
// level and their child ids, build one parent node per distinct code >> 3.

// Level dedup by hash set + ordering of the distinct keys (dedup.cu): same
// outputs as sort pairs + unique_runs on (key, item) for one level.
constexpr uint32_t kDedupPerBucket = 256;            // expected distinct keys per bucket (node hashes)
constexpr uint32_t kDedupTopBitCap = 1024;           // bucket room (128-256 expected)
constexpr uint32_t kDedupMaxBuckets = 16384;
constexpr uint64_t kDedupMaxItems = 1ull << 24;
constexpr uint64_t kDedupMaxUnique = (uint64_t)kDedupMaxBuckets * kDedupPerBucket;
// Bucket entries for up to uniq_cap distinct keys: the buckets for n items
// (a power of two, n / 256 <= buckets < 2n / 256) hold fewer than 8n entries.
DAGC_HD uint64_t dedup_bucket_area(uint64_t uniq_cap) {
    const uint64_t a = 8 * uniq_cap > kDedupTopBitCap ? 8 * uniq_cap : kDedupTopBitCap;
    const uint64_t most = (uint64_t)kDedupMaxBuckets * kDedupTopBitCap;
    return a < most ? a : most;
}
// Table slots for n items. Leaf masks repeat (about one distinct mask per ten
// bricks): 1.25 n slots, at most 0.8 full even when every mask is distinct,
// small enough to stay largely in the L2. Node hashes are about half distinct
// and each probe step is a dependent round trip: kNodeTableQuarters / 4 * n
// slots keep the load low. At least 1024 slots, a multiple of 32.
constexpr uint64_t kNodeTableQuarters = 8;
DAGC_HD uint64_t table_size_for(uint64_t n, bool leaf_masks) {
    const uint64_t want = leaf_masks ? n + (n >> 2) : n * kNodeTableQuarters / 4;
    return want < 1024 ? 1024 : (want + 31) & ~31ull;
}
struct DedupState {
    unsigned long long u;  // distinct keys found (zero before the level)
    uint32_t nbuckets, pad0;
    uint32_t inserted, pad;  // 1: extract_level already inserted the level's hashes
};
struct DedupArgs {
    const uint64_t* keys; const uint64_t* d_n;       // items: key per item
    const uint8_t* masks; const uint32_t* children;  // item payloads (null for leaves)
    // Leaf masks (far from uniform): winners go to the unique list, which the
    // caller sorts. Node hashes: winners go to the bucket of their top bits.
    bool to_list;
    uint64_t item_cap;
    // Table of table_cap slots, 16 bytes each so that a
    // slot's key and aux share a sector: table_key[2s] = key, 0 = empty (all
    // 0 on entry and exit); table_aux[2s] = representative item | unique id
    // << 32 (table_aux = table_key + 1).
    uint64_t* table_key; uint64_t* table_aux; uint64_t table_cap;
    uint32_t* item_slot;
    uint64_t* uniq_key; uint64_t uniq_cap;  // the unique list (leaf masks)
    uint32_t* bucket_count;                                       // kDedupMaxBuckets
    // Bucket entries, one 16-byte store each: key (two words), slot, representative.
    uint4* bucket; uint64_t bucket_area;
    DedupState* state;
    uint64_t* out_keys; uint8_t* out_masks; uint32_t* out_children; uint64_t out_capacity;
    uint64_t* d_out_n;
    uint32_t* map;  // item -> unique id
    uint32_t* err;
};
void dedup_configure(int sms);
// Node levels: insert (unless extract_level did), bucket sort, map; returns
// the number of launches.
int launch_dedup(const DedupArgs& a, cudaStream_t s);
// Leaf masks: insert into the table and the unique list; after the caller's
// sort of the list (keys only), assign the unique ids; then map.
void launch_dedup_insert(const DedupArgs& a, cudaStream_t s);
void launch_dedup_assign(const DedupArgs& a, const uint64_t* sorted, cudaStream_t s);
void launch_dedup_map(const DedupArgs& a, cudaStream_t s);

constexpr uint64_t kFuseInsertMax = 1ull << 20;
struct ExtractArgs {
    const uint64_t* child_codes; const uint32_t* child_map; const uint64_t* d_n; uint64_t n_bound;
    const uint64_t* child_hashes;  // unique child hashes (or leaf masks), indexed by child id
    uint64_t* node_codes; uint8_t* node_masks; uint32_t* node_children; uint64_t* node_hashes;
    uint64_t out_capacity;
    uint64_t* d_out_n;
    uint64_t* status; uint32_t* tile_counter; uint32_t* err; int grid;
    // Node levels of the hash-set form with at most kFuseInsertMax children:
    // every node's hash goes straight into the dedup table and its top-bit
    // bucket here (table and bucket count sized by the child count, a bound
    // on the node count), and the level's dedup_insert returns at once.
    // Larger levels keep the separate insert, whose probes overlap.
    int fuse_insert;
    DedupArgs dedup;
};
void launch_extract(const ExtractArgs& a, cudaStream_t s);

// Headless tracer (trace.cu): one primary ray per pixel through the final
// word layout of a depth-`depth` DAG (depth >= 3).
struct TraceArgs {
    const uint32_t* words; uint64_t n_words; int depth;
    uint32_t debug_level, width, height;
    double camera[3], ray_min[3], ray_ddx[3], ray_ddy[3];
    uint32_t* colors;  // width * height, row-major
    uint64_t* hits;    // optional: Morton code of the voxel hit, ~0 for a miss
    uint32_t* err;
};
void launch_trace(const TraceArgs& a, cudaStream_t s);

// Triangle voxelizer (voxelize.cu).
constexpr int kVoxGL = 0;   // the reference's GL rule: one voxel per covered pixel of the dominant view
constexpr int kVoxSAT = 1;  // every voxel the triangle touches (separating axis test)
struct VoxArgs {
    const double* vertices; uint64_t n_tri;  // 9 doubles per triangle
    double aabb[6];                          // box mapped onto the grid: min xyz, max xyz
    int depth, mode;
    uint64_t* codes; uint64_t capacity;
    uint64_t* d_total;                       // fragments produced (may exceed capacity)
    uint64_t* status; uint32_t* tile_counter; uint32_t* err;  // status: voxelize_tiles + 1 words, zero
};
void launch_voxelize(const VoxArgs& a, int grid, cudaStream_t s);
uint64_t voxelize_tiles(uint64_t n_tri);

// The top levels in one single-CTA launch: every level l <= first_level has at
// most kTailCap nodes, so extract + hash + sort + unique run in shared memory.
constexpr int kTailThreads = 1024;
constexpr int kTailCap = 4096;
constexpr int kMaxTailLevels = 8;
constexpr int kTailChildCap = 8192;  // most children of the tail's first level
struct TailLevelOut {
    uint64_t* hashes; uint8_t* masks; uint32_t* children; uint64_t capacity;
    uint64_t* d_nodes; uint64_t* d_unique;
};
struct TailArgs {
    int first_level;
    const uint64_t* child_codes; const uint32_t* child_map; const uint64_t* child_hashes;
    const uint64_t* d_child_n;
    TailLevelOut lv[kMaxTailLevels];
    uint32_t* err;
};
void launch_tail(const TailArgs& a, cudaStream_t s);

// Final layout: word position of every node (exclusive scan of popc+1 over all
// levels concatenated), then headers, child pointers and leaves.
// Node levels root first: level l holds nodes [lv_off[l], lv_off[l + 1]) of
// the concatenated numbering, their masks at lv_masks[l] and children (8 per
// node, ids in level l + 1 or leaf ids) at lv_children[l]: slices of one
// DAG's arrays, or a call's separate per-level pools.
constexpr int kFinalMaxLevels = 24;
struct FinalArgs {
    const uint8_t* lv_masks[kFinalMaxLevels];
    const uint32_t* lv_children[kFinalMaxLevels];
    uint64_t lv_off[kFinalMaxLevels + 1];
    int num_levels;
    uint64_t num_nodes;  // lv_off[num_levels]
    const uint64_t* leaves; uint64_t num_leaves;
    uint32_t* word_pos;  // num_nodes + 1
    uint64_t* d_total;   // exact 64-bit sum of node words
    uint32_t* words;
    uint64_t* status; uint32_t* tile_counter; uint32_t* err; int grid_scan, grid_write;
};
void launch_final_positions(const FinalArgs& a, cudaStream_t s);
void launch_final_write(const FinalArgs& a, cudaStream_t s);

// Gathers / copies used by the merge and the compaction of level outputs.
void launch_remap_children(const uint32_t* in, const uint32_t* map, uint32_t* out, uint64_t n_nodes,
                           cudaStream_t s);
void launch_iota_offset(uint32_t* out, uint64_t n, uint32_t offset, cudaStream_t s);

// Several device-to-device copies in one launch (a DAG's levels out of the
// call's scratch): each copy moves 16, 8, 4 or 1 bytes per thread step,
// whichever its addresses and size allow.
struct CopySeg {
    const void* src;
    void* dst;
    uint64_t bytes;
};
constexpr int kMaxCopySegs = 64;
constexpr uint64_t kCopyPiece = 32768;  // bytes per CTA: eight 16-byte units per thread
struct CopyTable {
    CopySeg seg[kMaxCopySegs];
    uint32_t first_cta[kMaxCopySegs + 1];  // filled by launch_copy_segments
    int count;
    uint64_t* lit_dst;  // and up to 24 words given by value (a DAG's level offsets)
    uint64_t lit[24];
    int lit_count;
};
void launch_copy_segments(const CopyTable& t, cudaStream_t s);

void kernels_configure();

// Resident CTAs per SM of the persistent kernels (for grid sizing).
enum KernelId { kKernelLeafBuild = 0, kKernelExtract = 1, kKernelUnique = 2, kKernelFinalScan = 3, kKernelFinalWrite = 4 };
int occupancy_kernel(int which);

}  // namespace dagc
