/* dagc — GB300-native sparse voxel DAG compression: C ABI.
 *
 * Shuffled uint64 Morton fragment codes go in; a deduplicated sparse voxel DAG
 * comes out, first in the reference's intermediate hash-sorted form (FCpuDag,
 * src/DAGCompression.h:6-40 of Phyronnaz/DAG_Compression_Fast), then in its
 * final uint32 node/leaf word layout (src/DAGCompression.cu:1550-1610).
 *
 * Every entry point takes plain pointers and sizes; device pointers are
 * prefixed d_, host pointers h_. `stream` is a cudaStream_t passed as void*
 * (NULL = the legacy default stream). Every function returns a dagc status
 * code; dagc_last_error() gives the message of the last failure on a context.
 * The library never aborts or traps.
 *
 * Limits: depth in [2, 21] (3 * depth <= 64 code bits), at most 2^31 - 2
 * fragments per call (the reference's int32 counts allow 2^31 - 1), fewer
 * than 2^32 words in a final DAG.
 */
#ifndef DAGC_H
#define DAGC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DAGC_OK 0
#define DAGC_ERR_INVALID_ARGUMENT 1
#define DAGC_ERR_OUT_OF_MEMORY 2
#define DAGC_ERR_BAD_INPUT 3        /* a fragment code >= 2^(3*depth) */
#define DAGC_ERR_HASH_COLLISION 4   /* two different nodes with one 64-bit hash */
#define DAGC_ERR_DEVICE_TIMEOUT 5   /* a bounded device-side wait ran out */
#define DAGC_ERR_CUDA 6
#define DAGC_ERR_TOO_LARGE 7        /* beyond the limits above */

typedef struct dagc_context_t* dagc_context;
typedef struct dagc_dag_t* dagc_dag;

/* ------------------------------------------------------------ context ---- */
/* One context per host thread (or lock around it). It owns the device scratch
 * arena and the stream-ordered pool the DAG arrays come from. */
int dagc_context_create(int device, dagc_context* out);
void dagc_context_destroy(dagc_context ctx);
const char* dagc_last_error(dagc_context ctx);
const char* dagc_status_string(int status);
int dagc_version(void);
/* The node hash: MurmurHash128xN of the 8 child hashes (0 = empty child) as
 * 4 x 128-bit blocks, seed 0, low 64 bits, 0 mapped to 1 (HashChildrenHashes,
 * src/DAGCompression.cu:758-763; src/Utils.h:119-154). Host function. */
uint64_t dagc_hash_children(const uint64_t* h8);

/* ------------------------------------------------------------ CreateDAG ---- */
/* Replaces DAGCompression::CreateDAG (src/DAGCompression.h:45,
 * src/DAGCompression.cu:1003-1107). d_fragments: n device Morton codes, each
 * < 2^(3*depth), duplicates allowed, any order; left unchanged (the reference
 * reuses that buffer as scratch, this library does not). Synchronous on return
 * like the reference. *out receives a device-resident DAG: depth-2 levels,
 * level 0 = root, each level ascending by node hash, plus ascending leaves. */
int dagc_create(dagc_context ctx, const uint64_t* d_fragments, uint64_t n, int depth,
                void* stream, dagc_dag* out);

/* --------------------------------------------------- batched CreateDAG ---- */
/* Many subvolume chunks in one call: the batched form of the reference's
 * per-chunk CreateDAG loop followed by MergeDAGs (src/DAG_Compression_Fast.cpp
 * :283-320). The volume is a grid of 2^top_levels chunks per side, each chunk
 * 2^chunk_depth voxels per side; k of its chunks are given (the others are
 * empty), in ascending Morton order of their chunk coordinates
 * h_chunk_morton[i] < 8^top_levels. d_fragments holds every chunk's
 * chunk-local codes (< 2^(3*chunk_depth)) back to back, chunk i at
 * [h_chunk_offsets[i], h_chunk_offsets[i+1]). The result, a DAG of depth
 * chunk_depth + top_levels, is bit-exact with dagc_merge over 8^top_levels
 * dagc_create results (one per chunk slot, empty slots included). All chunks
 * go through one segmented sort and one level loop; the per-level dedup over
 * all chunks is the merge. Synchronous on return. */
int dagc_create_batched(dagc_context ctx, const uint64_t* d_fragments,
                        const uint64_t* h_chunk_offsets, const uint64_t* h_chunk_morton,
                        uint64_t k, int chunk_depth, int top_levels, void* stream, dagc_dag* out);

/* -------------------------------------------------------- DAG accessors ---- */
int dagc_dag_num_levels(dagc_dag dag, int* num_levels);
int dagc_dag_level_size(dagc_dag dag, int level, uint64_t* num_nodes);
int dagc_dag_num_leaves(dagc_dag dag, uint64_t* num_leaves);
/* Device arrays of one level: masks uint8[n], children uint32[n][8]
 * (0xFFFFFFFF = empty slot; indices into level+1, or into the leaves for the
 * last level), hashes uint64[n]. Valid until the DAG is freed or consumed. */
int dagc_dag_level_device(dagc_dag dag, int level, const uint8_t** d_masks,
                          const uint32_t** d_children, const uint64_t** d_hashes);
int dagc_dag_leaves_device(dagc_dag dag, const uint64_t** d_leaves);
/* Host copies (FCpuLevel::ToCPU, src/DAGCompression.cu:788-803). Any of the
 * output pointers may be NULL. */
int dagc_dag_download_level(dagc_dag dag, int level, uint8_t* h_masks, uint32_t* h_children,
                            uint64_t* h_hashes);
int dagc_dag_download_leaves(dagc_dag dag, uint64_t* h_leaves);
/* Builds a device DAG from host arrays (FGpuLevel::FromCPU,
 * src/DAGCompression.cu:804-816), e.g. an FCpuDag produced elsewhere. */
int dagc_dag_upload(dagc_context ctx, int num_levels, const uint64_t* level_sizes,
                    const uint8_t* const* h_masks, const uint32_t* const* h_children,
                    const uint64_t* const* h_hashes, const uint64_t* h_leaves,
                    uint64_t num_leaves, void* stream, dagc_dag* out);
/* Device copy of a DAG into (possibly another) context on the same device. */
int dagc_dag_copy(dagc_context ctx, dagc_dag src, void* stream, dagc_dag* out);
void dagc_dag_free(dagc_dag dag);
/* Bytes of device scratch one dagc_create call of n fragments at this depth
 * lays out (its arena; the DAG itself comes on top). 0 for n == 0. */
uint64_t dagc_create_footprint(uint64_t n, int depth);

/* ------------------------------------------------------------ MergeDAGs ---- */
/* Replaces DAGCompression::MergeDAGs (src/DAGCompression.h:46,
 * src/DAGCompression.cu:1446-1548). k = 8^m sub-DAGs of equal depth in Morton
 * order of their subvolumes (empty ones allowed); the result has m more
 * levels. Consumes (frees) the inputs, like the reference's rvalue argument.
 * Runs entirely on the device. */
int dagc_merge(dagc_context ctx, dagc_dag* dags, uint64_t k, void* stream, dagc_dag* out);

/* Per-level union of k >= 1 DAGs of equal depth, the reference's pairwise
 * MergeDAGs(FPool&, FCpuDag&&, FCpuDag&&) (src/DAGCompression.cu:1165-1320)
 * for any number of inputs: no level is added, the result's top level holds
 * every input's root. Does not consume the inputs. root_hashes (k entries,
 * may be NULL) receives each input's root hash, 0 for an empty input. */
int dagc_union(dagc_context ctx, dagc_dag* dags, uint64_t k, void* stream, dagc_dag* out,
               uint64_t* root_hashes);
/* The DAG over a grid of `slots` = 8^m chunk slots (Morton order) whose chunk
 * roots are in the top level of `body` (a union of chunk DAGs): slot i holds
 * the chunk with root hash slot_root_hashes[i] (0: empty). The m top levels
 * are built as MergeDAGs builds them (src/DAGCompression.cu:1504-1533); the
 * result equals dagc_merge of the chunk DAGs in their slots when body is their
 * union. */
int dagc_dag_lift(dagc_context ctx, dagc_dag body, const uint64_t* slot_root_hashes, uint64_t slots,
                  void* stream, dagc_dag* out);

/* ------------------------------------------------------- CreateFinalDAG ---- */
/* Replaces DAGCompression::CreateFinalDAG (src/DAGCompression.h:47,
 * src/DAGCompression.cu:1550-1610). Consumes the DAG. *d_words receives a
 * device array of *n_words uint32 (root at word 0), owned by the caller and
 * released with dagc_free_words. An empty DAG gives 0 words and NULL. */
int dagc_final(dagc_context ctx, dagc_dag dag, void* stream, uint32_t** d_words,
               uint64_t* n_words);
/* Returns a word array to the context's pool. Work already queued on `stream`
 * that reads the words (a copy out, a tracer launch) completes before the
 * memory is handed out again: an event recorded on `stream` guards it. Work on
 * other streams must be ordered before this call by the caller. */
int dagc_free_words(dagc_context ctx, uint32_t* d_words, void* stream);
/* Copies n words of a final DAG to host memory (synchronous). */
int dagc_words_download(dagc_context ctx, const uint32_t* d_words, uint64_t n, uint32_t* h_words);

/* -------------------------------------------------------------- FreeAll ---- */
/* Replaces DAGCompression::FreeAll (src/DAGCompression.h:48): releases the
 * cached scratch arena and trims the pool. */
int dagc_free_all(dagc_context ctx);

/* --------------------------------------------------- end-to-end (host) ---- */
/* CreateDAG + CreateFinalDAG from host fragments to host words: copies the
 * fragments in, compresses, copies the words out. If h_words is NULL or
 * capacity is too small only *n_words is set (and DAGC_ERR_INVALID_ARGUMENT is
 * returned when h_words is non-NULL). */
int dagc_compress_host(dagc_context ctx, const uint64_t* h_fragments, uint64_t n, int depth,
                       void* stream, uint32_t* h_words, uint64_t capacity, uint64_t* n_words);

/* Fused device path: CreateDAG + CreateFinalDAG in one call, the words laid
 * out straight from the call's per-level scratch (no intermediate DAG is
 * allocated or copied). Same result as dagc_create followed by dagc_final. */
int dagc_compress(dagc_context ctx, const uint64_t* d_fragments, uint64_t n, int depth,
                  void* stream, uint32_t** d_words, uint64_t* n_words);

/* --------------------------------------------------------- statistics ---- */
/* Counts of the last dagc_create / dagc_compress on this context:
 * out[0] = fragments, out[1] = distinct 4x4x4 bricks (leaf parents),
 * out[2] = unique leaves, out[3 + l] = nodes of level l before dedup for
 * l in [0, depth-2). Returns the number of values written (<= cap). */
int dagc_last_counts(dagc_context ctx, uint64_t* out, int cap);

/* ------------------------------------------------------------ options ---- */
/* Digit-pass plans (the autotuner's knobs). A plan is a kernel shape, as
 * (keys per thread, minimum resident CTAs per SM, equal-digit matching by
 * ballots / match.any / alternating), and the widest digit of the sort.
 * Keys-only shapes (each built for 8- to 11-bit digits): 0 = (16, 3,
 * alternate), 1 = (16, 2, alternate), 2 = (16, 4, alternate), 3 = (12, 4,
 * alternate), 4 = (16, 3, ballot), 5 = (16, 3, match), 6 = (16, 4, or),
 * 7 = (12, 4, or), 8 = (24, 3, or), where "or" finds equal digits by each
 * lane ORing its bit into its digit's word in shared memory. Key/value
 * shapes (8-bit digits):
 * 0 = (16, 2, ballot), 1 = (16, 3, ballot), 2 = (12, 3, ballot), 3 = (8, 4,
 * ballot), 4 = (16, 3, match), 5 = (16, 3, alternate), 6 = (16, 2,
 * alternate), 7 = (12, 3, alternate), 8 = (8, 4, or), 9 = (16, 3, or).
 * Value -1 (default): each
 * sort takes the plan of its class from the context's tuning table (see
 * dagc_tune_sort), else keys (0, 8 bits) and pairs (3, 8 bits). Setting any
 * of these forces it for every sort of its kind. */
#define DAGC_OPT_SORT_SHAPE_KEYS 1   /* keys-only sorts (the fragment sort) */
#define DAGC_OPT_SORT_SHAPE_PAIRS 2  /* key/value sorts (leaf and node hashes) */
#define DAGC_OPT_SORT_RADIX_BITS 8   /* widest digit of keys-only sorts: 8..11, or -1 */
/* 1 (default): launch a CreateDAG kernel sequence directly the first time its
 * input pointer, size and depth are seen, record it as a CUDA graph the second
 * time and replay the graph for later calls with the same shape (recording
 * costs more than one direct launch, so one-off shapes never pay it);
 * 0: launch every kernel directly. Profiling always launches directly. */
#define DAGC_OPT_GRAPHS 3
/* 1 (default): deduplicate the leaves and each level with a hash set and sort
 * only the distinct hashes (bucket sort); 0: sort every (hash, index) pair with
 * the radix sort, as the reference's SortLevel does. Results are identical.
 * An input the hash-set form cannot hold is rerun in the radix form. */
#define DAGC_OPT_DEDUP 4
/* Testing: caps the hash-set form's unique list at `value` keys per level, so
 * that larger levels take the rerun. */
#define DAGC_OPT_DEDUP_UNIQUE_LIMIT 5
/* How fragments are grouped into bricks (SortKeys + SelectUnique +
 * ReduceByKey): 1 (default) choose on the device per call, from a sketch of
 * the distinct bricks in a sample of the fragments: hash partitions and
 * per-partition tables when the fragments hold >= 8 per brick (and the
 * tables can hold the bricks), else the radix sort; 0 always the radix sort;
 * 2 always the hash partitions (an input they cannot hold reruns on the radix
 * sort). Results are identical. */
#define DAGC_OPT_GROUP 6
/* 1: launch every kernel of a call with programmatic dependent launch (the
 * next kernel is scheduled while the previous one runs and waits for it on the
 * device); 0 (default): plain stream order, which measured faster on GB300 for
 * every workload here (config 3: 7.1 ms against 8.3 ms). Results are
 * identical. */
#define DAGC_OPT_PDL 7
/* Batched calls (dagc_create_batched): 1 (default) every chunk's leaves in
 * one persistent launch that takes per-chunk work items from a device queue
 * (bins of each chunk's bricks counted, scattered and turned into leaves in
 * shared memory); 0 the composite-key path (chunk rank above the local code,
 * one sort or grouping over all chunks). Results are identical. */
#define DAGC_OPT_BATCH_PATH 12
/* Failure-path test hooks (off by default; no counterpart in the reference).
 * TEST_SPIN_LIMIT: polls before a bounded device wait of the sorts gives up
 * (0: the production limit, about a second). TEST_STALL_LOOKBACK: 1 makes the
 * first digit pass of every sort leave its tile 0 unpublished, so the waits of
 * the tiles after it run out and the call returns DAGC_ERR_DEVICE_TIMEOUT (the
 * context stays usable). TEST_FAIL_ALLOCS: the context's next `value` device
 * allocations fail as on a full device (dagc_memory_events counts them). */
#define DAGC_OPT_TEST_SPIN_LIMIT 9
#define DAGC_OPT_TEST_STALL_LOOKBACK 10
#define DAGC_OPT_TEST_FAIL_ALLOCS 11
int dagc_set_option(dagc_context ctx, int option, int value);
/* Calls of this context rerun in the radix form so far. */
int dagc_dedup_fallbacks(dagc_context ctx, uint64_t* count);

/* ---------------------------------------------------- instrumentation ---- */
/* Off by default. When enabled, each stage of a call is bracketed by CUDA
 * events recorded on the call's own stream; device time, kernel launches and
 * algorithmic bytes (the bytes each stage must read and write at minimum)
 * accumulate per stage until dagc_profile_reset. The fragment-sort digit passes
 * are bracketed one launch at a time. */
#define DAGC_STAGE_FRAGMENT_HIST 0  /* histogram + key-range check of the fragment sort */
#define DAGC_STAGE_FRAGMENT_PASS 1  /* one 8-bit digit pass of the fragment sort */
#define DAGC_STAGE_LEAF_BUILD 2     /* fused unique + 4x4x4 leaf build */
#define DAGC_STAGE_LEAF_DEDUP 3     /* leaf sort + unique */
#define DAGC_STAGE_LEVELS 4         /* every inner level: extract, hash, sort, unique */
#define DAGC_STAGE_MATERIALISE 5    /* copy of the level outputs into the DAG */
#define DAGC_STAGE_FINAL 6          /* final word layout */
#define DAGC_STAGE_MERGE 7          /* MergeDAGs */
#define DAGC_STAGE_GROUP 8             /* fragment grouping by hash: brick sort, gather */
#define DAGC_STAGE_GROUP_SKETCH 9      /* its probe (a sampled sketch of the distinct bricks) and the path choice */
#define DAGC_STAGE_GROUP_AGGREGATE 10  /* its per-partition tables (one read of the partitioned fragments) */
#define DAGC_STAGE_GROUP_SCATTER 11    /* its partitioning (one read and one write of the fragments) */
#define DAGC_STAGE_CHUNK_LEAVES 12     /* batched form: the persistent per-chunk leaf build, scan and pack */
#define DAGC_NUM_STAGES 13
int dagc_profile_enable(dagc_context ctx, int enable);
int dagc_profile_reset(dagc_context ctx);
int dagc_profile_read(dagc_context ctx, int stage, double* device_ms, uint64_t* launches,
                      uint64_t* bytes);
/* Total kernels this context has launched since it was created. */
int dagc_kernel_launches(dagc_context ctx, uint64_t* launches);

/* ------------------------------------------------------------- sorting ---- */
/* The fragment sort as a standalone primitive: stable LSD radix sort of n
 * uint64 keys on bits [lo_bit, hi_bit), d_in -> d_out (may not alias). The
 * reference wraps cub::DeviceRadixSort::SortKeys (src/DAGCompression.cu:336-357). */
int dagc_sort_keys(dagc_context ctx, const uint64_t* d_in, uint64_t* d_out, uint64_t n,
                   int lo_bit, int hi_bit, void* stream);
/* Pairs variant with uint32 values (src/DAGCompression.cu:359-394). d_vals_in
 * may be NULL: the values are then the input positions 0..n-1 (MakeSequence,
 * src/DAGCompression.cu:743-750). */
int dagc_sort_pairs(dagc_context ctx, const uint64_t* d_keys_in, uint64_t* d_keys_out,
                    const uint32_t* d_vals_in, uint32_t* d_vals_out, uint64_t n, int lo_bit,
                    int hi_bit, void* stream);

/* ----------------------------------------------------------- autotuner ---- */
/* No counterpart in the reference, whose sort takes CUB's static per-arch
 * policy (src/cub/device/dispatch/dispatch_radix_sort.cuh:700-724). Sorts are
 * grouped in classes: keys-only or key/value, number of sorted bits, and the
 * key count's power of two. dagc_tune_sort times every valid plan (shape x
 * digit width, wider digits only where they save a pass) of one class on
 * n pseudo-random keys on this context's device, `reps` sorts each after one
 * untimed sort, and stores the fastest in the context's tuning table (later
 * sorts of the class use it); it reports that plan, its time per sort and
 * the default plan's. dagc_tune_save / dagc_tune_load write / read the table
 * as JSON. At creation a context loads the file named by the environment
 * variable DAGC_TUNE_FILE (empty: none), else sort_plans.json one directory
 * above the library, if it exists. dagc_sort_plan reports the plan a sort of
 * the given class would take. */
int dagc_tune_sort(dagc_context ctx, uint64_t n, int lo_bit, int hi_bit, int with_values, int reps,
                   int* best_shape, int* best_radix_bits, double* best_ms, double* default_ms);
int dagc_tune_save(dagc_context ctx, const char* path);
int dagc_tune_load(dagc_context ctx, const char* path);
int dagc_tune_clear(dagc_context ctx);
int dagc_sort_plan(dagc_context ctx, uint64_t n, int lo_bit, int hi_bit, int with_values, int* shape,
                   int* radix_bits);

/* ------------------------------------------------------------ .dag.bin ---- */
/* The reference's final-DAG file (src/Serializer.h:10-100, used at
 * src/DAG_Compression_Fast.cpp:361-379): six doubles (AABB min x,y,z, max
 * x,y,z), uint32 depth, uint64 word count, then the uint32 words. Host only. */
int dagc_file_write(const char* path, const double* aabb6, uint32_t depth, const uint32_t* h_words,
                    uint64_t n_words);
/* Reads the header (aabb6, depth may be NULL) and, when h_words is not NULL
 * and capacity >= *n_words, the words. */
int dagc_file_read(const char* path, double* aabb6, uint32_t* depth, uint32_t* h_words,
                   uint64_t capacity, uint64_t* n_words);

/* --------------------------------------------------------- memory stats ---- */
/* Device memory of a context (the reference's FMemory statistics,
 * src/Memory.cpp:222-262): bytes held by live DAGs and word arrays, their
 * peak, bytes cached for reuse, and the scratch arena's size. */
int dagc_memory_stats(dagc_context ctx, uint64_t* in_use, uint64_t* peak, uint64_t* cached,
                      uint64_t* arena);
/* Text report of a context's device memory, after the reference's
 * FMemory::GetStatsString (src/Memory.cpp:222-262): total, the peak of DAG
 * and word blocks, and an overview by allocation name (bytes, count), largest
 * first. Writes at most `capacity` bytes (NUL-terminated) to buf (may be
 * NULL); *needed receives the full size including the NUL. */
int dagc_memory_report(dagc_context ctx, char* buf, uint64_t capacity, uint64_t* needed);
/* Allocation events of a context: failed device allocations (injected or
 * real) and allocations that succeeded on their retry after the cache was
 * released (src/Memory.cpp:56-70 retries once after freeing its pool). */
int dagc_memory_events(dagc_context ctx, uint64_t* alloc_failures, uint64_t* retries_ok);

/* ------------------------------------------------------------- tracer ---- */
/* Headless counterpart of the reference's FDAGTracer (src/DAGTracer.h:8-93,
 * src/DAGTracer.cu:297-443): one primary ray per pixel through a final DAG
 * (the words dagc_final returns), written to device buffers instead of an
 * OpenGL surface. Ray parameters are in voxel units of the 2^depth grid, as in
 * the reference's TracePathsParams. */
typedef struct dagc_trace_params {
    uint32_t debug_level; /* 0xFFFFFFFF: colour = hit position (low 8 bits per axis);
                             else colour = MurmurHash32 of the node word index at
                             level depth - 2 - debug_level on the ray's path */
    uint32_t width, height, pad;
    double camera[3];  /* ray origin */
    double ray_min[3]; /* point seen by pixel (0, 0) */
    double ray_ddx[3]; /* step per pixel in x */
    double ray_ddy[3]; /* step per pixel in y */
} dagc_trace_params;
/* The reference's FDAGTracer::GetTraceParams (src/DAGTracer.h:26-79): camera
 * position and basis (right, up, forward), vertical field of view in degrees,
 * scene box; maps the box onto the 2^depth grid. */
int dagc_trace_camera(const double position[3], const double right[3], const double up[3], const double forward[3],
                      double fov_degrees, uint32_t width, uint32_t height, const double aabb_min[3],
                      const double aabb_max[3], int depth, uint32_t debug_level, dagc_trace_params* out);
/* Traces width x height rays (pixel (x, y) at y * width + x). d_colors:
 * RGBA8 words; d_hits (may be NULL): Morton code of the voxel hit, ~0 for a
 * miss. Needs depth in [3, 21]. A word array that is not a valid final DAG
 * gives DAGC_ERR_BAD_INPUT (reads stay inside n_words). Synchronous. */
int dagc_trace(dagc_context ctx, const uint32_t* d_words, uint64_t n_words, int depth,
               const dagc_trace_params* params, uint32_t* d_colors, uint64_t* d_hits, void* stream);

/* ---------------------------------------------------------- voxelizer ---- */
/* The fragment producer: CUDA counterpart of the reference's OpenGL
 * voxelization pass (FVoxelizer::GenerateFragments, src/Voxelizer.cpp:254-369,
 * with its shaders). Triangles: 9 doubles each (v0, v1, v2) in DEVICE memory,
 * in scene units; aabb (host): min xyz, max xyz, mapped onto the 2^depth grid.
 * Writes up to `capacity` Morton codes to d_codes (triangles in input order,
 * each triangle's fragments in a fixed order) and the total produced to
 * *n_codes; a total above capacity gives DAGC_ERR_TOO_LARGE (the buffer then
 * holds the first `capacity` codes), as the reference's fragment buffer check
 * (src/Voxelizer.cpp:312). Synchronous. */
#define DAGC_VOXELIZE_GL 0  /* the reference's rule: each triangle projected on
                               its dominant axis, one voxel per covered pixel at
                               the smallest depth over the pixel (float32) */
#define DAGC_VOXELIZE_SAT 1 /* every voxel the triangle touches (separating
                               axis test, float64) */
int dagc_voxelize(dagc_context ctx, const double* d_vertices, uint64_t n_triangles, const double aabb[6], int depth,
                  int mode, uint64_t* d_codes, uint64_t capacity, uint64_t* n_codes, void* stream);

/* -------------------------------------------------------------- serving ---- */
/* A request loop: compression jobs are admitted in arrival order as soon as
 * one of `slots` worker slots is free and their device-memory footprint fits
 * in hbm_budget_bytes (a job larger than the budget runs alone); admitted jobs
 * run concurrently, each slot with its own context and stream, so their work
 * overlaps on the GPU. Each job: host fragments in, final words out. The
 * reference has no counterpart (it compresses one subvolume after another). */
typedef struct dagc_server_t* dagc_server;
int dagc_server_create(int device, int slots, uint64_t hbm_budget_bytes, dagc_server* out);
/* Queues a job; h_fragments must stay valid until dagc_server_wait returns for
 * it. chunk_morton >= 0 marks the job as a chunk of a larger volume (all
 * chunks of a server share one depth): its DAG is kept on the device for
 * dagc_server_shared_dag. */
int dagc_server_submit(dagc_server server, const uint64_t* h_fragments, uint64_t n, int depth,
                       int64_t chunk_morton, uint64_t* ticket);
/* The same, with the job's words copied straight into h_words (capacity
 * words; page-locked memory makes the copy a DMA) when they fit: the job is
 * then collected by its first dagc_server_wait, which only reports *n_words.
 * Words that do not fit are kept as for dagc_server_submit. */
int dagc_server_submit_into(dagc_server server, const uint64_t* h_fragments, uint64_t n, int depth,
                            int64_t chunk_morton, uint32_t* h_words, uint64_t capacity, uint64_t* ticket);
/* Blocks until the job is done. With h_words == NULL only *n_words (and the
 * latency from submission to completion) is returned; otherwise the words are
 * copied out (capacity >= *n_words) and the job is forgotten. */
int dagc_server_wait(dagc_server server, uint64_t ticket, uint32_t* h_words, uint64_t capacity,
                     uint64_t* n_words, double* latency_ms);
int dagc_server_stats(dagc_server server, uint64_t* completed, uint64_t* fragments,
                      uint64_t* max_concurrent, uint64_t* peak_footprint);
/* The shared DAG of every chunk job finished so far, over a grid of
 * 2^top_levels chunks per side (missing chunks empty); equal to dagc_merge of
 * the chunk DAGs in their slots. A merge thread folds each finished chunk into
 * a resident union (dagc_union) as it completes; this call waits for the
 * folds in progress and builds the top levels over the union (dagc_dag_lift).
 * The DAG belongs to *ctx_out (the server's merge context). */
int dagc_server_shared_dag(dagc_server server, int top_levels, dagc_context* ctx_out, dagc_dag* out);
/* dagc_set_option on every worker slot's context. */
int dagc_server_set_option(dagc_server server, int option, int value);
/* Unions the merge thread has made so far. */
int dagc_server_folds(dagc_server server, uint64_t* folds);
/* Device interval of a finished job's work (CreateDAG to CreateFinalDAG on its
 * slot's stream), in ms after an event recorded when the server was created;
 * jobs whose intervals intersect had work in flight on the GPU at the same time. */
int dagc_server_timeline(dagc_server server, uint64_t ticket, double* gpu_start_ms, double* gpu_end_ms);
void dagc_server_destroy(dagc_server server);

/* No counterpart in the reference. The key sort of dagc_sort_keys without any
 * allocation, for callers that must not allocate device memory once running:
 * engines and servers that reserve the device through their own allocator
 * (an ad-hoc cudaMalloc would fail or fragment that reservation) and callers
 * that cannot take cudaMalloc's implicit device synchronisation. Scratch is a
 * fixed ~9.1 MB device array inside the library, present on every GPU that
 * loads it until the process exits. n <= 1048576 keys (else
 * DAGC_ERR_TOO_LARGE, nothing touched); d_in is left intact; no context. The
 * first call on a device sets the array up: make that first call before any
 * stream capture. Calls share the array, so calls whose GPU work overlaps
 * race. Every call reads its error word back from the device and
 * synchronises `stream` before it returns; returns a dagc status. */
int dagc_sort_keys_noalloc(const uint64_t* d_in, uint64_t* d_out, uint64_t n, int lo_bit,
                           int hi_bit, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DAGC_H */
