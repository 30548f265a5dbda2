// Serving loop over the dagc C ABI (include/dagc.h): compression requests are
// admitted by their device-memory footprint into a fixed number of worker
// slots and run concurrently, each slot on its own context (scratch arena,
// DAG pool, recorded CUDA graphs) and its own stream, so that requests that
// arrive while others run start as soon as a slot and memory are free and
// their kernels overlap on the GPU. The reference has no counterpart (its
// app compresses its subvolumes one after another,
// src/DAG_Compression_Fast.cpp:283-302).
//
// Requests that name a chunk (its Morton index in a grid of chunks) keep their
// intermediate DAG on the device after finishing, and a merge thread folds
// each finished chunk into a resident union of all chunks so far (the growing
// shared DAG, dagc_union); dagc_server_shared_dag builds the levels above the
// chunks over that union (dagc_dag_lift) instead of merging every chunk again.
//
// Every job records CUDA events around its device work on its slot's stream;
// dagc_server_timeline reports that interval against an event recorded when
// the server was created, so overlap of jobs on the device can be read off.

#include "../../include/dagc.h"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    const uint64_t* h_fragments = nullptr;  // caller-owned until the request is done
    uint64_t n = 0;
    int depth = 0;
    int64_t chunk = -1;      // Morton index of the chunk, or -1
    uint64_t footprint = 0;  // admission estimate, bytes
    Clock::time_point submitted, started, finished;
    int status = DAGC_OK;
    std::string error;
    std::vector<uint32_t> words;
    uint32_t* h_out = nullptr;  // caller's word buffer (dagc_server_submit_into), or null
    uint64_t out_cap = 0;
    uint64_t n_out = 0;          // words written to h_out
    bool into = false;           // the words went to h_out
    bool done = false;
    double gpu_start_ms = -1, gpu_end_ms = -1;  // device interval of its work (see dagc_server_timeline)
};

}  // namespace

struct dagc_server_t {
    int device = 0;
    uint64_t budget = 0, in_use = 0, peak_in_use = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::map<uint64_t, std::shared_ptr<Request>> requests;
    std::vector<std::thread> workers;
    std::vector<dagc_context> contexts;
    std::map<int64_t, dagc_dag> chunk_dags;  // kept on the device, by chunk Morton index
    int chunk_depth = -1;
    dagc_context merge_ctx = nullptr;
    uint64_t next_ticket = 1;
    uint64_t completed = 0, fragments_done = 0, running = 0, max_running = 0;
    bool stop = false;
    // Growing shared DAG (merge thread; guarded by `mu`): the union of the
    // folded chunks, their root hashes by slot, chunks waiting to be folded,
    // DAGs retired while a fold may read them.
    dagc_dag body = nullptr;
    std::map<int64_t, uint64_t> slot_root;
    std::vector<int64_t> fold_queue;
    bool body_stale = false;  // a folded chunk was replaced: rebuild from chunk_dags
    bool folding = false;
    int fold_status = DAGC_OK;
    uint64_t folds = 0;       // unions made so far
    std::vector<dagc_dag> retired;
    std::condition_variable cv_fold, cv_folded;
    std::thread merger;
    // Device timeline: reference event and each job's interval, by ticket.
    cudaEvent_t origin = nullptr;
    std::map<uint64_t, std::pair<double, double>> timeline;
};

namespace {

void worker_loop(dagc_server_t* sv, int slot) {
    cudaSetDevice(sv->device);
    dagc_context ctx = sv->contexts[slot];
    cudaStream_t stream = nullptr;
    cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    // Staging buffer for the fragments, kept across requests: a cudaFree per
    // request would synchronise the whole device and serialise the slots.
    void* stage = nullptr;
    uint64_t stage_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    for (;;) {
        std::shared_ptr<Request> r;
        {
            std::unique_lock<std::mutex> lock(sv->mu);
            // FIFO admission: the head of the queue starts when a slot (this
            // thread) is free and its footprint fits in the budget.
            sv->cv_work.wait(lock, [&] {
                return sv->stop ||
                       (!sv->queue.empty() &&
                        (sv->in_use + sv->queue.front()->footprint <= sv->budget || sv->in_use == 0));
            });
            if (sv->stop && sv->queue.empty()) break;
            r = sv->queue.front();
            sv->queue.pop_front();
            sv->in_use += r->footprint;
            sv->peak_in_use = std::max(sv->peak_in_use, sv->in_use);
            ++sv->running;
            sv->max_running = std::max(sv->max_running, sv->running);
            r->started = Clock::now();
        }
        int st = DAGC_OK;
        std::string err;
        std::vector<uint32_t> words;
        dagc_dag keep = nullptr;
        {
            // Host fragments in, host words out, on this slot's stream.
            if (r->n > stage_cap) {
                if (stage) cudaFree(stage);
                stage = nullptr;
                stage_cap = 0;
                if (cudaMalloc(&stage, r->n * 8) != cudaSuccess) { cudaGetLastError(); st = DAGC_ERR_OUT_OF_MEMORY; }
                else stage_cap = r->n;
            }
            if (!st && r->n && cudaMemcpyAsync(stage, r->h_fragments, r->n * 8, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
                cudaGetLastError();
                st = DAGC_ERR_CUDA;
            }
            if (!st && ev0) cudaEventRecord(ev0, stream);
            uint32_t* d_words = nullptr;
            uint64_t nw = 0;
            if (!st && r->chunk < 0) {
                // No DAG to keep: CreateDAG + CreateFinalDAG in one call.
                st = dagc_compress(ctx, static_cast<const uint64_t*>(stage), r->n, r->depth, stream, &d_words, &nw);
            } else if (!st) {
                dagc_dag dag = nullptr;
                st = dagc_create(ctx, static_cast<const uint64_t*>(stage), r->n, r->depth, stream, &dag);
                // Keep a device copy of the chunk's DAG for the shared DAG
                // (the merge context serialises its own calls).
                if (!st) st = dagc_dag_copy(sv->merge_ctx, dag, stream, &keep);
                if (!st) st = dagc_final(ctx, dag, stream, &d_words, &nw);
                else if (dag) dagc_dag_free(dag);
            }
            if (!st && ev1) cudaEventRecord(ev1, stream);
            if (!st && r->h_out && nw <= r->out_cap) {
                // Straight into the caller's buffer (pinned memory makes this
                // a DMA at link speed).
                cudaError_t e = nw ? cudaMemcpyAsync(r->h_out, d_words, nw * 4, cudaMemcpyDeviceToHost, stream)
                                   : cudaSuccess;
                if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess) { cudaGetLastError(); st = DAGC_ERR_CUDA; }
                dagc_free_words(ctx, d_words, stream);
                r->n_out = nw;
                r->into = true;
            } else if (!st) {
                words.resize(nw);
                st = dagc_words_download(ctx, d_words, nw, words.data());
                dagc_free_words(ctx, d_words, stream);
            }
            if (st) err = dagc_last_error(ctx);
            if (!st && ev0 && ev1 && sv->origin && cudaEventSynchronize(ev1) == cudaSuccess) {
                float a = 0, b = 0;
                if (cudaEventElapsedTime(&a, sv->origin, ev0) == cudaSuccess &&
                    cudaEventElapsedTime(&b, sv->origin, ev1) == cudaSuccess) {
                    r->gpu_start_ms = a;
                    r->gpu_end_ms = b;
                }
                cudaGetLastError();
            }
        }
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            r->status = st;
            r->error = err;
            r->words.swap(words);
            r->finished = Clock::now();
            r->done = true;
            sv->in_use -= r->footprint;
            --sv->running;
            ++sv->completed;
            sv->fragments_done += r->n;
            sv->timeline[r->ticket] = {r->gpu_start_ms, r->gpu_end_ms};
            if (keep) {
                auto it = sv->chunk_dags.find(r->chunk);
                if (it != sv->chunk_dags.end()) {
                    // A fold may be reading the old DAG: the merge thread frees it.
                    sv->retired.push_back(it->second);
                    if (sv->slot_root.count(r->chunk)) sv->body_stale = true;
                }
                sv->chunk_dags[r->chunk] = keep;
                sv->fold_queue.push_back(r->chunk);
                sv->cv_fold.notify_all();
            }
        }
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
    if (stage) cudaFree(stage);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    cudaStreamDestroy(stream);
}

// Folds finished chunks into the resident union, several at a time: one
// dagc_union of the current body and the waiting chunks (or, after a chunk was
// replaced, of every kept chunk).
void merge_loop(dagc_server_t* sv) {
    cudaSetDevice(sv->device);
    cudaStream_t stream = nullptr;
    cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    for (;;) {
        std::vector<int64_t> slots;
        std::vector<dagc_dag> inputs;
        dagc_dag old_body = nullptr;
        bool rebuild = false;
        {
            std::unique_lock<std::mutex> lock(sv->mu);
            sv->cv_fold.wait(lock, [&] { return sv->stop || !sv->fold_queue.empty() || sv->body_stale; });
            if (sv->fold_queue.empty() && !sv->body_stale) break;  // stopping, nothing left
            rebuild = sv->body_stale;
            sv->body_stale = false;
            sv->fold_queue.clear();
            sv->folding = true;
            old_body = sv->body;
            if (rebuild) {
                for (auto& kv : sv->chunk_dags) { slots.push_back(kv.first); inputs.push_back(kv.second); }
            } else {
                if (old_body) inputs.push_back(old_body);
                for (auto& kv : sv->chunk_dags)
                    if (!sv->slot_root.count(kv.first)) { slots.push_back(kv.first); inputs.push_back(kv.second); }
            }
        }
        dagc_dag body = nullptr;
        std::vector<uint64_t> roots(inputs.size(), 0);
        int st = inputs.empty() ? DAGC_OK
                                : dagc_union(sv->merge_ctx, inputs.data(), inputs.size(), stream, &body, roots.data());
        std::vector<dagc_dag> to_free;
        {
            std::lock_guard<std::mutex> lock(sv->mu);
            const size_t first = rebuild || !old_body ? 0 : 1;
            if (!st && body) {
                if (rebuild) sv->slot_root.clear();
                for (size_t i = 0; i < slots.size(); ++i) sv->slot_root[slots[i]] = roots[first + i];
                if (old_body) to_free.push_back(old_body);
                sv->body = body;
                ++sv->folds;
            } else if (st) {
                sv->fold_status = st;
            }
            to_free.insert(to_free.end(), sv->retired.begin(), sv->retired.end());
            sv->retired.clear();
            sv->folding = false;
        }
        for (dagc_dag d : to_free) dagc_dag_free(d);
        sv->cv_folded.notify_all();
    }
    cudaStreamDestroy(stream);
}

}  // namespace

extern "C" {

int dagc_server_create(int device, int slots, uint64_t hbm_budget_bytes, dagc_server* out) {
    if (!out || slots < 1 || slots > 64) return DAGC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::unique_ptr<dagc_server_t> sv(new dagc_server_t);
    sv->device = device;
    sv->budget = hbm_budget_bytes;
    for (int i = 0; i <= slots; ++i) {
        dagc_context c = nullptr;
        const int st = dagc_context_create(device, &c);
        if (st) {
            for (dagc_context x : sv->contexts) dagc_context_destroy(x);
            if (sv->merge_ctx) dagc_context_destroy(sv->merge_ctx);
            return st;
        }
        if (i < slots) sv->contexts.push_back(c);
        else sv->merge_ctx = c;
    }
    cudaSetDevice(device);
    if (cudaEventCreate(&sv->origin) == cudaSuccess) {
        cudaEventRecord(sv->origin, nullptr);
        cudaEventSynchronize(sv->origin);
    } else {
        cudaGetLastError();
        sv->origin = nullptr;
    }
    for (int i = 0; i < slots; ++i) sv->workers.emplace_back(worker_loop, sv.get(), i);
    sv->merger = std::thread(merge_loop, sv.get());
    *out = sv.release();
    return DAGC_OK;
}

int dagc_server_submit(dagc_server sv, const uint64_t* h_fragments, uint64_t n, int depth, int64_t chunk_morton,
                       uint64_t* ticket) {
    return dagc_server_submit_into(sv, h_fragments, n, depth, chunk_morton, nullptr, 0, ticket);
}

int dagc_server_submit_into(dagc_server sv, const uint64_t* h_fragments, uint64_t n, int depth, int64_t chunk_morton,
                            uint32_t* h_words, uint64_t capacity, uint64_t* ticket) {
    if (!sv || !ticket || (n && !h_fragments) || depth < 2 || depth > 21) return DAGC_ERR_INVALID_ARGUMENT;
    auto r = std::make_shared<Request>();
    r->h_out = h_words;
    r->out_cap = h_words ? capacity : 0;
    r->h_fragments = h_fragments;
    r->n = n;
    r->depth = depth;
    r->chunk = chunk_morton;
    // Scratch of the call + staged fragments + the DAG and its words (bounded
    // by 16 bytes per fragment).
    r->footprint = dagc_create_footprint(n, depth) + 8 * n + 16 * n;
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        if (chunk_morton >= 0) {
            if (sv->chunk_depth >= 0 && sv->chunk_depth != depth) return DAGC_ERR_INVALID_ARGUMENT;
            sv->chunk_depth = depth;
        }
        r->ticket = sv->next_ticket++;
        sv->requests[r->ticket] = r;
        sv->queue.push_back(r);
        *ticket = r->ticket;
    }
    sv->cv_work.notify_all();
    return DAGC_OK;
}

int dagc_server_wait(dagc_server sv, uint64_t ticket, uint32_t* h_words, uint64_t capacity, uint64_t* n_words,
                     double* latency_ms) {
    if (!sv || !n_words) return DAGC_ERR_INVALID_ARGUMENT;
    std::shared_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lock(sv->mu);
        auto it = sv->requests.find(ticket);
        if (it == sv->requests.end()) return DAGC_ERR_INVALID_ARGUMENT;
        r = it->second;
        sv->cv_done.wait(lock, [&] { return r->done; });
    }
    *n_words = r->into ? r->n_out : r->words.size();
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(r->finished - r->submitted).count();
    if (r->status) return r->status;
    if (r->into) {  // already in the caller's buffer: collected
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->requests.erase(ticket);
        return DAGC_OK;
    }
    if (h_words) {
        if (capacity < r->words.size()) return DAGC_ERR_INVALID_ARGUMENT;
        if (!r->words.empty()) std::memcpy(h_words, r->words.data(), r->words.size() * 4);
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->requests.erase(ticket);  // the result has been collected
    }
    return DAGC_OK;
}

int dagc_server_stats(dagc_server sv, uint64_t* completed, uint64_t* fragments, uint64_t* max_concurrent,
                      uint64_t* peak_footprint) {
    if (!sv) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(sv->mu);
    if (completed) *completed = sv->completed;
    if (fragments) *fragments = sv->fragments_done;
    if (max_concurrent) *max_concurrent = sv->max_running;
    if (peak_footprint) *peak_footprint = sv->peak_in_use;
    return DAGC_OK;
}

int dagc_server_shared_dag(dagc_server sv, int top_levels, dagc_context* ctx_out, dagc_dag* out) {
    if (!sv || !out || !ctx_out || top_levels < 0 || top_levels > 6) return DAGC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::unique_lock<std::mutex> lock(sv->mu);
    if (sv->chunk_depth < 0 || sv->chunk_depth + top_levels > 21) return DAGC_ERR_INVALID_ARGUMENT;
    const uint64_t slots = 1ull << (3 * top_levels);
    // Every chunk finished so far is folded first.
    sv->cv_folded.wait(lock, [&] { return sv->fold_queue.empty() && !sv->body_stale && !sv->folding; });
    if (sv->fold_status) return sv->fold_status;
    *ctx_out = sv->merge_ctx;
    std::vector<uint64_t> hashes(slots, 0);
    for (auto& kv : sv->slot_root) {
        if (kv.first < 0 || (uint64_t)kv.first >= slots) return DAGC_ERR_INVALID_ARGUMENT;
        hashes[kv.first] = kv.second;
    }
    if (!sv->body) return dagc_create(sv->merge_ctx, nullptr, 0, sv->chunk_depth + top_levels, nullptr, out);
    return dagc_dag_lift(sv->merge_ctx, sv->body, hashes.data(), slots, nullptr, out);
}

int dagc_server_set_option(dagc_server sv, int option, int value) {
    if (!sv) return DAGC_ERR_INVALID_ARGUMENT;
    for (dagc_context c : sv->contexts) {
        const int st = dagc_set_option(c, option, value);
        if (st) return st;
    }
    return DAGC_OK;
}

int dagc_server_folds(dagc_server sv, uint64_t* folds) {
    if (!sv || !folds) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(sv->mu);
    *folds = sv->folds;
    return DAGC_OK;
}

int dagc_server_timeline(dagc_server sv, uint64_t ticket, double* gpu_start_ms, double* gpu_end_ms) {
    if (!sv || !gpu_start_ms || !gpu_end_ms) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(sv->mu);
    auto it = sv->timeline.find(ticket);
    if (it == sv->timeline.end()) return DAGC_ERR_INVALID_ARGUMENT;
    *gpu_start_ms = it->second.first;
    *gpu_end_ms = it->second.second;
    return DAGC_OK;
}

void dagc_server_destroy(dagc_server sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->workers) t.join();
    sv->cv_fold.notify_all();
    if (sv->merger.joinable()) sv->merger.join();
    for (auto& kv : sv->chunk_dags) dagc_dag_free(kv.second);
    for (dagc_dag d : sv->retired) dagc_dag_free(d);
    if (sv->body) dagc_dag_free(sv->body);
    if (sv->origin) cudaEventDestroy(sv->origin);
    for (dagc_context c : sv->contexts) dagc_context_destroy(c);
    if (sv->merge_ctx) dagc_context_destroy(sv->merge_ctx);
    delete sv;
}

}  // extern "C"
