// Drop-in replacement for src/DAGCompression.h of Phyronnaz/DAG_Compression_Fast.
//
// Same namespace, function names, signatures and types as the reference
// (src/DAGCompression.h:6-49), with byte-compatible layouts:
//   FChildrenIndices  = 8 x uint32                      (DAGCompression.h:6-10)
//   TStaticArray<T,M> = { T* ArrayData; uint64 ArraySize } (Array.h:222-224)
//   FCpuLevel / FCpuDag                                  (DAGCompression.h:12-40)
// implemented inline over the dagc C ABI (include/dagc.h), so a program built
// against the reference links against libdagc.so instead.
//
// Semantics follow the reference: CreateDAG borrows device fragments and
// returns a host FCpuDag (levels root first, each ascending by hash);
// MergeDAGs consumes 8^k sub-DAGs in Morton order; CreateFinalDAG consumes the
// DAG and returns the device uint32 word array (Free() releases it); FreeAll
// drops cached device memory. Like the reference (src/Core.h:196-217), any
// failure prints a message and aborts. One process-wide dagc context on the
// current CUDA device plays the part of the reference's global pool.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <vector>

#include "dagc.h"

using int32 = std::int32_t;
using int64 = std::int64_t;
using uint8 = std::uint8_t;
using uint32 = std::uint32_t;
using uint64 = std::uint64_t;
using FMortonCode = uint64;  // src/Core.h:252

enum class EMemoryType { GPU, CPU };  // src/Memory.h:8-12

namespace dagc_dropin {

inline dagc_context& context() {
    static dagc_context ctx = [] {
        int dev = 0;
        cudaGetDevice(&dev);
        dagc_context c = nullptr;
        const int st = dagc_context_create(dev, &c);
        if (st != DAGC_OK) {
            std::fprintf(stderr, "ERROR dagc: context creation failed (%s)\n", dagc_status_string(st));
            std::abort();
        }
        return c;
    }();
    return ctx;
}

inline void check(int status, const char* what) {
    if (status != DAGC_OK) {
        std::fprintf(stderr, "ERROR dagc: %s failed: %s (%s)\n", what, dagc_status_string(status),
                     dagc_last_error(context()));
        std::abort();
    }
}

inline void* alloc(uint64 bytes, EMemoryType type) {
    if (bytes == 0) return nullptr;
    void* p = nullptr;
    if (type == EMemoryType::GPU) {
        if (cudaMalloc(&p, bytes) != cudaSuccess) p = nullptr;
    } else {
        p = std::malloc(bytes);
    }
    if (!p) {
        std::fprintf(stderr, "ERROR dagc: out of %s memory (%llu bytes)\n",
                     type == EMemoryType::GPU ? "GPU" : "CPU", (unsigned long long)bytes);
        std::abort();
    }
    return p;
}

// Final DAG word arrays come from the library's pool; other GPU arrays from
// cudaMalloc. The registry tells Free() which release to call.
inline std::vector<void*>& library_words() {
    static std::vector<void*> v;
    return v;
}

inline void release(void* p, EMemoryType type) {
    if (!p) return;
    if (type == EMemoryType::CPU) { std::free(p); return; }
    auto& lw = library_words();
    for (size_t i = 0; i < lw.size(); ++i) {
        if (lw[i] == p) {
            lw[i] = lw.back();
            lw.pop_back();
            check(dagc_free_words(context(), static_cast<uint32_t*>(p), nullptr), "free");
            return;
        }
    }
    cudaFree(p);
}

}  // namespace dagc_dropin

template <typename TElementType, EMemoryType MemoryType, typename TSize = uint64>
struct TStaticArray {
    TStaticArray() = default;
    TStaticArray(TElementType* Data, TSize Size) : ArrayData(Data), ArraySize(Size) {}
    TStaticArray(const char* /*Name*/, TSize Size)
        : ArrayData(static_cast<TElementType*>(dagc_dropin::alloc(Size * sizeof(TElementType), MemoryType))),
          ArraySize(Size) {}
    TStaticArray(const char* Name, std::initializer_list<TElementType> List) : TStaticArray(Name, List.size()) {
        static_assert(MemoryType == EMemoryType::CPU, "initializer lists build CPU arrays");
        if (List.size()) std::memcpy(ArrayData, List.begin(), List.size() * sizeof(TElementType));
    }

    void Free() {
        dagc_dropin::release(ArrayData, MemoryType);
        ArrayData = nullptr;
        ArraySize = 0;
    }
    void Reset() { ArrayData = nullptr; ArraySize = 0; }
    TSize Num() const { return ArraySize; }
    const TElementType* GetData() const { return ArrayData; }
    TElementType* GetData() { return ArrayData; }
    bool IsValid() const { return ArrayData != nullptr; }
    uint64 SizeInBytes() const { return ArraySize * sizeof(TElementType); }
    TElementType& operator[](TSize i) { return ArrayData[i]; }
    const TElementType& operator[](TSize i) const { return ArrayData[i]; }
    TElementType* begin() { return ArrayData; }
    TElementType* end() { return ArrayData + ArraySize; }
    const TElementType* begin() const { return ArrayData; }
    const TElementType* end() const { return ArrayData + ArraySize; }

    TElementType* ArrayData = nullptr;
    TSize ArraySize = 0;
};

struct FChildrenIndices {
    uint32 Indices[8];
};
static_assert(sizeof(FChildrenIndices) == 8 * sizeof(uint32), "");

struct FCpuLevel {
    TStaticArray<uint8, EMemoryType::CPU> ChildMasks;
    TStaticArray<FChildrenIndices, EMemoryType::CPU> ChildrenIndices;
    TStaticArray<uint64, EMemoryType::CPU> Hashes;

    inline void Free() {
        ChildMasks.Free();
        ChildrenIndices.Free();
        Hashes.Free();
    }
};

struct FCpuDag {
    std::vector<FCpuLevel> Levels;
    TStaticArray<uint64, EMemoryType::CPU> Leaves;

    inline void Free() {
        for (auto& Level : Levels) Level.Free();
        Levels.clear();
        Leaves.Free();
    }
};

namespace dagc_dropin {

inline FCpuDag to_cpu(dagc_dag d) {
    FCpuDag out;
    int nl = 0;
    check(dagc_dag_num_levels(d, &nl), "dag levels");
    out.Levels.resize(nl);
    for (int l = 0; l < nl; ++l) {
        uint64_t n = 0;
        check(dagc_dag_level_size(d, l, &n), "level size");
        FCpuLevel& L = out.Levels[l];
        L.ChildMasks = TStaticArray<uint8, EMemoryType::CPU>("ChildMasks", n);
        L.ChildrenIndices = TStaticArray<FChildrenIndices, EMemoryType::CPU>("ChildrenIndices", n);
        L.Hashes = TStaticArray<uint64, EMemoryType::CPU>("Hashes", n);
        check(dagc_dag_download_level(d, l, L.ChildMasks.GetData(),
                                      reinterpret_cast<uint32_t*>(L.ChildrenIndices.GetData()),
                                      L.Hashes.GetData()),
              "download level");
    }
    uint64_t nleaves = 0;
    check(dagc_dag_num_leaves(d, &nleaves), "leaves");
    out.Leaves = TStaticArray<uint64, EMemoryType::CPU>("Leaves", nleaves);
    check(dagc_dag_download_leaves(d, out.Leaves.GetData()), "download leaves");
    return out;
}

inline dagc_dag to_gpu(const FCpuDag& dag) {
    const int nl = (int)dag.Levels.size();
    std::vector<uint64_t> sizes(nl);
    std::vector<const uint8_t*> masks(nl);
    std::vector<const uint32_t*> children(nl);
    std::vector<const uint64_t*> hashes(nl);
    for (int l = 0; l < nl; ++l) {
        sizes[l] = dag.Levels[l].Hashes.Num();
        masks[l] = dag.Levels[l].ChildMasks.GetData();
        children[l] = reinterpret_cast<const uint32_t*>(dag.Levels[l].ChildrenIndices.GetData());
        hashes[l] = dag.Levels[l].Hashes.GetData();
    }
    dagc_dag out = nullptr;
    check(dagc_dag_upload(context(), nl, sizes.data(), masks.data(), children.data(), hashes.data(),
                          dag.Leaves.GetData(), dag.Leaves.Num(), nullptr, &out),
          "upload");
    return out;
}

}  // namespace dagc_dropin

namespace DAGCompression {

// src/DAGCompression.h:45
inline FCpuDag CreateDAG(const TStaticArray<FMortonCode, EMemoryType::GPU>& Fragments, int32 Depth) {
    dagc_dag d = nullptr;
    dagc_dropin::check(dagc_create(dagc_dropin::context(), Fragments.GetData(), Fragments.Num(), Depth, nullptr, &d),
                       "CreateDAG");
    FCpuDag out = dagc_dropin::to_cpu(d);
    dagc_dag_free(d);
    return out;
}

// src/DAGCompression.h:46
inline FCpuDag MergeDAGs(std::vector<FCpuDag>&& CpuDags) {
    std::vector<dagc_dag> dags;
    dags.reserve(CpuDags.size());
    for (auto& D : CpuDags) {
        dags.push_back(dagc_dropin::to_gpu(D));
        D.Free();
    }
    CpuDags.clear();
    dagc_dag merged = nullptr;
    dagc_dropin::check(dagc_merge(dagc_dropin::context(), dags.data(), dags.size(), nullptr, &merged), "MergeDAGs");
    FCpuDag out = dagc_dropin::to_cpu(merged);
    dagc_dag_free(merged);
    return out;
}

// src/DAGCompression.h:47
inline TStaticArray<uint32, EMemoryType::GPU> CreateFinalDAG(FCpuDag&& CpuDag) {
    dagc_dag d = dagc_dropin::to_gpu(CpuDag);
    CpuDag.Free();
    uint32_t* words = nullptr;
    uint64_t n = 0;
    dagc_dropin::check(dagc_final(dagc_dropin::context(), d, nullptr, &words, &n), "CreateFinalDAG");
    if (words) dagc_dropin::library_words().push_back(words);
    return TStaticArray<uint32, EMemoryType::GPU>(words, n);
}

// src/DAGCompression.h:48
inline void FreeAll() { dagc_dropin::check(dagc_free_all(dagc_dropin::context()), "FreeAll"); }

// src/DAGCompression.h:49 (the reference's unused threading smoke test,
// src/DAGCompression.cu:1617-1647, which ends in an endless loop): here a
// bounded self-check of one tiny compression instead.
inline void Test() {
    uint64 codes[3] = {0, 69, 0};
    FMortonCode* d = nullptr;
    if (cudaMalloc(&d, sizeof(codes)) != cudaSuccess ||
        cudaMemcpy(d, codes, sizeof(codes), cudaMemcpyHostToDevice) != cudaSuccess) {
        std::fprintf(stderr, "ERROR dagc: Test could not stage its input\n");
        std::abort();
    }
    FCpuDag dag = CreateDAG(TStaticArray<FMortonCode, EMemoryType::GPU>(d, 3), 3);
    cudaFree(d);
    if (dag.Levels.size() != 1 || dag.Levels[0].Hashes.Num() != 1 || dag.Leaves.Num() != 2) {
        std::fprintf(stderr, "ERROR dagc: Test produced an unexpected DAG\n");
        std::abort();
    }
    dag.Free();
}

}  // namespace DAGCompression
