// A program written against the reference's DAGCompression.h API, built with
// the drop-in header (include/DAGCompression.h) and libdagc. It follows the
// reference's main() (src/DAG_Compression_Fast.cpp:283-349): CreateDAG per
// subvolume in Morton order, MergeDAGs, CreateFinalDAG, FreeAll.
//
//   dropin_main <codes.u64> <depth> <split_levels> <words.u32>
// Reads uint64 Morton codes of a 2^depth volume, splits them into
// 8^split_levels subvolumes, writes the final uint32 DAG.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "DAGCompression.h"

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: %s codes.u64 depth split_levels words.u32\n", argv[0]);
        return 2;
    }
    const int depth = std::atoi(argv[2]);
    const int split = std::atoi(argv[3]);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    std::vector<uint64> codes;
    uint64 c;
    while (std::fread(&c, 8, 1, f) == 1) codes.push_back(c);
    std::fclose(f);

    const int sub = depth - split;
    const uint64 slots = 1ull << (3 * split);
    std::vector<std::vector<uint64>> chunks(slots);
    for (uint64 code : codes) chunks[code >> (3 * sub)].push_back(code & ((1ull << (3 * sub)) - 1));

    std::vector<FCpuDag> DagsToMerge;
    for (uint64 i = 0; i < slots; ++i) {
        TStaticArray<FMortonCode, EMemoryType::GPU> Fragments("Fragments", chunks[i].size());
        if (chunks[i].size())
            cudaMemcpy(Fragments.GetData(), chunks[i].data(), chunks[i].size() * 8, cudaMemcpyHostToDevice);
        DagsToMerge.push_back(DAGCompression::CreateDAG(Fragments, sub));
        Fragments.Free();
    }
    FCpuDag MergedDag = DagsToMerge.size() == 1 ? DagsToMerge[0] : DAGCompression::MergeDAGs(std::move(DagsToMerge));
    auto Dag = DAGCompression::CreateFinalDAG(std::move(MergedDag));

    std::vector<uint32> words(Dag.Num());
    if (Dag.Num()) cudaMemcpy(words.data(), Dag.GetData(), Dag.Num() * 4, cudaMemcpyDeviceToHost);
    Dag.Free();
    DAGCompression::FreeAll();
    DAGCompression::Test();

    FILE* o = std::fopen(argv[4], "wb");
    if (!o) return 4;
    if (!words.empty()) std::fwrite(words.data(), 4, words.size(), o);
    std::fclose(o);
    std::printf("%zu fragments -> %zu words\n", codes.size(), words.size());
    return 0;
}
