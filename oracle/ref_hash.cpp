// Host build of the reference's own hash and bit helpers (src/Utils.h of
// Phyronnaz/DAG_Compression_Fast), compiled straight from the reference
// sources by oracle/Makefile into oracle/_ref/. TEST INFRASTRUCTURE ONLY: it
// pins the oracle's hash restatement and produces tests/golden/hash_kats.json.
// Only builds where the reference checkout is present.
#include <string>
#include "Utils.h"

extern "C" {

// MurmurHash128xN(ChildrenHashes as 4 x uint128, Size = 4, Seed = 0).Data[0],
// exactly as HashChildrenHashes calls it (src/DAGCompression.cu:758-763), before
// its 0 -> 1 substitution.
unsigned long long ref_murmur128x4_lo(const unsigned long long* h8) {
    uint64 c[8];
    for (int i = 0; i < 8; ++i) c[i] = h8[i];
    return Utils::MurmurHash128xN(reinterpret_cast<const uint128*>(c), 4).Data[0];
}

unsigned long long ref_murmur64(unsigned long long h) { return Utils::MurmurHash64(h); }

unsigned int ref_child_offset(unsigned int mask, unsigned int child) {
    return Utils::ChildOffset(uint8(mask), uint8(child));
}

unsigned int ref_total_size(unsigned int node) { return Utils::TotalSize(node); }

}
