// .dag.bin files: the reference's on-disk final DAG (src/Serializer.h:10-100,
// written/read at src/DAG_Compression_Fast.cpp:361-379): six doubles (AABB
// min x, y, z, max x, y, z), uint32 depth, uint64 word count, the uint32 words;
// all little-endian, no padding.

#include "../../include/dagc.h"

#include <cstdio>
#include <cstring>

extern "C" {

int dagc_file_write(const char* path, const double* aabb6, uint32_t depth, const uint32_t* h_words,
                    uint64_t n_words) {
    if (!path || !aabb6 || (n_words && !h_words)) return DAGC_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return DAGC_ERR_INVALID_ARGUMENT;
    bool ok = std::fwrite(aabb6, sizeof(double), 6, f) == 6 && std::fwrite(&depth, 4, 1, f) == 1 &&
              std::fwrite(&n_words, 8, 1, f) == 1 &&
              (n_words == 0 || std::fwrite(h_words, 4, n_words, f) == n_words);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? DAGC_OK : DAGC_ERR_INVALID_ARGUMENT;
}

int dagc_file_read(const char* path, double* aabb6, uint32_t* depth, uint32_t* h_words, uint64_t capacity,
                   uint64_t* n_words) {
    if (!path || !n_words) return DAGC_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return DAGC_ERR_INVALID_ARGUMENT;
    double box[6];
    uint32_t d = 0;
    uint64_t n = 0;
    bool ok = std::fread(box, sizeof(double), 6, f) == 6 && std::fread(&d, 4, 1, f) == 1 &&
              std::fread(&n, 8, 1, f) == 1;
    if (ok) {
        *n_words = n;
        if (aabb6) std::memcpy(aabb6, box, sizeof(box));
        if (depth) *depth = d;
        if (h_words) {
            if (capacity < n) ok = false;
            else ok = n == 0 || std::fread(h_words, 4, n, f) == n;
        }
    }
    std::fclose(f);
    return ok ? DAGC_OK : DAGC_ERR_BAD_INPUT;
}

}  // extern "C"
