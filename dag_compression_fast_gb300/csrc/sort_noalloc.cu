// Key sort that allocates nothing: the same histogram + digit-pass kernels as
// dagc_sort_keys, with every scratch buffer (ping-pong keys, histograms,
// look-back status, tile counters, error word) in one file-scope device array
// of fixed size instead of a context's arena.
//
// It exists for callers that must not allocate device memory after start-up:
// engines and servers that hand the whole device to their own allocator (a
// cudaMalloc from a library would then fail or fragment their reservation),
// and callers that cannot afford cudaMalloc's implicit device-wide
// synchronisation on their critical path.
//
// Properties a caller has to know:
//   * at most kNoAllocMaxKeys keys per call; larger n returns
//     DAGC_ERR_TOO_LARGE before touching any memory;
//   * the scratch array (about 9.1 MB) exists on every GPU that loads the
//     library, for the lifetime of the process;
//   * the first call on a device resolves the array's device address
//     (cudaGetSymbolAddress) and configures the kernels; make that first call
//     before any stream capture;
//   * every call reads its error word back and synchronises its stream
//     before it returns;
//   * all calls share the one array: calls whose work overlaps on the GPU
//     (different streams, or host threads without ordering) race and give
//     wrong results. Each call clears the parts that must start at zero.

#include "../../include/dagc.h"
#include "dagc_device.cuh"
#include "dagc_kernels.h"
#include "dagc_launch.h"

#include <cstddef>
#include <mutex>

namespace dagc {
namespace {

constexpr uint64_t kNoAllocMaxKeys = 1ull << 20;  // 1,048,576 uint64 keys per call
constexpr uint64_t kNoAllocTiles = (kNoAllocMaxKeys + kSortTile - 1) / kSortTile;
constexpr int kNoAllocShape = 0;  // keys-only digit-pass shape used for these sorts (8-bit digits)
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    // Cleared by every call (one memset of everything before `status`).
    uint32_t err;
    uint32_t pad[63];
    uint32_t tile_counters[kMaxPasses];
    uint32_t hist[kMaxPasses * 256];
    // Look-back status of the digit passes: status[0] is cleared by the
    // histogram kernel, the other region by the pass before its use.
    uint32_t status[2][kNoAllocTiles * 256];
    // Ping-pong key buffer.
    uint64_t keys_alt[kNoAllocMaxKeys];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

struct DeviceSetup {
    void* scratch = nullptr;  // device address of g_noalloc_scratch on this device
    int sms = 0;
    int occ_pass = 0;
    int hist_per_sm = 0;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

// Once per device, with that device current: resolve the array's address and
// configure the kernels. Returns a dagc status.
int setup_current_device(DeviceSetup* out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return DAGC_ERR_CUDA; }
    if (dev < 0 || dev >= kMaxDevices) return DAGC_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup& d = g_setup[dev];
    if (!d.scratch) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) { cudaGetLastError(); return DAGC_ERR_CUDA; }
        sort_configure();
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            return DAGC_ERR_CUDA;
        }
        d.sms = sms;
        d.occ_pass = occupancy_sort_shape(kNoAllocShape, false, kRadixBits);
        if (d.occ_pass < 1) d.occ_pass = 1;
        d.hist_per_sm = occupancy_sort_histogram();
        if (d.hist_per_sm < 1) d.hist_per_sm = 1;
        d.scratch = p;
    }
    *out = d;
    return DAGC_OK;
}

}  // namespace
}  // namespace dagc

using namespace dagc;

extern "C" int dagc_sort_keys_noalloc(const uint64_t* d_in, uint64_t* d_out, uint64_t n, int lo_bit, int hi_bit,
                                      void* stream) {
    if (lo_bit < 0 || hi_bit > 64 || lo_bit > hi_bit) return DAGC_ERR_INVALID_ARGUMENT;
    if (n > kNoAllocMaxKeys) return DAGC_ERR_TOO_LARGE;
    if (n == 0) return DAGC_OK;
    if (!d_in || !d_out || d_in == d_out) return DAGC_ERR_INVALID_ARGUMENT;
    DeviceSetup dev;
    int st = setup_current_device(&dev);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Plain stream order for these launches, whatever a context call made
    // earlier on this thread asked for.
    t_pdl = false;
    char* base = static_cast<char*>(dev.scratch);
    NoAllocScratch* S = reinterpret_cast<NoAllocScratch*>(base);  // device address: offsets only on the host
    if (cudaMemsetAsync(base, 0, offsetof(NoAllocScratch, status), s) != cudaSuccess) {
        cudaGetLastError();
        return DAGC_ERR_CUDA;
    }
    SortArgs a{};
    a.keys_in = d_in;
    a.keys_out = d_out;
    a.keys_alt = S->keys_alt;
    a.with_values = false;
    a.n = n;
    a.d_n = nullptr;
    a.lo_bit = lo_bit;
    a.hi_bit = hi_bit;
    a.validate_bits = 0;
    a.hist = S->hist;
    a.status[0] = S->status[0];
    a.status[1] = S->status[1];
    a.tile_counters = S->tile_counters;
    a.err = &S->err;
    const uint64_t tile = 256ull * sort_shape_items(kNoAllocShape, false);
    const uint64_t tiles = (n + tile - 1) / tile;
    const uint64_t resident = (uint64_t)dev.occ_pass * (uint64_t)dev.sms;
    a.grid_pass = (int)(tiles < resident ? tiles : resident);
    const uint64_t hist_blocks = (n + 4095) / 4096, hist_cap = (uint64_t)dev.hist_per_sm * (uint64_t)dev.sms;
    a.grid_hist = (int)(hist_blocks < hist_cap ? hist_blocks : hist_cap);
    a.shape = kNoAllocShape;
    a.radix_bits = kRadixBits;
    launch_sort(a, s);
    if (cudaGetLastError() != cudaSuccess) return DAGC_ERR_CUDA;
    uint32_t err = 0;
    if (cudaMemcpyAsync(&err, &S->err, sizeof(err), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return DAGC_ERR_CUDA;
    }
    if (err & kErrTimeout) return DAGC_ERR_DEVICE_TIMEOUT;
    if (err) return DAGC_ERR_CUDA;
    return DAGC_OK;
}
