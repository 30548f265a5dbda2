// Headless DAG tracer for sm_103a: primary rays through the final uint32 DAG
// layout, written to device buffers (a colour per pixel and the Morton code of
// the voxel hit) instead of the reference's OpenGL surface
// (src/DAGTracer.cu:297-427, FDAGTracer::ResolvePaths :429-443). It reads
// exactly the layout CreateFinalDAG writes (src/DAGCompression.cu:1550-1610),
// so it doubles as an end-to-end check of that format.
//
// The traversal is the reference's: a per-ray stack of (node word index, child
// mask, children still to visit), children visited in the order given by the
// ray's direction signs, each child's intersection found with the slab test
// around the node's centre (epsilon 1e-4 near the splitting planes), the last
// two levels read from the 64-bit leaf. Float arithmetic follows the
// reference's operation order; this file is compiled with --fmad=false, so
// every operation is one IEEE rounding and the result is reproducible on the
// CPU.
//
// Reads of the word array are bounds-checked and each ray stops after
// kTraceMaxSteps descents: a malformed array sets kErrBadInput, never a read
// outside it.

#include "dagc_device.cuh"
#include "dagc_kernels.h"

namespace dagc {
namespace {

constexpr uint32_t kTraceMaxSteps = 1u << 22;
constexpr int kTraceMaxDepth = 21;  // the deepest DAG the library builds

__device__ __forceinline__ float max_ref(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float min_ref(float a, float b) { return a < b ? a : b; }

// Children of the node around `path` at `level` that the ray crosses.
__device__ uint32_t crossed_children(bool root, int depth, int level, const uint32_t path[3], float3 org,
                                     float3 dir, float3 inv) {
    const uint32_t shift = (uint32_t)(depth - level);
    const float radius = float(1u << (shift - 1));
    const float3 cr = make_float3(radius + float(path[0] << shift) - org.x, radius + float(path[1] << shift) - org.y,
                                  radius + float(path[2] << shift) - org.z);
    const float3 tmid = make_float3(cr.x * inv.x, cr.y * inv.y, cr.z * inv.z);
    const float3 slab = make_float3(radius * fabsf(inv.x), radius * fabsf(inv.y), radius * fabsf(inv.z));
    const float tmin = max_ref(max_ref(tmid.x - slab.x, max_ref(tmid.y - slab.y, tmid.z - slab.z)), 0.0f);
    const float tmax = min_ref(tmid.x + slab.x, min_ref(tmid.y + slab.y, tmid.z + slab.z));
    if (root && tmin >= tmax) return 0;
    // The child holding the midpoint of the ray's span inside the node...
    const float half = 0.5f * (tmin + tmax);
    uint32_t mask = 1u << ((half * dir.x >= cr.x ? 4 : 0) + (half * dir.y >= cr.y ? 2 : 0) +
                           (half * dir.z >= cr.z ? 1 : 0));
    // ... and, where the ray crosses a splitting plane inside the span, the
    // children on both sides of it (both, near another plane).
    const float eps = 1e-4f;
    if (tmin <= tmid.x && tmid.x <= tmax) {
        const float py = tmid.x * dir.y, pz = tmid.x * dir.z;
        const uint32_t a = (py >= cr.y - eps ? 0xCCu : 0u) | (py <= cr.y + eps ? 0x33u : 0u);
        const uint32_t b = (pz >= cr.z - eps ? 0xAAu : 0u) | (pz <= cr.z + eps ? 0x55u : 0u);
        mask |= a & b;
    }
    if (tmin <= tmid.y && tmid.y <= tmax) {
        const float px = tmid.y * dir.x, pz = tmid.y * dir.z;
        const uint32_t c = (px >= cr.x - eps ? 0xF0u : 0u) | (px <= cr.x + eps ? 0x0Fu : 0u);
        const uint32_t d = (pz >= cr.z - eps ? 0xAAu : 0u) | (pz <= cr.z + eps ? 0x55u : 0u);
        mask |= c & d;
    }
    if (tmin <= tmid.z && tmid.z <= tmax) {
        const float px = tmid.z * dir.x, py = tmid.z * dir.y;
        const uint32_t e = (px >= cr.x - eps ? 0xF0u : 0u) | (px <= cr.x + eps ? 0x0Fu : 0u);
        const uint32_t f = (py >= cr.y - eps ? 0xCCu : 0u) | (py <= cr.y + eps ? 0x33u : 0u);
        mask |= e & f;
    }
    return mask;
}

__device__ __forceinline__ uint32_t murmur32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ uint32_t channel(uint32_t v) {
    const float c = float(v & 0xFFu) / 255.0f;
    return uint32_t(fminf(1.0f, fmaxf(0.0f, c)) * 255.0f);
}

// Stack entry: node word index | child mask << 32 | children to visit << 40.
__device__ __forceinline__ uint64_t pack(uint32_t index, uint32_t cm, uint32_t vm) {
    return (uint64_t)index | (uint64_t)cm << 32 | (uint64_t)vm << 40;
}

__global__ void __launch_bounds__(128) trace_rays(TraceArgs a) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= a.width || py >= a.height) return;
    const int depth = a.depth, leaf_level = depth - 2;
    const uint32_t* w = a.words;
    const uint64_t nw = a.n_words;
    bool ok = true;
    auto word = [&](uint64_t i) -> uint32_t {
        if (i >= nw) { ok = false; return 0; }
        return __ldg(w + i);
    };

    // Ray: direction normalised in double, then float (src/DAGTracer.cu:310-318).
    const double vx = a.ray_min[0] + double(px) * a.ray_ddx[0] + double(py) * a.ray_ddy[0] - a.camera[0];
    const double vy = a.ray_min[1] + double(px) * a.ray_ddx[1] + double(py) * a.ray_ddy[1] - a.camera[1];
    const double vz = a.ray_min[2] + double(px) * a.ray_ddx[2] + double(py) * a.ray_ddy[2] - a.camera[2];
    const double s = 1 / sqrt(vx * vx + vy * vy + vz * vz);
    const float3 org = make_float3(float(a.camera[0]), float(a.camera[1]), float(a.camera[2]));
    const float3 dir = make_float3(float(s * vx), float(s * vy), float(s * vz));
    const float3 inv = make_float3(float(1. / double(dir.x)), float(1. / double(dir.y)), float(1. / double(dir.z)));
    const uint32_t order = (dir.x < 0.f ? 4u : 0u) + (dir.y < 0.f ? 2u : 0u) + (dir.z < 0.f ? 1u : 0u);

    uint64_t stack[kTraceMaxDepth];
    uint32_t path[3] = {0, 0, 0};
    uint32_t debug_index = 0, leaf_lo = 0, leaf_hi = 0;
    int level = 0;
    uint32_t index = 0;
    uint32_t cm = word(0) & 0xFFu;
    uint32_t vm = cm & crossed_children(true, depth, 0, path, org, dir, inv);
    bool hit = false;
    for (uint32_t step = 0;; ++step) {
        if (step >= kTraceMaxSteps) { ok = false; break; }
        // Ascend to the deepest level with a child left.
        int nl = level;
        while (nl > 0 && !vm) {
            --nl;
            const uint64_t e = stack[nl];
            index = (uint32_t)e;
            cm = (uint32_t)(e >> 32) & 0xFFu;
            vm = (uint32_t)(e >> 40) & 0xFFu;
        }
        if (nl == 0 && !vm) {
            path[0] = path[1] = path[2] = 0;
            break;
        }
        path[0] >>= (level - nl);
        path[1] >>= (level - nl);
        path[2] >>= (level - nl);
        level = nl;
        // Next child in the ray's order: the first set bit of vm after
        // relabelling the children by child ^ order.
        uint32_t child = 0;
        for (uint32_t c = 0; c < 8; ++c)
            if (vm & (1u << (c ^ order))) { child = c ^ order; break; }
        vm &= ~(1u << child);
        path[0] = (path[0] << 1) | ((child >> 2) & 1u);
        path[1] = (path[1] << 1) | ((child >> 1) & 1u);
        path[2] = (path[2] << 1) | (child & 1u);
        stack[level] = pack(index, cm, vm);
        ++level;
        if ((uint32_t)(depth - 2 - level) == a.debug_level) debug_index = index;
        if (level == depth) { hit = true; break; }
        if (level <= leaf_level) {
            const uint32_t ptr = word((uint64_t)index + __popc(cm & ((1u << child) - 1u)) + 1);
            if (level < leaf_level) {
                index = ptr;
                cm = word(index) & 0xFFu;
            } else {
                leaf_lo = word(ptr);
                leaf_hi = word((uint64_t)ptr + 1);
                // Sub-block b of the leaf is byte b of the 64-bit mask.
                cm = 0;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    cm |= ((leaf_lo >> (8 * b)) & 0xFFu) ? 1u << b : 0u;
                    cm |= ((leaf_hi >> (8 * b)) & 0xFFu) ? 1u << (4 + b) : 0u;
                }
            }
        } else {
            cm = (((child & 4u) ? leaf_hi : leaf_lo) >> ((child & 3u) * 8)) & 0xFFu;
        }
        vm = cm & crossed_children(false, depth, level, path, org, dir, inv);
        if (!ok) break;
    }
    const uint64_t pix = (uint64_t)py * a.width + px;
    a.colors[pix] = a.debug_level == 0xFFFFFFFFu ? channel(path[0]) | channel(path[1]) << 8 | channel(path[2]) << 16
                                                 : murmur32(debug_index);
    if (a.hits) {
        uint64_t code = ~0ull;
        if (hit) {
            code = 0;
            for (int b = 0; b < depth; ++b)
                code |= (uint64_t)((path[0] >> b) & 1u) << (3 * b + 2) | (uint64_t)((path[1] >> b) & 1u) << (3 * b + 1) |
                        (uint64_t)((path[2] >> b) & 1u) << (3 * b);
        }
        a.hits[pix] = code;
    }
    if (!ok) atomicOr(a.err, kErrBadInput);
}

}  // namespace

void launch_trace(const TraceArgs& a, cudaStream_t s) {
    const dim3 block(8, 16);
    const dim3 grid((a.width + block.x - 1) / block.x, (a.height + block.y - 1) / block.y);
    trace_rays<<<grid, block, 0, s>>>(a);
}

}  // namespace dagc
