// TEST INFRASTRUCTURE ONLY: CPU restatement of the reference's DAG tracer,
// used as the checker of dagc_trace. Parity of this restatement is UNPINNED:
// the reference's tracer writes to an OpenGL surface and cannot run here, and
// its float arithmetic depends on that build's FMA contraction. This file and
// the CUDA tracer both use plain IEEE operations (no contraction: this file is
// built with -ffp-contract=off, the CUDA file with --fmad=false), so the two
// agree bit for bit.
//
// Follows src/DAGTracer.cu:
//   float3_to_rgb888         :23-31
//   next_child               :33-44
//   FPath ascend/descend     :59-74 (x = bit 2, y = bit 1, z = bit 0)
//   Leaf child masks         :99-137 (byte i of the 64-bit leaf = sub-block i)
//   compute_intersection_mask:177-288
//   trace_paths traversal    :297-414, colours :416-426
// and src/Utils.h:64-85 (ChildMask, ChildOffset, MurmurHash32), the ray set-up
// math of src/CudaMath.h:45 (normalize = (1 / length(a)) * a).

#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

struct F3 { float x, y, z; };
struct D3 { double x, y, z; };

float fmax_ref(float a, float b) { return a > b ? a : b; }  // constexpr_max
float fmin_ref(float a, float b) { return a < b ? a : b; }  // constexpr_min

uint32_t murmur32(uint32_t h) {  // Utils.h:77-85
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

uint32_t rgb888(float r, float g, float b) {  // DAGTracer.cu:23-31
    const float R = std::fmin(1.0f, std::fmax(0.0f, r));
    const float G = std::fmin(1.0f, std::fmax(0.0f, g));
    const float B = std::fmin(1.0f, std::fmax(0.0f, b));
    return (uint32_t(R * 255.0f) << 0) | (uint32_t(G * 255.0f) << 8) | (uint32_t(B * 255.0f) << 16);
}

int next_child(int order, int mask) {  // DAGTracer.cu:33-44
    for (int c = 0; c < 8; ++c) {
        const int in_order = c ^ order;
        if (mask & (1 << in_order)) return in_order;
    }
    return 0;
}

struct Params {
    uint32_t debug_level, width, height, pad;
    double camera[3], ray_min[3], ray_ddx[3], ray_ddy[3];
};

// DAGTracer.cu:177-288, with the node's level bounds taken from `depth`.
int intersection_mask(bool root, int depth, int level, const uint32_t path[3], const F3& org, const F3& dir,
                      const F3& inv) {
    const uint32_t shift = (uint32_t)(depth - level);
    const float radius = float(1u << (shift - 1));
    const F3 center = {radius + float(path[0] << shift), radius + float(path[1] << shift),
                       radius + float(path[2] << shift)};
    const F3 cr = {center.x - org.x, center.y - org.y, center.z - org.z};
    const F3 tmid = {cr.x * inv.x, cr.y * inv.y, cr.z * inv.z};
    const F3 slab = {radius * std::fabs(inv.x), radius * std::fabs(inv.y), radius * std::fabs(inv.z)};
    const F3 pmin = {tmid.x - slab.x, tmid.y - slab.y, tmid.z - slab.z};
    const float tmin = fmax_ref(fmax_ref(pmin.x, fmax_ref(pmin.y, pmin.z)), 0.0f);
    const F3 pmax = {tmid.x + slab.x, tmid.y + slab.y, tmid.z + slab.z};
    const float tmax = fmin_ref(pmax.x, fmin_ref(pmax.y, pmax.z));
    if (root && tmin >= tmax) return 0;
    int mask = 0;
    {
        const float half = 0.5f * (tmin + tmax);
        const F3 p = {half * dir.x, half * dir.y, half * dir.z};
        mask |= 1 << ((p.x >= cr.x ? 4 : 0) + (p.y >= cr.y ? 2 : 0) + (p.z >= cr.z ? 1 : 0));
    }
    const float eps = 1e-4f;
    if (tmin <= tmid.x && tmid.x <= tmax) {
        const F3 p = {tmid.x * dir.x, tmid.x * dir.y, tmid.x * dir.z};
        int a = 0, b = 0;
        if (p.y >= cr.y - eps) a |= 0xCC;
        if (p.y <= cr.y + eps) a |= 0x33;
        if (p.z >= cr.z - eps) b |= 0xAA;
        if (p.z <= cr.z + eps) b |= 0x55;
        mask |= a & b;
    }
    if (tmin <= tmid.y && tmid.y <= tmax) {
        const F3 p = {tmid.y * dir.x, tmid.y * dir.y, tmid.y * dir.z};
        int c = 0, d = 0;
        if (p.x >= cr.x - eps) c |= 0xF0;
        if (p.x <= cr.x + eps) c |= 0x0F;
        if (p.z >= cr.z - eps) d |= 0xAA;
        if (p.z <= cr.z + eps) d |= 0x55;
        mask |= c & d;
    }
    if (tmin <= tmid.z && tmid.z <= tmax) {
        const F3 p = {tmid.z * dir.x, tmid.z * dir.y, tmid.z * dir.z};
        int e = 0, f = 0;
        if (p.x >= cr.x - eps) e |= 0xF0;
        if (p.x <= cr.x + eps) e |= 0x0F;
        if (p.y >= cr.y - eps) f |= 0xCC;
        if (p.y <= cr.y + eps) f |= 0x33;
        mask |= e & f;
    }
    return mask;
}

struct Entry {
    uint32_t index;
    int child_mask, visit_mask;
};

uint64_t morton(const uint32_t p[3], int depth) {
    uint64_t code = 0;
    for (int b = 0; b < depth; ++b)
        code |= (uint64_t)((p[0] >> b) & 1) << (3 * b + 2) | (uint64_t)((p[1] >> b) & 1) << (3 * b + 1) |
                (uint64_t)((p[2] >> b) & 1) << (3 * b);
    return code;
}

// One pixel. Returns false on a read outside the word array.
bool trace_pixel(const uint32_t* w, uint64_t nw, int depth, const Params& P, uint32_t px, uint32_t py,
                 uint32_t* color, uint64_t* hit) {
    auto word = [&](uint64_t i, bool& ok) -> uint32_t {
        if (i >= nw) { ok = false; return 0; }
        return w[i];
    };
    bool ok = true;
    // DAGTracer.cu:310-318: ray in double, then float.
    D3 v;
    v.x = P.ray_min[0] + double(px) * P.ray_ddx[0] + double(py) * P.ray_ddy[0] - P.camera[0];
    v.y = P.ray_min[1] + double(px) * P.ray_ddx[1] + double(py) * P.ray_ddy[1] - P.camera[1];
    v.z = P.ray_min[2] + double(px) * P.ray_ddx[2] + double(py) * P.ray_ddy[2] - P.camera[2];
    const double len = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
    const double s = 1 / len;
    const F3 org = {float(P.camera[0]), float(P.camera[1]), float(P.camera[2])};
    const F3 dir = {float(s * v.x), float(s * v.y), float(s * v.z)};
    const F3 inv = {float(1. / double(dir.x)), float(1. / double(dir.y)), float(1. / double(dir.z))};
    const int order = (dir.x < 0.f ? 4 : 0) + (dir.y < 0.f ? 2 : 0) + (dir.z < 0.f ? 1 : 0);

    const int leaf_level = depth - 2;
    uint32_t debug_index = 0;
    int level = 0;
    uint32_t path[3] = {0, 0, 0};
    Entry stack[64];
    Entry cache;
    uint32_t leaf_lo = 0, leaf_hi = 0;
    cache.index = 0;
    cache.child_mask = (int)(word(0, ok) & 0xFF);
    cache.visit_mask = cache.child_mask & intersection_mask(true, depth, 0, path, org, dir, inv);
    bool hit_voxel = false;
    for (;;) {
        // Ascend while no child is left (DAGTracer.cu:327-341).
        int nl = level;
        while (nl > 0 && !cache.visit_mask) {
            --nl;
            cache = stack[nl];
        }
        if (nl == 0 && !cache.visit_mask) {
            path[0] = path[1] = path[2] = 0;
            break;
        }
        for (int a = 0; a < 3; ++a) path[a] >>= (level - nl);
        level = nl;
        const int child = next_child(order, cache.visit_mask);
        cache.visit_mask &= ~(1 << child);
        // Descend (DAGTracer.cu:350-412).
        path[0] = (path[0] << 1) | ((child & 4) >> 2);
        path[1] = (path[1] << 1) | ((child & 2) >> 1);
        path[2] = (path[2] << 1) | (child & 1);
        stack[level] = cache;
        ++level;
        if ((uint32_t)(depth - 2 - level) == P.debug_level) debug_index = cache.index;
        if (level == depth) { hit_voxel = true; break; }
        auto child_ptr = [&]() -> uint32_t {  // Utils.h:72-75
            const uint32_t m = (uint32_t)cache.child_mask & ((1u << child) - 1u);
            return word((uint64_t)cache.index + (uint64_t)__builtin_popcount(m) + 1, ok);
        };
        if (level < leaf_level) {
            cache.index = child_ptr();
            cache.child_mask = (int)(word(cache.index, ok) & 0xFF);
            cache.visit_mask = cache.child_mask & intersection_mask(false, depth, level, path, org, dir, inv);
        } else {
            int cm;
            if (level == leaf_level) {
                const uint32_t addr = child_ptr();
                leaf_lo = word(addr, ok);
                leaf_hi = word((uint64_t)addr + 1, ok);
                cm = 0;
                for (int b = 0; b < 4; ++b) {
                    if ((leaf_lo >> (8 * b)) & 0xFF) cm |= 1 << b;
                    if ((leaf_hi >> (8 * b)) & 0xFF) cm |= 1 << (4 + b);
                }
            } else {
                cm = (int)((((child & 4) ? leaf_hi : leaf_lo) >> ((child & 3) * 8)) & 0xFF);
            }
            cache.child_mask = cm;
            cache.visit_mask = cm & intersection_mask(false, depth, level, path, org, dir, inv);
        }
        if (!ok) break;
    }
    if (P.debug_level == 0xFFFFFFFFu)
        *color = rgb888(float(path[0] & 0xFF) / float(0xFF), float(path[1] & 0xFF) / float(0xFF),
                        float(path[2] & 0xFF) / float(0xFF));
    else
        *color = murmur32(debug_index);
    *hit = hit_voxel ? morton(path, depth) : ~0ull;
    return ok;
}

}  // namespace

extern "C" {

// Traces params->width x params->height rays (row-major, pixel (x, y) at
// y * width + x). hits: Morton code of the voxel hit, ~0 for a miss. Returns
// the number of pixels whose traversal read outside the word array.
uint64_t oracle_trace(const uint32_t* words, uint64_t n_words, int depth, const void* params, uint32_t* colors,
                      uint64_t* hits, int threads) {
    const Params& P = *static_cast<const Params*>(params);
    const uint64_t np = (uint64_t)P.width * P.height;
    std::vector<uint64_t> bad(threads > 0 ? threads : 1, 0);
    auto run = [&](int t, int nt) {
        for (uint64_t i = t; i < np; i += nt) {
            const uint32_t x = (uint32_t)(i % P.width), y = (uint32_t)(i / P.width);
            if (!trace_pixel(words, n_words, depth, P, x, y, colors + i, hits + i)) ++bad[t];
        }
    };
    const int nt = threads > 0 ? threads : 1;
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(run, t, nt);
    run(0, nt);
    for (auto& th : pool) th.join();
    uint64_t total = 0;
    for (uint64_t b : bad) total += b;
    return total;
}

}  // extern "C"
