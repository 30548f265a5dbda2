// Triangle voxelizer for sm_103a: the fragment producer in front of the DAG
// path. Restates in CUDA the reference's OpenGL voxelization pass
// (src/Voxelizer.cpp:254-369 with Shaders/GeometryShader.glsl and
// Shaders/FragmentShader.glsl), which cannot run on a compute-only box, and
// writes Morton codes to a device buffer, ready for dagc_create.
//
// Two rules:
//   kVoxGL  the reference's: each triangle is projected on the plane of its
//           dominant axis (face normal scaled by the box half-size), every
//           pixel (voxel column) the projection touches is covered
//           (conservative rasterisation), and each covered pixel emits ONE
//           voxel, at the smallest of the plane depths sampled at the pixel
//           centre and corners (truncated, clamped to the grid). float32.
//   kVoxSAT every voxel whose cube the triangle touches, by the separating
//           axis test (Akenine-Moller 2001); float64. The 26-connected
//           surface used for the triangle-soup workload.
//
// One warp per triangle, lanes striding over the triangle's bounding box
// (rows of pixels / voxel columns), so that large triangles spread over 32
// lanes; per-tile fragment counts give the output offsets through a single
// decoupled look-back, so the output order is fixed: triangles in input
// order, each triangle's fragments in bounding-box order. This file is
// compiled with --fmad=false: every float operation rounds once, as in the
// CPU checkers.

#include "dagc_device.cuh"
#include "dagc_kernels.h"

namespace dagc {
namespace {

constexpr int kVoxThreads = 256;
constexpr int kVoxWarps = kVoxThreads / 32;
constexpr int kVoxTile = kVoxThreads;  // triangles per tile, one per thread for the scan

__device__ __forceinline__ uint64_t morton3(uint64_t x, uint64_t y, uint64_t z) {
    uint64_t c = 0;
#pragma unroll 1
    for (int b = 0; b < 21; ++b)
        c |= ((x >> b) & 1) << (3 * b + 2) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b);
    return c;
}

// ---------------------------------------------------------------- GL rule --
struct GlTri {
    int axis;
    float U[3], V[3], W[3];
    float dwdu, dwdv;
    float nx[3], ny[3], dk[3];
    int i0, i1, j0, j1;
    bool empty;
};

__device__ __forceinline__ int lo_cell(float m, float Gf) {
    const int i = (int)floorf(fminf(fmaxf(m, -1.0f), Gf));
    return i < 0 ? 0 : i;
}
__device__ __forceinline__ int hi_cell(float m, float Gf, int G) {
    const int i = (int)floorf(fminf(fmaxf(m, -1.0f), Gf));
    return i > G - 1 ? G - 1 : i;
}
__device__ __forceinline__ int clamp_cell(float z, int G) {
    const int k = (int)fminf(fmaxf(z, -1.0f), (float)G);
    return k < 0 ? 0 : (k > G - 1 ? G - 1 : k);
}

__device__ GlTri gl_setup(const double* P, const double* aabb, int depth) {
    GlTri t;
    const int G = 1 << depth;
    const float Gf = (float)G;
    float p[3][3], mn[3], mx[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a) p[k][a] = (float)P[3 * k + a];
#pragma unroll
    for (int a = 0; a < 3; ++a) { mn[a] = (float)aabb[a]; mx[a] = (float)aabb[3 + a]; }
    const float e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    const float e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
    const float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const float len = sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    float nd[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) nd[a] = fabsf((c[a] / len) * ((mx[a] - mn[a]) * 0.5f));
    t.axis = nd[0] >= nd[2] ? (nd[0] >= nd[1] ? 0 : 1) : (nd[1] >= nd[2] ? 1 : 2);
    // View axes: X -> (u, v, w) = (z, y, x), Y -> (x, z, y), Z -> (y, x, z).
    const int ua = t.axis == 0 ? 2 : (t.axis == 1 ? 0 : 1);
    const int va = t.axis == 0 ? 1 : (t.axis == 1 ? 2 : 0);
    const int wa = t.axis;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float g[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) g[a] = (p[k][a] - mn[a]) * (Gf / (mx[a] - mn[a]));
        t.U[k] = g[ua];
        t.V[k] = g[va];
        t.W[k] = g[wa];
    }
    const float e1u = t.U[1] - t.U[0], e1v = t.V[1] - t.V[0], e1w = t.W[1] - t.W[0];
    const float e2u = t.U[2] - t.U[0], e2v = t.V[2] - t.V[0], e2w = t.W[2] - t.W[0];
    const float det = e1u * e2v - e2u * e1v;
    t.empty = !(det != 0.0f) || !isfinite(det);
    t.dwdu = (e1w * e2v - e2w * e1v) / det;
    t.dwdv = (e2w * e1u - e1w * e2u) / det;
    const float sgn = det > 0.0f ? 1.0f : -1.0f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int k1 = k == 2 ? 0 : k + 1;
        t.nx[k] = -(t.V[k1] - t.V[k]) * sgn;
        t.ny[k] = (t.U[k1] - t.U[k]) * sgn;
        t.dk[k] = fmaxf(t.nx[k], 0.0f) + fmaxf(t.ny[k], 0.0f);
    }
    t.i0 = lo_cell(fminf(t.U[0], fminf(t.U[1], t.U[2])), Gf);
    t.i1 = hi_cell(fmaxf(t.U[0], fmaxf(t.U[1], t.U[2])), Gf, G);
    t.j0 = lo_cell(fminf(t.V[0], fminf(t.V[1], t.V[2])), Gf);
    t.j1 = hi_cell(fmaxf(t.V[0], fmaxf(t.V[1], t.V[2])), Gf, G);
    if (t.i0 > t.i1 || t.j0 > t.j1) t.empty = true;
    return t;
}

// Pixel (i, j): covered? and its voxel's Morton code.
__device__ __forceinline__ bool gl_pixel(const GlTri& t, int i, int j, int G, uint64_t* code) {
    bool covered = true;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        covered = covered && t.nx[k] * ((float)i - t.U[k]) + t.ny[k] * ((float)j - t.V[k]) + t.dk[k] >= 0.0f;
    if (!covered) return false;
    const float zc = t.W[0] + t.dwdu * (((float)i + 0.5f) - t.U[0]) + t.dwdv * (((float)j + 0.5f) - t.V[0]);
    const float hx = 0.5f * t.dwdu, hy = 0.5f * t.dwdv;
    const int s0 = clamp_cell(zc, G);
    const int s1 = clamp_cell(zc + hx + hy, G), s2 = clamp_cell(zc + hx - hy, G);
    const int s3 = clamp_cell(zc - hx + hy, G), s4 = clamp_cell(zc - hx - hy, G);
    const int k = min(min(min(s0, s1), min(s2, s3)), s4);
    uint64_t xyz[3];
    const int ua = t.axis == 0 ? 2 : (t.axis == 1 ? 0 : 1);
    const int va = t.axis == 0 ? 1 : (t.axis == 1 ? 2 : 0);
    xyz[ua] = (uint64_t)i;
    xyz[va] = (uint64_t)j;
    xyz[t.axis] = (uint64_t)k;
    *code = morton3(xyz[0], xyz[1], xyz[2]);
    return true;
}

// --------------------------------------------------------------- SAT rule --
struct D3 { double x, y, z; };
__device__ __forceinline__ D3 dsub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 dcross(D3 a, D3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double ddot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }  // std::min
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }  // std::max

// Triangle (a, b, d) against the cube of half-size h around c: 9 edge-cross
// axes, the 3 box normals, the triangle normal; touching counts as overlap.
__device__ bool tri_box(D3 c, double h, D3 a, D3 b, D3 d) {
    const D3 v0 = dsub(a, c), v1 = dsub(b, c), v2 = dsub(d, c);
    const D3 e[3] = {dsub(v1, v0), dsub(v2, v1), dsub(v0, v2)};
    const D3 ax[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const D3 axis = dcross(ax[i], e[j]);
            const double p0 = ddot(axis, v0), p1 = ddot(axis, v1), p2 = ddot(axis, v2);
            const double mn = dmin(p0, dmin(p1, p2));
            const double mx = dmax(p0, dmax(p1, p2));
            const double r = h * (fabs(axis.x) + fabs(axis.y) + fabs(axis.z));
            if (mn > r || mx < -r) return false;
        }
    }
    if (dmin(v0.x, dmin(v1.x, v2.x)) > h || dmax(v0.x, dmax(v1.x, v2.x)) < -h) return false;
    if (dmin(v0.y, dmin(v1.y, v2.y)) > h || dmax(v0.y, dmax(v1.y, v2.y)) < -h) return false;
    if (dmin(v0.z, dmin(v1.z, v2.z)) > h || dmax(v0.z, dmax(v1.z, v2.z)) < -h) return false;
    const D3 nrm = dcross(e[0], e[1]);
    const double dist = ddot(nrm, v0);
    const double r = h * (fabs(nrm.x) + fabs(nrm.y) + fabs(nrm.z));
    return fabs(dist) <= r;
}

struct SatTri {
    D3 v[3];
    int64_t x0, y0, z0, nx, ny, nz;  // bounding box origin and extents (0 extent: empty)
};

__device__ __forceinline__ int64_t cell_floor(double m, double G) { return (int64_t)floor(dmin(dmax(m, -1.0), G)); }

__device__ SatTri sat_setup(const double* P, const double* aabb, int depth) {
    SatTri t;
    const double G = (double)((int64_t)1 << depth);
    const int64_t Gi = (int64_t)1 << depth;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        t.v[k].x = (P[3 * k + 0] - aabb[0]) * (G / (aabb[3] - aabb[0]));
        t.v[k].y = (P[3 * k + 1] - aabb[1]) * (G / (aabb[4] - aabb[1]));
        t.v[k].z = (P[3 * k + 2] - aabb[2]) * (G / (aabb[5] - aabb[2]));
    }
    const D3 a = t.v[0], b = t.v[1], c = t.v[2];
    int64_t x0 = cell_floor(dmin(a.x, dmin(b.x, c.x)), G), x1 = cell_floor(dmax(a.x, dmax(b.x, c.x)), G);
    int64_t y0 = cell_floor(dmin(a.y, dmin(b.y, c.y)), G), y1 = cell_floor(dmax(a.y, dmax(b.y, c.y)), G);
    int64_t z0 = cell_floor(dmin(a.z, dmin(b.z, c.z)), G), z1 = cell_floor(dmax(a.z, dmax(b.z, c.z)), G);
    x0 = x0 < 0 ? 0 : x0; y0 = y0 < 0 ? 0 : y0; z0 = z0 < 0 ? 0 : z0;
    x1 = x1 > Gi - 1 ? Gi - 1 : x1; y1 = y1 > Gi - 1 ? Gi - 1 : y1; z1 = z1 > Gi - 1 ? Gi - 1 : z1;
    t.x0 = x0; t.y0 = y0; t.z0 = z0;
    t.nx = x1 >= x0 ? x1 - x0 + 1 : 0;
    t.ny = y1 >= y0 ? y1 - y0 + 1 : 0;
    t.nz = z1 >= z0 ? z1 - z0 + 1 : 0;
    return t;
}

// ------------------------------------------------------------------ kernel --
struct VoxSmem {
    uint64_t count[kVoxTile];
    uint64_t scan[34];
    uint32_t slot;
    uint64_t base;
};

// Fragments of triangle `tri` counted (kEmit false) or written from
// out[pos] on (kEmit true) by the whole warp; returns the count. Every lane
// runs the same loop trip count, so each ballot is made by all 32 lanes.
template <int kMode, bool kEmit>
__device__ uint64_t warp_triangle(const VoxArgs& a, uint64_t tri, uint64_t pos) {
    const uint32_t lane = threadIdx.x & 31;
    const double* P = a.vertices + 9 * tri;
    const int G = 1 << a.depth;
    uint64_t n = 0;
    if (kMode == kVoxGL) {
        const GlTri t = gl_setup(P, a.aabb, a.depth);
        if (t.empty) return 0;
        const uint64_t w = (uint64_t)(t.i1 - t.i0 + 1), area = w * (uint64_t)(t.j1 - t.j0 + 1);
        for (uint64_t b = 0; b < area; b += 32) {
            const uint64_t idx = b + lane;
            uint64_t code = 0;
            const bool hit = idx < area && gl_pixel(t, t.i0 + (int)(idx % w), t.j0 + (int)(idx / w), G, &code);
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, hit);
            if (kEmit && hit) {
                const uint64_t o = pos + n + __popc(m & lanemask_lt());
                if (o < a.capacity) a.codes[o] = code;
            }
            n += __popc(m);
        }
    } else {
        const SatTri t = sat_setup(P, a.aabb, a.depth);
        const uint64_t area = (uint64_t)t.nx * (uint64_t)t.ny * (uint64_t)t.nz;
        const uint64_t yz = (uint64_t)t.ny * (uint64_t)t.nz;
        for (uint64_t b = 0; b < area; b += 32) {
            const uint64_t idx = b + lane;
            bool hit = false;
            int64_t x = 0, y = 0, z = 0;
            if (idx < area) {
                x = t.x0 + (int64_t)(idx / yz);
                const uint64_t r = idx % yz;
                y = t.y0 + (int64_t)(r / (uint64_t)t.nz);
                z = t.z0 + (int64_t)(r % (uint64_t)t.nz);
                const D3 c{(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
                hit = tri_box(c, 0.5, t.v[0], t.v[1], t.v[2]);
            }
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, hit);
            if (kEmit && hit) {
                const uint64_t o = pos + n + __popc(m & lanemask_lt());
                if (o < a.capacity) a.codes[o] = morton3((uint64_t)x, (uint64_t)y, (uint64_t)z);
            }
            n += __popc(m);
        }
    }
    return n;
}

template <int kMode>
__global__ void __launch_bounds__(kVoxThreads) voxelize(VoxArgs a) {
    __shared__ VoxSmem S;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t ntiles = (a.n_tri + kVoxTile - 1) / kVoxTile;
    while (true) {
        if (tid == 0) S.slot = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const uint64_t tile = S.slot;
        __syncthreads();
        if (tile >= ntiles) break;
        const uint64_t t0 = tile * kVoxTile;
        // Count: warp w takes triangles t0 + w, t0 + w + 8, ...
        for (uint32_t k = warp; k < kVoxTile; k += kVoxWarps) {
            const uint64_t tri = t0 + k;
            const uint64_t c = tri < a.n_tri ? warp_triangle<kMode, false>(a, tri, 0) : 0;
            if (lane == 0) S.count[k] = c;
        }
        __syncthreads();
        uint64_t total;
        const uint64_t excl = block_exclusive_sum<uint64_t>(S.count[tid], S.scan, &total);
        __syncthreads();
        S.count[tid] = excl;  // now the triangle's offset inside the tile
        if (warp == 0) {
            const uint64_t b = sv_lookback(a.status, (uint32_t)tile, total, a.err);
            if (lane == 0) S.base = b;
        }
        __syncthreads();
        const uint64_t base = S.base;
        for (uint32_t k = warp; k < kVoxTile; k += kVoxWarps) {
            const uint64_t tri = t0 + k;
            if (tri < a.n_tri) warp_triangle<kMode, true>(a, tri, base + S.count[k]);
        }
        if (tid == 0 && tile == ntiles - 1) *a.d_total = base + total;
        __syncthreads();
    }
}

}  // namespace

void launch_voxelize(const VoxArgs& a, int grid, cudaStream_t s) {
    if (a.mode == kVoxGL) voxelize<kVoxGL><<<grid, kVoxThreads, 0, s>>>(a);
    else voxelize<kVoxSAT><<<grid, kVoxThreads, 0, s>>>(a);
}

uint64_t voxelize_tiles(uint64_t n_tri) { return (n_tri + kVoxTile - 1) / kVoxTile; }

}  // namespace dagc
