// TEST INFRASTRUCTURE ONLY: CPU restatement of the reference's GL voxelizer,
// the checker of dagc_voxelize's reference mode. Parity of this restatement is
// UNPINNED: the reference rasterises with OpenGL (shaders + the GPU's
// conservative rasteriser), which cannot run here; this file fixes the
// rasteriser's behaviour as the ideal one (a pixel is covered when the
// projected triangle touches its square) and does all arithmetic in float32
// with one rounding per operation, like the CUDA kernel (built with
// --fmad=false; this file with -ffp-contract=off).
//
// Follows:
//   Shaders/GeometryShader.glsl:21-53   dominant axis of the face normal
//                                        scaled by the box half-size
//   src/Voxelizer.cpp:93-149            one orthographic view per axis over
//                                        the box (here: the affine map of the
//                                        box onto the 2^depth grid)
//   Shaders/FragmentShader.glsl:175-211 per covered pixel, depth samples at
//                                        the centre and the four corners
//                                        (+-dz/dx/2 +-dz/dy/2), truncated and
//                                        clamped to the grid, sorted; only the
//                                        first (the smallest) is emitted (the
//                                        loop `i < 1` at :191); axes swizzled
//                                        back (:196-207), Morton code (:19-32)

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

namespace {

uint64_t morton3(uint64_t x, uint64_t y, uint64_t z) {
    uint64_t c = 0;
    for (int b = 0; b < 21; ++b)
        c |= ((x >> b) & 1) << (3 * b + 2) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b);
    return c;
}

int clamp_cell(float z, int G) {
    const int k = (int)std::fmin(std::fmax(z, -1.0f), (float)G);
    return k < 0 ? 0 : (k > G - 1 ? G - 1 : k);
}

void gl_triangle(const double* P, const double* aabb, int depth, std::vector<uint64_t>& out) {
    const int G = 1 << depth;
    const float Gf = (float)G;
    float p[3][3], mn[3], mx[3];
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < 3; ++a) p[k][a] = (float)P[3 * k + a];
    for (int a = 0; a < 3; ++a) { mn[a] = (float)aabb[a]; mx[a] = (float)aabb[3 + a]; }
    // Dominant axis (GeometryShader.glsl:23-53).
    const float e1[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    const float e2[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
    const float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const float len = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    float nd[3];
    for (int a = 0; a < 3; ++a) nd[a] = std::fabs((c[a] / len) * ((mx[a] - mn[a]) * 0.5f));
    const int axis = nd[0] >= nd[2] ? (nd[0] >= nd[1] ? 0 : 1) : (nd[1] >= nd[2] ? 1 : 2);
    // Screen axes u, v and depth w of each view (Voxelizer.cpp:93-106 with
    // FragmentShader.glsl:196-207): X -> (z, y, x), Y -> (x, z, y), Z -> (y, x, z).
    static const int kU[3] = {2, 0, 1}, kV[3] = {1, 2, 0}, kW[3] = {0, 1, 2};
    float U[3], V[3], W[3];
    for (int k = 0; k < 3; ++k) {
        float g[3];
        for (int a = 0; a < 3; ++a) g[a] = (p[k][a] - mn[a]) * (Gf / (mx[a] - mn[a]));
        U[k] = g[kU[axis]];
        V[k] = g[kV[axis]];
        W[k] = g[kW[axis]];
    }
    const float e1u = U[1] - U[0], e1v = V[1] - V[0], e1w = W[1] - W[0];
    const float e2u = U[2] - U[0], e2v = V[2] - V[0], e2w = W[2] - W[0];
    const float det = e1u * e2v - e2u * e1v;
    if (!(det != 0.0f) || !std::isfinite(det)) return;  // no area in this view: no fragment
    const float dwdu = (e1w * e2v - e2w * e1v) / det;
    const float dwdv = (e2w * e1u - e1w * e2u) / det;
    const float sgn = det > 0.0f ? 1.0f : -1.0f;
    float nx[3], ny[3], dk[3];
    for (int k = 0; k < 3; ++k) {
        const int k1 = (k + 1) % 3;
        nx[k] = -(V[k1] - V[k]) * sgn;
        ny[k] = (U[k1] - U[k]) * sgn;
        dk[k] = std::fmax(nx[k], 0.0f) + std::fmax(ny[k], 0.0f);
    }
    auto lo_cell = [&](float a, float b, float c3) {
        const float m = std::fmin(a, std::fmin(b, c3));
        const int i = (int)std::floor(std::fmin(std::fmax(m, -1.0f), Gf));
        return i < 0 ? 0 : i;
    };
    auto hi_cell = [&](float a, float b, float c3) {
        const float m = std::fmax(a, std::fmax(b, c3));
        const int i = (int)std::floor(std::fmin(std::fmax(m, -1.0f), Gf));
        return i > G - 1 ? G - 1 : i;
    };
    const int i0 = lo_cell(U[0], U[1], U[2]), i1 = hi_cell(U[0], U[1], U[2]);
    const int j0 = lo_cell(V[0], V[1], V[2]), j1 = hi_cell(V[0], V[1], V[2]);
    for (int j = j0; j <= j1; ++j) {
        for (int i = i0; i <= i1; ++i) {
            bool covered = true;
            for (int k = 0; k < 3; ++k)
                covered = covered && nx[k] * ((float)i - U[k]) + ny[k] * ((float)j - V[k]) + dk[k] >= 0.0f;
            if (!covered) continue;
            const float zc = W[0] + dwdu * (((float)i + 0.5f) - U[0]) + dwdv * (((float)j + 0.5f) - V[0]);
            const float hx = 0.5f * dwdu, hy = 0.5f * dwdv;
            int k = clamp_cell(zc, G);
            const int s1 = clamp_cell(zc + hx + hy, G), s2 = clamp_cell(zc + hx - hy, G);
            const int s3 = clamp_cell(zc - hx + hy, G), s4 = clamp_cell(zc - hx - hy, G);
            k = std::min(std::min(std::min(k, s1), std::min(s2, s3)), s4);
            uint64_t xyz[3];
            xyz[kU[axis]] = (uint64_t)i;
            xyz[kV[axis]] = (uint64_t)j;
            xyz[kW[axis]] = (uint64_t)k;
            out.push_back(morton3(xyz[0], xyz[1], xyz[2]));
        }
    }
}

}  // namespace

extern "C" {

// GL-rule voxelisation of n triangles (9 doubles each, world units) in the box
// aabb = (min xyz, max xyz) onto the 2^depth grid. Codes in triangle order,
// per triangle in row-major pixel order (rows of the view's v axis). Writes
// up to cap codes; returns the total.
uint64_t oracle_voxelize_gl(const double* vertices, uint64_t n, const double* aabb, int depth, uint64_t* codes,
                            uint64_t cap) {
    std::vector<uint64_t> out;
    for (uint64_t t = 0; t < n; ++t) gl_triangle(vertices + 9 * t, aabb, depth, out);
    for (uint64_t i = 0; i < out.size() && i < cap; ++i) codes[i] = out[i];
    return out.size();
}

}  // extern "C"
