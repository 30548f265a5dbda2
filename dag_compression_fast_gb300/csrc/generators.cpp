// Seeded synthetic voxel-fragment generators.
//
// They stand in for the reference's OpenGL voxelizer (src/Voxelizer.cpp:254-310,
// Shaders/FragmentShader.glsl:164-211), which cannot run without a graphics
// stack: each returns shuffled uint64 Morton fragment codes with duplicates,
// exactly the input DAGCompression::CreateDAG consumes.
//
// Morton order follows mortonEncode64 (src/DAG_Compression_Fast.cpp:223-236):
// in every 3-bit group bit 2 is x, bit 1 is y, bit 0 is z.
//
// Determinism: PRNG = SplitMix64 seeding xoshiro256**; every per-item random
// stream is derived from (seed, item index), so the multi-threaded generators
// give the same output for any thread count. Floating point is IEEE double
// with contraction disabled (-ffp-contract=off) and no libm transcendental
// calls, so x86-64 and aarch64 hosts produce identical codes.

#include "../../include/dagc_gen.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- PRNG ----
inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix64(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint64_t below(uint64_t bound) {  // Lemire multiply-shift, bound > 0
        return (uint64_t)(((unsigned __int128)next() * bound) >> 64);
    }
};

inline uint64_t mix3(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
    uint64_t s = seed ^ (a * 0x9e3779b97f4a7c15ull);
    splitmix64(s);
    s ^= b * 0xc2b2ae3d27d4eb4full;
    splitmix64(s);
    s ^= c * 0x165667b19e3779f9ull;
    return splitmix64(s);
}

// ------------------------------------------------------------- Morton ----
inline uint64_t split_by_3(uint64_t a) {
    uint64_t x = a & 0x1fffff;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}
inline uint64_t morton(uint64_t x, uint64_t y, uint64_t z) {
    return split_by_3(x) << 2 | split_by_3(y) << 1 | split_by_3(z);
}

// ------------------------------------------- deterministic math helpers ----
// 2^x for x in [0, 8): integer part by doubling, fractional part by the
// Taylor series of e^(f ln 2) (20 terms, below one ulp on [0, 1)).
double exp2_det(double x) {
    int k = (int)x;
    double f = x - k;
    const double ln2 = 0.6931471805599453;
    double t = f * ln2, term = 1.0, sum = 1.0;
    for (int i = 1; i < 20; ++i) { term = term * t / i; sum += term; }
    double r = sum;
    for (int i = 0; i < k; ++i) r *= 2.0;
    return r;
}

// log2(x) for x > 0: exact exponent from frexp, mantissa by the atanh series
// ln(m) = 2 atanh((m - 1) / (m + 1)), |z| <= 1/3 so 40 terms are exact to an ulp.
double log2_det(double x) {
    int e = 0;
    const double m = std::frexp(x, &e);  // x = m * 2^e, m in [0.5, 1)
    const double z = (m - 1.0) / (m + 1.0), z2 = z * z;
    double term = z, sum = 0.0;
    for (int k = 0; k < 40; ++k) { sum += term / (2 * k + 1); term *= z2; }
    return (double)e + 2.0 * sum / 0.6931471805599453;
}

inline double smoothstep(double t) { return t * t * (3.0 - 2.0 * t); }

// Value noise on a seeded hash lattice with smoothstep interpolation.
double value_noise(uint64_t seed, uint64_t octave, double x, double z) {
    const double fx = std::floor(x), fz = std::floor(z);
    const int64_t ix = (int64_t)fx, iz = (int64_t)fz;
    const double tx = smoothstep(x - fx), tz = smoothstep(z - fz);
    auto lat = [&](int64_t a, int64_t b) {
        return (double)(mix3(seed, octave, (uint64_t)a, (uint64_t)b) >> 11) * (1.0 / 9007199254740992.0);
    };
    const double v00 = lat(ix, iz), v10 = lat(ix + 1, iz);
    const double v01 = lat(ix, iz + 1), v11 = lat(ix + 1, iz + 1);
    const double a = v00 + (v10 - v00) * tx;
    const double b = v01 + (v11 - v01) * tx;
    return a + (b - a) * tz;
}

// 4-octave fBm, lacunarity 2, gain 0.5, normalised to [0, 1).
double fbm4(uint64_t seed, double x, double z, double period) {
    double sum = 0.0, amp = 1.0, norm = 0.0, freq = 1.0 / period;
    for (int o = 0; o < 4; ++o) {
        sum += amp * value_noise(seed, (uint64_t)o, x * freq, z * freq);
        norm += amp;
        amp *= 0.5;
        freq *= 2.0;
    }
    return sum / norm;
}

// Emits each voxel 1..4 times (uniform) and shuffles (Fisher-Yates).
std::vector<uint64_t> duplicate_and_shuffle(const std::vector<uint64_t>& voxels, uint64_t seed,
                                            int max_dup) {
    Xoshiro rng(seed ^ 0xD0B1E5ull);
    std::vector<uint64_t> out;
    out.reserve(voxels.size() * (max_dup + 1) / 2 + 16);
    for (uint64_t v : voxels) {
        const uint64_t k = 1 + rng.below((uint64_t)max_dup);
        for (uint64_t i = 0; i < k; ++i) out.push_back(v);
    }
    for (uint64_t i = out.size(); i > 1; --i) {
        const uint64_t j = rng.below(i);
        std::swap(out[i - 1], out[j]);
    }
    return out;
}

int emit(std::vector<uint64_t>&& v, uint64_t** out, uint64_t* n) {
    *n = v.size();
    *out = (uint64_t*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(uint64_t));
    if (!*out) return 2;
    if (!v.empty()) std::memcpy(*out, v.data(), v.size() * sizeof(uint64_t));
    return 0;
}

// ------------------------------------------------------- sphere shell ----
void sphere_voxels(int depth, uint64_t seed, double target_fragments, std::vector<uint64_t>& vox) {
    const int64_t G = (int64_t)1 << depth;
    Xoshiro rng(seed);
    double R = 0.4375 * (double)G;  // 56 in a 128^3 grid
    if (target_fragments > 0) {
        // Shell of thickness 1 holds ~4 pi R^2 voxels; 2.5 fragments per voxel.
        R = std::sqrt(target_fragments / (2.5 * 4.0 * 3.141592653589793));
        R = std::min(R, 0.44 * (double)G);
        R = std::max(R, 3.0);
    }
    const double sign = (rng.next() & 1) ? 1.0 : -1.0;
    R += sign * 2.0 * rng.uniform();
    double c[3];
    for (double& ci : c) ci = 0.5 * (double)G + (4.0 * rng.uniform() - 2.0);
    const double rlo = R - 0.5, rhi = R + 0.5;
    auto axis_range = [&](double ci, int64_t& lo, int64_t& hi) {
        lo = std::max<int64_t>(0, (int64_t)std::floor(ci - rhi) - 1);
        hi = std::min<int64_t>(G - 1, (int64_t)std::floor(ci + rhi) + 1);
    };
    int64_t x0, x1, y0, y1;
    axis_range(c[0], x0, x1);
    axis_range(c[1], y0, y1);
    auto test_z = [&](int64_t x, int64_t y, double r2, int64_t z0, int64_t z1) {
        z0 = std::max<int64_t>(0, z0);
        z1 = std::min<int64_t>(G - 1, z1);
        for (int64_t z = z0; z <= z1; ++z) {
            const double dz = (double)z + 0.5 - c[2];
            const double d = std::sqrt(r2 + dz * dz);
            if (std::fabs(d - R) <= 0.5) vox.push_back(morton((uint64_t)x, (uint64_t)y, (uint64_t)z));
        }
    };
    for (int64_t x = x0; x <= x1; ++x) {
        const double dx = (double)x + 0.5 - c[0];
        for (int64_t y = y0; y <= y1; ++y) {
            const double dy = (double)y + 0.5 - c[1];
            const double r2 = dx * dx + dy * dy;
            if (r2 > rhi * rhi) continue;
            // Candidate z: |dz| between the inner and outer sphere, widened by
            // one voxel; the exact test above decides.
            const double zo = std::sqrt(rhi * rhi - r2);
            const double zi = r2 < rlo * rlo ? std::sqrt(rlo * rlo - r2) : 0.0;
            const int64_t a0 = (int64_t)std::floor(c[2] - zo) - 1, a1 = (int64_t)std::floor(c[2] - zi) + 1;
            const int64_t b0 = (int64_t)std::floor(c[2] + zi) - 1, b1 = (int64_t)std::floor(c[2] + zo) + 1;
            if (a1 >= b0) {
                test_z(x, y, r2, a0, b1);
            } else {
                test_z(x, y, r2, a0, a1);
                test_z(x, y, r2, b0, b1);
            }
        }
    }
}

// ------------------------------------------------------------ terrain ----
// Heightfield h(x, z) = G/4 + fbm * G/2; surface voxels y in [h-2, h].
void terrain_columns(int depth, uint64_t seed, double keep, int64_t x_lo, int64_t x_hi,
                     int64_t z_lo, int64_t z_hi, double period, int64_t base, int64_t amp,
                     int64_t y_offset, int local_depth, std::vector<uint64_t>& vox) {
    const int64_t G = (int64_t)1 << depth;
    (void)G;
    const uint64_t keep_q = keep >= 1.0 ? ~0ull : (uint64_t)(keep * 18446744073709551616.0);
    for (int64_t x = x_lo; x < x_hi; ++x) {
        for (int64_t z = z_lo; z < z_hi; ++z) {
            if (keep < 1.0 && mix3(seed ^ 0xC01ull, (uint64_t)x, (uint64_t)z, 7) >= keep_q) continue;
            const double f = fbm4(seed, (double)x, (double)z, period);
            const int64_t h = base + (int64_t)std::floor(f * (double)amp);
            for (int64_t y = h - 2; y <= h; ++y) {
                const int64_t ly = y - y_offset;
                if (ly < 0 || ly >= ((int64_t)1 << local_depth)) continue;
                const int64_t lx = x - x_lo, lz = z - z_lo;
                vox.push_back(morton((uint64_t)lx, (uint64_t)ly, (uint64_t)lz));
            }
        }
    }
}

// ------------------------------------------------------ triangle soup ----
struct V3 { double x, y, z; };
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Triangle / axis-aligned box overlap by the separating axis theorem
// (Akenine-Moller, "Fast 3D Triangle-Box Overlap Testing", 2001): 9 edge
// cross axes, the 3 box normals and the triangle normal. Touching counts as
// overlap (conservative).
bool tri_box_overlap(V3 c, double h, V3 a, V3 b, V3 d) {
    const V3 v0 = sub(a, c), v1 = sub(b, c), v2 = sub(d, c);
    const V3 e[3] = {sub(v1, v0), sub(v2, v1), sub(v0, v2)};
    const V3 ax[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < 3; ++j) {
            const V3 axis = cross(ax[i], e[j]);
            const double p0 = dot(axis, v0), p1 = dot(axis, v1), p2 = dot(axis, v2);
            const double mn = std::min(p0, std::min(p1, p2));
            const double mx = std::max(p0, std::max(p1, p2));
            const double r = h * (std::fabs(axis.x) + std::fabs(axis.y) + std::fabs(axis.z));
            if (mn > r || mx < -r) return false;
        }
    }
    if (std::min(v0.x, std::min(v1.x, v2.x)) > h || std::max(v0.x, std::max(v1.x, v2.x)) < -h) return false;
    if (std::min(v0.y, std::min(v1.y, v2.y)) > h || std::max(v0.y, std::max(v1.y, v2.y)) < -h) return false;
    if (std::min(v0.z, std::min(v1.z, v2.z)) > h || std::max(v0.z, std::max(v1.z, v2.z)) < -h) return false;
    const V3 nrm = cross(e[0], e[1]);
    const double dist = dot(nrm, v0);
    const double r = h * (std::fabs(nrm.x) + std::fabs(nrm.y) + std::fabs(nrm.z));
    return std::fabs(dist) <= r;
}

V3 random_direction(Xoshiro& rng) {
    for (;;) {
        V3 v{2 * rng.uniform() - 1, 2 * rng.uniform() - 1, 2 * rng.uniform() - 1};
        const double l2 = dot(v, v);
        if (l2 > 1e-6 && l2 <= 1.0) {
            const double inv = 1.0 / std::sqrt(l2);
            return {v.x * inv, v.y * inv, v.z * inv};
        }
    }
}

// Triangle t of the soup: v0 uniform in the grid, two edges of log-uniform
// length in [1, 16] along uniform directions, clamped into the grid.
void soup_triangle(int depth, uint64_t seed, uint64_t t, V3 v[3]) {
    const double G = (double)((int64_t)1 << depth);
    Xoshiro rng(mix3(seed, t, 0x7A1, 0));
    const V3 v0{rng.uniform() * G, rng.uniform() * G, rng.uniform() * G};
    const double l1 = exp2_det(4.0 * rng.uniform());  // log-uniform in [1, 16]
    const double l2 = exp2_det(4.0 * rng.uniform());
    const V3 d1 = random_direction(rng), d2 = random_direction(rng);
    V3 v1{v0.x + l1 * d1.x, v0.y + l1 * d1.y, v0.z + l1 * d1.z};
    V3 v2{v0.x + l2 * d2.x, v0.y + l2 * d2.y, v0.z + l2 * d2.z};
    auto clampv = [&](V3& q) {
        q.x = std::min(std::max(q.x, 0.0), G - 1e-9);
        q.y = std::min(std::max(q.y, 0.0), G - 1e-9);
        q.z = std::min(std::max(q.z, 0.0), G - 1e-9);
    };
    clampv(v1);
    clampv(v2);
    v[0] = v0;
    v[1] = v1;
    v[2] = v2;
}

void soup_triangles(int depth, uint64_t seed, uint64_t t_lo, uint64_t t_hi, std::vector<uint64_t>& out) {
    const int64_t Gi = (int64_t)1 << depth;
    for (uint64_t t = t_lo; t < t_hi; ++t) {
        V3 v[3];
        soup_triangle(depth, seed, t, v);
        const V3 v0 = v[0], v1 = v[1], v2 = v[2];
        const int64_t bx0 = (int64_t)std::floor(std::min(v0.x, std::min(v1.x, v2.x)));
        const int64_t by0 = (int64_t)std::floor(std::min(v0.y, std::min(v1.y, v2.y)));
        const int64_t bz0 = (int64_t)std::floor(std::min(v0.z, std::min(v1.z, v2.z)));
        const int64_t bx1 = std::min(Gi - 1, (int64_t)std::floor(std::max(v0.x, std::max(v1.x, v2.x))));
        const int64_t by1 = std::min(Gi - 1, (int64_t)std::floor(std::max(v0.y, std::max(v1.y, v2.y))));
        const int64_t bz1 = std::min(Gi - 1, (int64_t)std::floor(std::max(v0.z, std::max(v1.z, v2.z))));
        for (int64_t x = std::max<int64_t>(0, bx0); x <= bx1; ++x)
            for (int64_t y = std::max<int64_t>(0, by0); y <= by1; ++y)
                for (int64_t z = std::max<int64_t>(0, bz0); z <= bz1; ++z) {
                    const V3 c{(double)x + 0.5, (double)y + 0.5, (double)z + 0.5};
                    if (tri_box_overlap(c, 0.5, v0, v1, v2)) out.push_back(morton(x, y, z));
                }
    }
}

void shuffle(std::vector<uint64_t>& v, uint64_t seed) {
    Xoshiro rng(seed ^ 0x5EEDull);
    for (uint64_t i = v.size(); i > 1; --i) std::swap(v[i - 1], v[rng.below(i)]);
}

// ---------------------------------------------------- Menger sponge ----
bool menger_solid(int64_t x, int64_t y, int64_t z) {
    while (x || y || z) {
        const int ones = (x % 3 == 1) + (y % 3 == 1) + (z % 3 == 1);
        if (ones >= 2) return false;
        x /= 3; y /= 3; z /= 3;
    }
    return true;
}

}  // namespace

extern "C" {

void dagc_gen_free(void* p) { std::free(p); }

int dagc_gen_sphere_shell(int depth, uint64_t seed, double target_fragments, uint64_t** out,
                          uint64_t* n) {
    if (depth < 2 || depth > 21 || !out || !n) return 1;
    std::vector<uint64_t> vox;
    sphere_voxels(depth, seed, target_fragments, vox);
    return emit(duplicate_and_shuffle(vox, seed, 4), out, n);
}

int dagc_gen_terrain(int depth, uint64_t seed, double column_fraction, uint64_t** out, uint64_t* n) {
    if (depth < 3 || depth > 21 || !out || !n) return 1;
    const int64_t G = (int64_t)1 << depth;
    std::vector<uint64_t> vox;
    terrain_columns(depth, seed, column_fraction, 0, G, 0, G, (double)G / 4.0, G / 4, G / 2, 0, depth, vox);
    return emit(duplicate_and_shuffle(vox, seed, 4), out, n);
}

int dagc_gen_soup_triangles(int depth, uint64_t seed, uint64_t num_triangles, double* vertices) {
    if (depth < 2 || depth > 21 || (num_triangles && !vertices)) return 1;
    for (uint64_t t = 0; t < num_triangles; ++t) {
        V3 v[3];
        soup_triangle(depth, seed, t, v);
        for (int k = 0; k < 3; ++k) {
            vertices[9 * t + 3 * k + 0] = v[k].x;
            vertices[9 * t + 3 * k + 1] = v[k].y;
            vertices[9 * t + 3 * k + 2] = v[k].z;
        }
    }
    return 0;
}

int dagc_gen_triangle_soup(int depth, uint64_t seed, uint64_t num_triangles, int threads,
                           uint64_t** out, uint64_t* n) {
    if (depth < 2 || depth > 21 || !out || !n) return 1;
    if (threads < 1) threads = 1;
    const uint64_t per = (num_triangles + threads - 1) / threads;
    std::vector<std::vector<uint64_t>> parts(threads);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const uint64_t lo = std::min(num_triangles, per * t), hi = std::min(num_triangles, lo + per);
        pool.emplace_back([&, t, lo, hi] { soup_triangles(depth, seed, lo, hi, parts[t]); });
    }
    for (auto& th : pool) th.join();
    size_t total = 0;
    for (auto& p : parts) total += p.size();
    std::vector<uint64_t> all;
    all.reserve(total);
    for (auto& p : parts) { all.insert(all.end(), p.begin(), p.end()); std::vector<uint64_t>().swap(p); }
    shuffle(all, seed);
    return emit(std::move(all), out, n);
}

// Batched workload: chunks of 2^chunk_depth voxels per side laid on a
// grid_xz x grid_xz footprint at chunk row y = chunk_row, over one global fBm
// terrain (period = footprint / 4) with a level-5 Menger sponge (243^3) in
// every 8th chunk. Each chunk keeps a seeded random subset of its columns so
// that its fragment count follows its target (log-uniform in
// [min_fragments, max_fragments]). Chunks are returned in ascending Morton
// order of their (x, y, z) chunk coordinates; codes are chunk-local.
int dagc_gen_batched(int chunk_depth, int grid_xz, int chunk_row, uint64_t seed,
                     double min_fragments, double max_fragments, int threads,
                     uint64_t** codes, uint64_t* total, uint64_t** counts,
                     uint64_t** chunk_morton, uint64_t* num_chunks) {
    if (chunk_depth < 3 || chunk_depth > 16 || grid_xz < 1 || grid_xz > 64 || !codes || !total ||
        !counts || !chunk_morton || !num_chunks || min_fragments <= 0 || max_fragments < min_fragments)
        return 1;
    if (threads < 1) threads = 1;
    const int64_t C = (int64_t)1 << chunk_depth;
    const uint64_t K = (uint64_t)grid_xz * (uint64_t)grid_xz;
    struct Chunk { uint64_t morton_index; int64_t cx, cz; double target; };
    std::vector<Chunk> chunks;
    Xoshiro rng(seed);
    const double lmin = log2_det(min_fragments), lmax = log2_det(max_fragments);
    for (int cx = 0; cx < grid_xz; ++cx)
        for (int cz = 0; cz < grid_xz; ++cz) {
            const double u = rng.uniform();
            const double lt = lmin + (lmax - lmin) * u;
            const int ki = (int)std::floor(lt);
            const double target = exp2_det(lt - ki) * (double)((uint64_t)1 << ki);
            chunks.push_back({morton((uint64_t)cx, (uint64_t)chunk_row, (uint64_t)cz), cx, cz, target});
        }
    std::sort(chunks.begin(), chunks.end(), [](const Chunk& a, const Chunk& b) { return a.morton_index < b.morton_index; });
    std::vector<std::vector<uint64_t>> frags(K);
    std::vector<std::thread> pool;
    std::atomic_uint64_t next{0};
    const double period = (double)(C * grid_xz) / 4.0;
    for (int t = 0; t < threads; ++t) {
        pool.emplace_back([&] {
            for (;;) {
                const uint64_t k = next.fetch_add(1);
                if (k >= K) break;
                const Chunk& ch = chunks[k];
                const bool sponge = (mix3(seed, ch.cx, ch.cz, 0x5B0) & 7) == 0;
                const double full = 2.5 * (3.0 * (double)C * (double)C + (sponge ? 3200000.0 : 0.0));
                const double keep = std::min(1.0, ch.target / full);
                std::vector<uint64_t> vox;
                terrain_columns(chunk_depth + 4, seed, keep, ch.cx * C, ch.cx * C + C, ch.cz * C, ch.cz * C + C,
                                period, C / 4, C / 2, 0, chunk_depth, vox);
                if (sponge && C >= 243) {
                    const int64_t ox = (int64_t)(mix3(seed, ch.cx, ch.cz, 1) % (uint64_t)(C - 243));
                    const int64_t oy = C / 2;
                    const int64_t oz = (int64_t)(mix3(seed, ch.cx, ch.cz, 2) % (uint64_t)(C - 243));
                    const uint64_t keep_q = keep >= 1.0 ? ~0ull : (uint64_t)(keep * 18446744073709551616.0);
                    for (int64_t x = 0; x < 243; ++x)
                        for (int64_t z = 0; z < 243; ++z) {
                            if (keep < 1.0 && mix3(seed ^ 0xC01ull, (uint64_t)(ch.cx * C + ox + x),
                                                   (uint64_t)(ch.cz * C + oz + z), 7) >= keep_q)
                                continue;
                            for (int64_t y = 0; y < 243; ++y)
                                if (oy + y < C && menger_solid(x, y, z))
                                    vox.push_back(morton((uint64_t)(ox + x), (uint64_t)(oy + y), (uint64_t)(oz + z)));
                        }
                }
                frags[k] = duplicate_and_shuffle(vox, mix3(seed, ch.morton_index, 0xBA7, 3), 4);
            }
        });
    }
    for (auto& th : pool) th.join();
    uint64_t sum = 0;
    for (auto& f : frags) sum += f.size();
    *codes = (uint64_t*)std::malloc(std::max<uint64_t>(1, sum) * 8);
    *counts = (uint64_t*)std::malloc(K * 8);
    *chunk_morton = (uint64_t*)std::malloc(K * 8);
    if (!*codes || !*counts || !*chunk_morton) return 2;
    uint64_t at = 0;
    for (uint64_t k = 0; k < K; ++k) {
        if (!frags[k].empty()) std::memcpy(*codes + at, frags[k].data(), frags[k].size() * 8);
        at += frags[k].size();
        (*counts)[k] = frags[k].size();
        (*chunk_morton)[k] = chunks[k].morton_index;
    }
    *total = sum;
    *num_chunks = K;
    return 0;
}

}  // extern "C"
