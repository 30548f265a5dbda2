/* Seeded synthetic voxel-fragment generators (host only).
 *
 * They stand in for the reference's OpenGL voxelizer
 * (src/Voxelizer.h:32 FVoxelizer::GenerateFragments), which needs a graphics
 * stack: each call returns a malloc'd array of shuffled uint64 Morton codes with
 * duplicates (x at bit 2, y at bit 1, z at bit 0 of every 3-bit group, as
 * mortonEncode64 in src/DAG_Compression_Fast.cpp:223-236). Free the arrays with
 * dagc_gen_free. Results are identical on every host and thread count.
 * Return value: 0 on success, 1 for bad arguments, 2 when out of host memory. */
#ifndef DAGC_GEN_H
#define DAGC_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

void dagc_gen_free(void* p);

/* Sphere shell in a 2^depth grid: radius 0.4375 * 2^depth +/- U(0,2) (or sized
 * for about target_fragments when > 0), centre jittered by U(-2,2) per axis,
 * voxel kept iff | |p + 0.5 - c| - R | <= 0.5, each voxel emitted U{1..4}
 * times. */
int dagc_gen_sphere_shell(int depth, uint64_t seed, double target_fragments, uint64_t** out,
                          uint64_t* n);

/* Heightfield terrain in a 2^depth grid: 4-octave fBm value noise (lacunarity
 * 2, gain 0.5, seeded hash lattice, smoothstep interpolation, base period
 * 2^depth / 4) sets h in [G/4, 3G/4); voxels y in [h-2, h] of a seeded
 * column_fraction of the columns, each emitted U{1..4} times. */
int dagc_gen_terrain(int depth, uint64_t seed, double column_fraction, uint64_t** out, uint64_t* n);

/* The triangles of dagc_gen_triangle_soup (same depth, seed and count), in
 * grid units: 9 doubles per triangle (v0, v1, v2). */
int dagc_gen_soup_triangles(int depth, uint64_t seed, uint64_t num_triangles, double* vertices);

/* Random triangle soup in a 2^depth grid: vertex v0 uniform, two edges of
 * log-uniform length in [1, 16] voxels and uniform direction, conservatively
 * surface-voxelized by a triangle/box separating-axis test. */
int dagc_gen_triangle_soup(int depth, uint64_t seed, uint64_t num_triangles, int threads,
                           uint64_t** out, uint64_t* n);

/* Batched chunks: grid_xz^2 chunks of 2^chunk_depth voxels per side at chunk
 * row chunk_row, cut from one fBm terrain with a level-5 Menger sponge in
 * every 8th chunk; per-chunk fragment counts follow log-uniform targets in
 * [min_fragments, max_fragments]. Outputs chunk-local codes concatenated in
 * ascending chunk Morton order, per-chunk counts and chunk Morton indices
 * (4 bits per axis for a 16^3 chunk grid). */
int dagc_gen_batched(int chunk_depth, int grid_xz, int chunk_row, uint64_t seed,
                     double min_fragments, double max_fragments, int threads,
                     uint64_t** codes, uint64_t* total, uint64_t** counts,
                     uint64_t** chunk_morton, uint64_t* num_chunks);

#ifdef __cplusplus
}
#endif

#endif
