/*
 * hydrant_gb300_synth.h -- seeded synthetic volumes for the benchmark and
 * test workloads.
 *
 * The reference reads bricked datasets built by external varch tools
 * (build_dataset.sh:77-126); none of those datasets is available, so the
 * workloads use seeded procedural volumes with the shapes and value
 * distributions below.  All generators are deterministic functions of
 * (seed, dims, count): the same bytes on every machine and thread count.
 * Random draws come from splitmix64; arithmetic is double precision.
 */
#ifndef HYDRANT_GB300_SYNTH_H
#define HYDRANT_GB300_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* u8 = clamp(round(sum_b peak_b * exp(-|x - c_b|^2 / (2 sigma_b^2))), 0, 255)
 * with x at voxel centres ((i+0.5)/n per axis, fractions of the extent),
 * c ~ U[0.2,0.8]^3, sigma ~ U[0.03,0.12], peak ~ U[40,255]; draws per blob in
 * the order cx, cy, cz, sigma, peak. */
int hy_synth_blobs_u8(uint64_t seed, const int32_t dim[3], int32_t nblobs, uint8_t *out,
                      int32_t nthreads);

/* f32 density in [0,1]: min(1, sum_b w_b * exp(...)), same centre and sigma
 * draws, weight w ~ U[0.15, 0.6]. */
int hy_synth_blobs_f32(uint64_t seed, const int32_t dim[3], int32_t nblobs, float *out,
                       int32_t nthreads);

/* u8 tubes: background ~ U{0..30} per voxel; ntubes cubic Bezier curves with
 * control points ~ U[0.05,0.95]^3 and radius ~ U[2,10] voxels; a voxel inside
 * any tube holds clamp(round(N(200, 20))).  Per-voxel draws are hashes of
 * (seed, voxel index), so the result does not depend on the stamping order. */
int hy_synth_tubes_u8(uint64_t seed, const int32_t dim[3], int32_t ntubes, uint8_t *out,
                      int32_t nthreads);

#ifdef __cplusplus
}
#endif
#endif
