/*
 * hy_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of Hydrant's multi-thread CPU shading backend for the
 * ray-marching path (src/slave/core/cpu_shading.cc:9-90 driving the shared
 * __host__ __device__ shaders of src/slave/renderers/{volume,blocks,
 * isosurface}/<name>_shader.cu through CpuSampler, include/hydrant/bridge/
 * cpu_sampler.hpp:72-166).  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it, and only as the
 * checker or the timed CPU baseline; the product never links it.
 *
 * PARITY UNPINNED: the reference's path cannot be compiled here (it needs
 * glm-cuda, cuda-fx, VMUtils and varch, none vendored) and the reference
 * ships no tests or golden vectors.  This oracle is pinned instead by
 * analytic known-answer cases (tests/test_oracle_kat.py) and committed
 * fixtures it generated (tests/golden/).
 */
#ifndef HY_ORACLE_H
#define HY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_volume orc_volume;

/* Same field order and types as the product's shader parameters so one
 * ctypes structure can fill both. */
typedef struct orc_params {
    int32_t shader;
    int32_t mode;
    float sample_rate;
    int32_t max_steps;
    float density;
    float isovalue;
    float surface_color[3];
    float clear_color[3];
    float rank;
    int32_t lowest_blkcnt;
    float to_world[16];
    float eye_pos[3];
    float light_pos[3];
    int32_t composite;
    int32_t srgb;
    int32_t count_samples;
    float early_termination;  /* ignored: every ray marches to its exit */
} orc_params;

/* Bricks a raw volume (x fastest) the way the dataset is defined for this
 * path: padded bricks of (bs+2*pad)^3 with the apron read from the
 * neighbouring voxels, clamped at the volume border. */
orc_volume *orc_volume_create(const int32_t dim[3], int32_t block_size, int32_t padding,
                              int32_t dtype, const void *voxels);
void orc_volume_free(orc_volume *v);
void orc_volume_grid(const orc_volume *v, int32_t grid[3], int32_t *nonempty);
void orc_volume_thumbnails(const orc_volume *v, int32_t *chebyshev, float *mean);
/* Mark bricks absent (page table -1) or present again; for paging tests. */
void orc_volume_set_present(orc_volume *v, const uint8_t *present_mask);
/* Normalised float contents of one padded brick (P^3 floats). */
void orc_volume_brick(const orc_volume *v, int32_t brick, float *out);
/* Coarse (lowest) sample level for the realtime paging fallback; afterwards
 * absent bricks sample it and fine bricks are registry ids >= lowest_blkcnt.
 * Returns 0, or -1 when block_size is not a multiple of 2^level. */
int orc_volume_build_coarse(orc_volume *v, int32_t level);
int32_t orc_volume_lowest_blkcnt(const orc_volume *v);
void orc_volume_coarse_brick(const orc_volume *v, int32_t brick, float *out);

/* camera: out[0..2] position, [3..5] target, [6..8] up, [9] ctg_fovy_2 */
void orc_camera_orbit(const float arm[3], const float center[3], float fovy_deg, float out[10]);
void orc_camera_ptu(const float pos[3], const float target[3], const float up[3], float fovy_deg,
                    float out[10]);
/* view: [0..15] trans (column-major), [16] ctg_fovy_2, [17..19] ray_o */
void orc_camera_view(const orc_volume *v, const float cam[10], float view[20]);
void orc_iso_lighting(const orc_volume *v, const float cam[10], orc_params *p);

/* Renders one view.  v_out: W*H*4 floats (pre-quantisation v), rgba_out:
 * W*H*4 bytes, aux_out: W*H*4 floats (Volume theta.xyz, phi; Isosurface depth
 * in .x), film_out: the final film pixel in the reference layout (64 B for
 * Volume/Isosurface, 48 B for Blocks; composite == 0 only).  Any output may
 * be NULL.  Rows are interleaved over nthreads std::threads like
 * cpu_shading.cc.  Returns the number of brick samples. */
int64_t orc_render(const orc_volume *v, const float *tf_rgba, int32_t ntf, const orc_params *p,
                   const float view[20], int32_t width, int32_t height, int32_t nthreads,
                   float *v_out, uint8_t *rgba_out, float *aux_out, void *film_out);

/* Same, but only for pixel rows y0 <= y < y1 (a bounded CPU-baseline sample). */
int64_t orc_render_rows(const orc_volume *v, const float *tf_rgba, int32_t ntf,
                        const orc_params *p, const float view[20], int32_t width,
                        int32_t height, int32_t y0, int32_t y1, int32_t nthreads,
                        float *v_out, uint8_t *rgba_out, float *aux_out, void *film_out);

/* Rows y0, y0 + ystep, ... below y1 only (v_out / rgba_out are full-image
 * buffers, written at those rows). */
int64_t orc_render_row_step(const orc_volume *v, const float *tf_rgba, int32_t ntf,
                            const orc_params *p, const float view[20], int32_t width,
                            int32_t height, int32_t y0, int32_t y1, int32_t ystep,
                            int32_t nthreads, float *v_out, uint8_t *rgba_out);

/* Seeded synthetic volumes (oracle/synth.cc): the benchmark's generators,
 * byte for byte, for the CPU side of the measurement. */
int orc_synth_blobs_u8(uint64_t seed, const int32_t dim[3], int32_t nblobs, uint8_t *out,
                       int32_t nthreads);
int orc_synth_blobs_f32(uint64_t seed, const int32_t dim[3], int32_t nblobs, float *out,
                        int32_t nthreads);
int orc_synth_tubes_u8(uint64_t seed, const int32_t dim[3], int32_t ntubes, uint8_t *out,
                       int32_t nthreads);

/* Visible non-empty bricks (OctreeCuller::cull): the nearest `limit` (< 0:
 * all) by squared distance of the brick centre to the frustum origin, ties by
 * index, returned in index order.  rect = {min.x, min.y, max.x, max.y} or NULL
 * for [-1,1]^2.  Returns the count. */
int32_t orc_cull(const orc_volume *v, const float view[20], const float rect[4], int32_t limit,
                 int32_t *ids_out, float *dist2_out);
/* LosslessBlockPagingServer::start ordering of brick ids. */
void orc_lossless_order(const orc_volume *v, const float cam[10], const int32_t *ids, int32_t n,
                        int32_t *order_out);

/* Resume a film (RAY_MARCH pass) with the current page table. */
int64_t orc_march_film(const orc_volume *v, const float *tf_rgba, int32_t ntf,
                       const orc_params *p, int32_t width, int32_t height, int32_t nthreads,
                       void *film_inout);

#ifdef __cplusplus
}
#endif
#endif
