/*
 * hydrant_gb300.h -- C ABI of the GB300 (sm_103a) ray-marching path.
 *
 * This is the drop-in boundary for Hydrant's CUDA shading backend.  In the
 * reference a renderer reaches the GPU through
 *   ShaderRegistrar::cuda<K>()  (include/hydrant/core/shader.hpp:319-345)
 * which installs ShaderMeta.devices[Cuda] = std::function<ShadingResult(void*)>
 * taking CudaShadingArgs{launch_info, BasicKernelArgs*, IShaderTypeErased*}
 * (shader.hpp:202-276), called per pass from Raycaster::*_pass
 * (include/hydrant/core/raycaster.hpp:32-123).  The entry points below take
 * the same information as plain pointers and sizes: the shader parameters
 * (the shader struct the reference copies into __constant__ memory), the view
 * (ViewArgs, shader.hpp:63-68), the film / destination images (ImageDesc,
 * shader.hpp:70-83) and the pass (ShadingPass, shader.hpp:55-61).
 *
 * Conventions
 *  - Every call returns an int status: HY_OK (0) or a negative HY_ERR_*.
 *    hy_last_error() gives a message for the last failure on a context.
 *    No exception crosses this boundary.
 *  - Buffers are caller-owned.  *_device entry points take device pointers and
 *    are asynchronous on the context's stream; the others take host pointers
 *    and return after the result is on the host.
 *  - One stream per context; a context is not thread-safe (the reference
 *    serialises renderers with cufx::Device::Lock, basic_renderer.hpp:89-92).
 *  - Coordinates follow the reference: object space is measured in bricks,
 *    the volume's bounding box is [0, raw/block_size] (basic_renderer.hpp:104-118).
 */
#ifndef HYDRANT_GB300_H
#define HYDRANT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HY_OK 0
#define HY_ERR_INVALID (-1)     /* bad argument or size */
#define HY_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define HY_ERR_OOM (-3)         /* device or pinned allocation failed */
#define HY_ERR_TIMEOUT (-4)     /* a bounded device-side wait gave up */
#define HY_ERR_UNSUPPORTED (-5) /* combination not built */
#define HY_ERR_STATE (-6)       /* object not ready (e.g. no transfer function) */

/* Shaders: the REGISTER_SHADER_BUILDER registrations on the path
 * (volume_shader.cu:84-88, blocks_shader.cu:53-57, isosurface_shader.cu:128-132,
 * paging_shader.cu:63-68).  Paging is the paging debug view: a constant
 * colour per brick, green for resident fine bricks, red for coarse ones
 * (registry ids below lowest_blkcnt); it has no modes and no compositing. */
enum { HY_SHADER_VOLUME = 0, HY_SHADER_BLOCKS = 1, HY_SHADER_ISOSURFACE = 2, HY_SHADER_PAGING = 3 };
/* VolumeRenderMode (ui/volume.schema.hpp:11-14) */
enum { HY_VOLUME_DEFAULT = 0, HY_VOLUME_PARTITION = 1, HY_VOLUME_PAGING = 2 };
/* BlocksRenderMode (ui/blocks.schema.hpp:10-11) */
enum { HY_BLOCKS_VOLUME = 0, HY_BLOCKS_SOLID = 1 };
/* IsosurfaceRenderMode (ui/isosurface.schema.hpp:10-11) */
enum { HY_ISO_COLOR = 0, HY_ISO_NORMAL = 1, HY_ISO_POSITION = 2 };
/* ShadingPass (shader.hpp:55-61) */
enum { HY_PASS_RAY_EMIT = 0, HY_PASS_RAY_MARCH = 1, HY_PASS_PIXEL = 2, HY_PASS_FETCH = 3 };
/* voxel types: u8 is read as clamp(u/255,0,1) (texture_3d.hpp:78-86), f32 raw */
enum { HY_DTYPE_U8 = 0, HY_DTYPE_F32 = 1 };

typedef struct hy_ctx hy_ctx;
typedef struct hy_volume hy_volume;

/* ViewArgs (shader.hpp:63-68): trans = iet * inverse(lookAt) (column-major,
 * camera -> object space), ctg_fovy_2 = 1/tan(fovy/2), ray_o = iet * eye. */
typedef struct hy_view {
    float trans[16];
    float ctg_fovy_2;
    float ray_o[3];
} hy_view;

/* Camera (include/hydrant/core/scene.hpp:32-82), world space. */
typedef struct hy_camera {
    float position[3];
    float target[3];
    float up[3];
    float ctg_fovy_2;
} hy_camera;

/* The shader struct of each registered shader, flattened.  Fields a shader
 * does not read are ignored.  step/du/bbox/max_steps of IShaderTypeErased
 * (shader.hpp:16-22) are derived from the volume and sample_rate/max_steps
 * exactly as BasicRenderer::init/update do (basic_renderer.hpp:104-131). */
typedef struct hy_shader_params {
    int32_t shader;          /* HY_SHADER_* */
    int32_t mode;            /* the shader's render mode */
    float sample_rate;       /* step = du / 4 / sample_rate */
    int32_t max_steps;
    float density;           /* Blocks: density*mean; Volume: opacity scale (1 = reference) */
    float isovalue;          /* Isosurface, normalised */
    float surface_color[3];  /* Isosurface */
    float clear_color[3];    /* written where v.a == 0 (pixel_template.hpp:11-20) */
    float rank;              /* Volume Partition tint, rank/(size-1) */
    int32_t lowest_blkcnt;   /* Volume Paging tint: registry ids below are coarse bricks */
    float to_world[16];      /* Isosurface: inverse(exhibit.get_iet()) */
    float eye_pos[3];        /* Isosurface: camera position (world) */
    float light_pos[3];      /* Isosurface: pos+target+up+cross(target,up) */
    int32_t composite;       /* 0: one march through the volume box (offline path);
                                1: per-brick segments composited front to back
                                   (sort-last operator of volume.cc:267-280 /
                                   isosurface.cc:272-290) */
    int32_t srgb;            /* Volume: linear_to_srgb before quantising (volume.cc:282-292) */
    int32_t count_samples;   /* 1: count trilinear brick samples into hy_render_stats */
    float early_termination; /* Volume, Default mode, no compositing: 0 = off (the
                                reference: every ray marches to its exit).  t in
                                (0, 1]: a warp stops marching once v.a >= t on all
                                of its rays (one vote per step).  What the skipped
                                samples would add is at most 1 - t per channel:
                                t = 1 - 2^-16 keeps images within 1 LSB and 1e-4
                                of the full march. */
} hy_shader_params;

/* Film pixel layouts of the reference (shader.hpp:26-34, pixel_template.hpp:11-20,
 * volume_shader.hpp:11-22, isosurface_shader.hpp:11-21).  The pass-level entry
 * point reads and writes films in exactly these layouts. */
typedef struct hy_ray_pixel {
    float o[3];
    float d[3];
    int32_t nsteps;
    int32_t step_size;
} hy_ray_pixel; /* IPixel, 32 B */

typedef struct hy_std_pixel {
    hy_ray_pixel ray;
    float v[4];
} hy_std_pixel; /* StdVec4Pixel (Blocks film), 48 B */

typedef struct hy_volume_pixel {
    hy_ray_pixel ray;
    float v[4];
    float theta[3];
    float phi;
} hy_volume_pixel; /* VolumePixel, 64 B */

typedef struct hy_iso_pixel {
    hy_ray_pixel ray;
    float v[4];
    float origin[3];
    float depth;
} hy_iso_pixel; /* IsosurfacePixel, 64 B */

typedef struct hy_volume_fetch_pixel {
    float theta[3];
    float phi;
    float val[4];
} hy_volume_fetch_pixel; /* VolumeFetchPixel, 32 B */

typedef struct hy_iso_fetch_pixel {
    uint8_t val[3];
    uint8_t pad_;
    float depth;
} hy_iso_fetch_pixel; /* IsosurfaceFetchPixel, 8 B */

typedef struct hy_paging_fetch_pixel {
    uint8_t val[3];
} hy_paging_fetch_pixel; /* PagingFetchPixel (paging_shader.hpp:11-14), 3 B */

/* Dataset meta the renderers read (basic_renderer.hpp:104-118,
 * lossless_block_paging.cc:17-22): raw dims, block size, apron. */
typedef struct hy_volume_desc {
    int32_t dim[3];
    int32_t block_size;
    int32_t padding;
    int32_t dtype; /* HY_DTYPE_* */
} hy_volume_desc;

typedef struct hy_volume_info {
    int32_t grid[3];        /* bricks per axis = ceil(dim/block_size) */
    int32_t nbricks;
    int32_t nonempty;       /* bricks with any non-zero voxel in core + apron */
    int32_t resident;       /* bricks with a device slot */
    int32_t padded;         /* block_size + 2*padding */
    int64_t slot_bytes;     /* bytes between slots in the brick pool */
    int64_t pool_bytes;
    float bbox_max[3];      /* raw / block_size */
} hy_volume_info;

typedef struct hy_render_stats {
    int64_t samples;        /* trilinear brick samples of the last render (count_samples=1) */
    int64_t pixels;
    float ms;               /* device time of the last render's kernels */
} hy_render_stats;

/* ---- context ----------------------------------------------------------------
 * One CUDA device and its stream: the cufx::Device a BasicRenderer selects by
 * comm_rank and holds a lock on while it renders (basic_renderer.hpp:43-52,
 * 87-92, 170-176).  Errors are status codes; hy_last_error has the message. */
int hy_ctx_create(int device, hy_ctx **out);
int hy_ctx_destroy(hy_ctx *ctx);
const char *hy_last_error(const hy_ctx *ctx);
int hy_ctx_synchronize(hy_ctx *ctx);
/* The context's cudaStream_t, for callers that order their own work with it. */
void *hy_ctx_stream(hy_ctx *ctx);
int hy_render_stats_get(hy_ctx *ctx, hy_render_stats *out);

/* Transfer function: n RGBA knots, float, flattened (transfer_fn.schema.hpp:12,
 * transfer_fn.hpp:16-23: Border, Linear, normalised coordinates). */
int hy_tf_set(hy_ctx *ctx, const float *rgba, int32_t n);

/* ---- volume (brick pool, page table, thumbnails) ----------------------------
 * The bricks, the vaddr page table and the chebyshev / mean thumbnails a
 * renderer builds from its dataset (basic_renderer.hpp:140-168,
 * block_paging.hpp:38-44). */
int hy_volume_create(hy_ctx *ctx, const hy_volume_desc *desc, hy_volume **out);
int hy_volume_destroy(hy_volume *vol);
/* Upload a whole raw volume (x fastest) from host memory; bricks it on the
 * device with a replicate-edge apron, builds the chebyshev and mean
 * thumbnails and makes every non-empty brick resident.  Replaces the
 * decode + Texture3D::source upload of LosslessBlockPagingServer (
 * src/slave/paging/lossless_block_paging.cc:137-174) for resident volumes.
 * Once per volume (HY_ERR_STATE after that): new data is a new volume. */
int hy_volume_upload(hy_volume *vol, const void *host_voxels);
int hy_volume_get_info(const hy_volume *vol, hy_volume_info *out);
/* Sampler of the Volume march in Default mode without compositing or aux
 * output (hy_render*, hy_batch_*, hy_render_views_noalloc) over a resident
 * u8 volume with an apron: the eight taps of a trilinear sample fetched by
 * two texture gathers (on, the default) or by eight loads from the brick
 * pool (off).  A batch takes the setting when it is created.  Both give the same floats: the upload places every brick in a gather texture whose
 * texels the texture unit returns as u / 255, checked bit for bit against
 * IEEE division once per device (a device that fails uses the loads).  The
 * reference samples its bricks through textures as well (texture_3d.hpp:
 * 78-86), there with hardware filtering; here the lerps stay in FP32 as the
 * CPU backend computes them.  hy_volume_gather_sampling reports whether the
 * gathers are in use (on, and the volume has gather textures). */
int hy_volume_set_gather_sampling(hy_volume *vol, int32_t enable);
int hy_volume_gather_sampling(const hy_volume *vol, int32_t *active);
/* Copy the per-brick thumbnails to the host (grid x fastest). */
int hy_volume_thumbnails(const hy_volume *vol, int32_t *chebyshev, float *mean);

/* ---- camera helpers (scene.hpp:20-81, raycaster.hpp:249-258) ----------------- */
/* Orbit camera: arm = (azimuth deg about y, elevation deg about z, distance). */
int hy_camera_orbit(const float arm[3], const float center[3], float fovy_deg, hy_camera *out);
int hy_camera_ptu(const float position[3], const float target[3], const float up[3],
                  float fovy_deg, hy_camera *out);
int hy_camera_view(const hy_volume *vol, const hy_camera *cam, hy_view *out);
/* Fill to_world / eye_pos / light_pos as IsosurfaceRenderer does (isosurface.cc:108-113). */
int hy_iso_lighting(const hy_volume *vol, const hy_camera *cam, hy_shader_params *inout);

/* ---- rendering --------------------------------------------------------------
 * A renderer's offline_render_ctxed for one view (basic_renderer.hpp:87-98;
 * volume.cc:95-134): Raycaster's emit and pixel passes (raycaster.hpp:32-123)
 * fused into one launch with no film in memory. */
/* Fused emit + march + pixel for one view: rgba8 out (RGB by the reference's
 * write_to rule, A = trunc(clamp(v.a,0,1)*255)); optional float outputs:
 * v_out (W*H*4, pre-quantisation v), aux_out (W*H*4: Volume theta.xyz,phi;
 * Isosurface depth in .x).  Host pointers; returns when results are on the host. */
int hy_render(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *params,
              const hy_view *view, int32_t width, int32_t height,
              uint8_t *rgba_out, float *v_out, float *aux_out);
/* Same with device pointers, asynchronous on the context's stream. */
int hy_render_device(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *params,
                     const hy_view *view, int32_t width, int32_t height,
                     uint8_t *rgba_dev, float *v_dev, float *aux_dev);

/* One shading pass over a device film in the reference's pixel layout --
 * the body of ShaderMeta.devices[Cuda] (shader.hpp:319-345).
 *   RAY_EMIT : view -> film (hy_*_pixel)           (cuda_shading.cu:14-35)
 *   RAY_MARCH: film -> film, resumes every pixel    (cuda_shading.cu:41-54)
 *   PIXEL    : film -> dst uchar3 (RGB8)            (cuda_shading.cu:60-74)
 *   FETCH    : film -> dst fetch pixels             (cuda_shading.cu:80-94)
 * Asynchronous on the context's stream. */
int hy_shade_pass(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *params,
                  int32_t pass, const hy_view *view, void *film_dev, int32_t width,
                  int32_t height, void *dst_dev, const uint8_t clear_rgb[3]);

/* ---- out-of-core volumes: brick store, culling, pager ------------------------
 * A store keeps every non-empty padded brick of a dataset in pinned host
 * memory mapped into the device's address space (the decoded form of the
 * varch archive the reference streams from, lossless_block_paging.cc:
 * 149-167).  A pager owns a paged volume whose brick pool is a fixed cache of
 * `slots` device slots and keeps it filled from the store, with one of the
 * reference's two policies; a gather kernel reads each batch's or frame's
 * bricks straight from the mapped store into their slots. */
typedef struct hy_store hy_store;
typedef struct hy_pager hy_pager;

enum { HY_PAGER_LOSSLESS = 0, HY_PAGER_REALTIME = 1 };
/* Realtime eviction: which slot a missing brick takes once no slot is free
 * (only slots of bricks the frame does not require are candidates).
 * LRU: the brick visible least recently (a brick counts as used in every
 * frame in which the cull finds it visible); REFERENCE: the highest brick
 * index, as RtBlockPagingServer pops its redundant set (rt_block_paging.cc:
 * 256-265, 299-326). */
enum { HY_EVICT_LRU = 0, HY_EVICT_REFERENCE = 1 };
/* Where a realtime cache keeps its bricks: a device pool read by loads (every
 * shader), or gather textures (u8 stores with an apron; the Volume shader in
 * Default mode without compositing or aux output samples them by texture
 * gathers, Blocks and Paging read no voxels; other uses of the pager's volume
 * return HY_ERR_UNSUPPORTED).  Same images and the same bytes per brick. */
enum { HY_PAGER_LOADS = 0, HY_PAGER_GATHERS = 1 };

typedef struct hy_pager_desc {
    int32_t slots;                 /* bricks per batch (lossless) / cache size (realtime) */
    int32_t mode;                  /* HY_PAGER_* */
    int32_t max_uploads_per_frame; /* realtime: 0 = every missing brick */
    int32_t eviction;              /* realtime: HY_EVICT_* */
    int32_t sampler;               /* realtime: HY_PAGER_LOADS / HY_PAGER_GATHERS */
} hy_pager_desc;

typedef struct hy_pager_stats {
    int64_t frames, passes, uploads, upload_bytes, hits, misses, evictions, visible;
    int64_t fallback;  /* realtime + coarse level: visible bricks drawn coarse, last frame */
    int64_t prefetched; /* realtime: bricks moved by hy_pager_prefetch */
} hy_pager_stats;

/* Store of a resident volume's bricks (copies its pool to pinned host memory). */
int hy_store_from_volume(const hy_volume *vol, hy_store **out);
/* Store of a procedural u8 volume: 3 octaves of lattice value noise (cell,
 * cell/2, cell/4 voxels; amplitudes 1, 1/2, 1/4), thresholded so that
 * `occupancy` of the voxels are non-zero, those rescaled to 1..255; generated
 * on the device brick by brick. */
int hy_store_create_noise(hy_ctx *ctx, const hy_volume_desc *desc, uint64_t seed,
                          float cell_voxels, float occupancy, hy_store **out);
int hy_store_destroy(hy_store *store);
int hy_store_get_info(const hy_store *store, hy_volume_info *out);
int hy_store_thumbnails(const hy_store *store, int32_t *chebyshev, float *mean);
/* Copy one padded brick (P^3 voxels; zeros for an empty brick). */
int hy_store_brick(const hy_store *store, int32_t brick, void *out);
/* Coarse level of the store: the lowest sample level RtBlockPagingServer
 * keeps resident (rt_block_paging.cc:119-196).  The volume box-filtered by
 * s = 2^level per axis (a coarse voxel is the mean of the fine voxels of its
 * s^3 cube that lie inside the volume; u8 rounds half up), bricked with the
 * same block size and apron as the fine level, so one coarse brick covers
 * s^3 fine bricks.  block_size must be a multiple of s.  Replaces an earlier
 * coarse level. */
int hy_store_build_coarse(hy_store *store, int32_t level);
/* Coarse brick grid ({0,0,0} without a coarse level) and one coarse brick. */
int hy_store_coarse_grid(const hy_store *store, int32_t grid[3]);
int hy_store_coarse_brick(const hy_store *store, int32_t brick, void *out);

/* On-disk dataset (replaces the varch archive set of build_dataset.sh:77-126
 * that RendererFactory reads, renderer.hpp:53-59): a directory holding
 * package_meta.json ("sample_levels" with the level-0 bricks, chebyshev and
 * mean thumbnails, and the coarse level if built) and uncompressed bricks.
 * hy_store_save writes one (creating the directory), hy_store_open reads it
 * into a pinned store. */
int hy_store_save(const hy_store *store, const char *dir);
int hy_store_open(hy_ctx *ctx, const char *dir, hy_store **out);
/* Ingest a raw volume file (x fastest, desc->dtype, exactly dim product
 * voxels) on the host: bricks with a border-clamped apron, emptiness,
 * chebyshev and mean thumbnails as for hy_volume_upload, in slabs of
 * block_size (+ apron) z-slices, so the volume never has to fit on the
 * device. */
int hy_store_ingest_raw(hy_ctx *ctx, const char *raw_path, const hy_volume_desc *desc,
                        hy_store **out);

/* OctreeCuller::cull (octree_culler.hpp:121-161) on the device: non-empty
 * bricks whose box meets the frustum, the nearest `limit` (< 0: all) by
 * squared distance of the brick centre to the eye (ties by index), returned in
 * index order.  rect = {min.x, min.y, max.x, max.y} (NULL: [-1,1]^2).
 * ids / dist2 must hold nbricks entries. */
int hy_cull(const hy_volume *vol, const hy_view *view, const float rect[4], int32_t limit,
            int32_t *ids_out, float *dist2_out, int32_t *n_out);

/* The store must outlive the pager (the pager's kernels read the store's
 * pinned memory); hy_pager_destroy waits for the pager's queued work.  A
 * coarse level must be built before the pager is created. */
int hy_pager_create(hy_ctx *ctx, hy_store *store, const hy_pager_desc *desc, hy_pager **out);
int hy_pager_destroy(hy_pager *pager);
/* Realtime cache size for a camera path: slots for the most visible bricks
 * any of `cams` sees plus 10 % (new bricks come into view between frames),
 * at most budget_bytes / slot bytes and the store's non-empty bricks; the
 * most visible bricks are returned too.  The reference derives its cache
 * from mem_limit_mb alone (rt_block_paging.cc:230-236); this sizes it to
 * the path, within the same kind of limit. */
int hy_pager_tune_slots(hy_ctx *ctx, const hy_store *store, const hy_camera *cams, int32_t ncams,
                        int64_t budget_bytes, int32_t *slots, int32_t *visible_max);
/* The paged volume (for hy_cull / hy_render); owned by the pager. */
int hy_pager_volume(hy_pager *pager, hy_volume **out);
int hy_pager_stats_get(const hy_pager *pager, hy_pager_stats *out);
/* Bricks resident after the last frame, one byte per brick. */
int hy_pager_present(const hy_pager *pager, uint8_t *mask);
/* One frame into a device RGBA8 image.  The pager sets params->lowest_blkcnt
 * itself (the Paging mode's coarse / fine split).
 *  LOSSLESS: LosslessBlockPagingServer::start/next (lossless_block_paging.cc:
 *    116-174) + Volume/Isosurface/Blocks passes: visible bricks ordered by the
 *    distance of their centres to inverse(iet) * eye (as the reference
 *    computes it), uploaded in batches of `slots`; the first batch's pass
 *    emits, later ones resume (ray_march); only the current batch is in the
 *    page table.  Uploads of batch k+1 overlap the march of batch k.  With
 *    count_samples the frame's samples over all its passes are counted.
 *  REALTIME: RtBlockPagingServer::update (rt_block_paging.cc:296-326): the
 *    nearest `slots` visible bricks are required; missing ones, nearest first,
 *    go to never-used slots and then to slots of bricks no longer required
 *    (desc.eviction: least recently visible, or highest index first as in the
 *    reference); one emit pass renders with what is resident.
 *    With a coarse level in the store (created before the pager), the coarse
 *    bricks stay resident and registry ids 0..nbricks-1 sample them, brick b
 *    through its sub-box of the coarse brick (k = bs/P/s, b = pad/P + d*k,
 *    rt_block_paging.cc:141-188); an absent brick's page entry is that id
 *    instead of -1, so rays read the coarse level rather than stop, and cache
 *    slot i is registry id nbricks + i (lowest_blkcnt = nbricks). */
int hy_pager_render(hy_pager *pager, const hy_shader_params *params, const hy_camera *cam,
                    int32_t width, int32_t height, uint8_t *rgba_dev);
/* REALTIME: start moving the bricks `next_cam` will require (nearest first,
 * within max_uploads_per_frame) while the frame just rendered is still
 * drawing: the moves run on the pager's copy stream, and the next
 * hy_pager_render takes the arrived bricks into its page table (its render
 * waits for their copies).  A frame loop that knows its next camera (a
 * camera path, or one extrapolated from the last two) calls this after each
 * hy_pager_render.  The moves may only use slots that no frame in flight can
 * read: never-used slots, or spares -- once prefetching, each frame evicts
 * (by the pager's policy, among the bricks it does not require) as many
 * bricks as it brought in and keeps those slots out of its page table for
 * the next prefetch.  The reference decodes arriving bricks on a worker
 * thread beside the render (unarchive_pipeline.cc:12-23). */
int hy_pager_prefetch(hy_pager *pager, const hy_camera *next_cam);
/* Same into a host image; returns when it is there. */
int hy_pager_render_host(hy_pager *pager, const hy_shader_params *params, const hy_camera *cam,
                         int32_t width, int32_t height, uint8_t *rgba_host);

/* ---- differentiable rendering (transfer function and voxel gradients) -------
 * No counterpart in the reference (its shaders have no derivatives).  The
 * forward is the Volume shader's march (volume_shader.cu:32-81) over one
 * dense f32 brick of n^3 voxels with a 1-voxel replicate apron, with step_size
 * held at 1 and no empty-space skipping (the two discontinuous parts); it
 * stores the ray state every ckpt_k steps.  The backward recomputes each
 * K-step segment from its checkpoint and back-propagates through compositing,
 * the transfer function and the trilinear weights, accumulating into
 * caller-zeroed gradient buffers.  All pointers are device pointers; views is
 * a host array; both calls are asynchronous on the context's stream. */
typedef struct hy_diff_params {
    int32_t n;            /* volume edge (voxels); bbox = [0,1]^3 */
    float sample_rate;    /* step = (1/n) / 4 / sample_rate */
    int32_t max_steps;
    float density;        /* opacity scale of the TF alpha */
    int32_t ntf;          /* knots (<= 256) */
    int32_t ckpt_k;       /* checkpoint interval, 1..64 */
} hy_diff_params;

/* Bytes of the checkpoint buffer for W x H x nviews rays. */
int hy_diff_ckpt_bytes(const hy_diff_params *p, int32_t width, int32_t height, int32_t nviews,
                       int64_t *bytes);
/* image: nviews*H*W RGBA floats.  ckpt / nsteps may both be NULL (no backward). */
int hy_diff_forward(hy_ctx *ctx, const hy_diff_params *p, const float *volume, const float *tf,
                    const hy_view *views, int32_t nviews, int32_t width, int32_t height,
                    float *image, float *ckpt, int32_t *nsteps);
/* dL/dimage in, dL/dvolume (n^3) and dL/dtf (ntf*4) accumulated. */
int hy_diff_backward(hy_ctx *ctx, const hy_diff_params *p, const float *volume, const float *tf,
                     const hy_view *views, int32_t nviews, int32_t width, int32_t height,
                     const float *dimage, const float *ckpt, const int32_t *nsteps,
                     float *dvolume, float *dtf);

/* ---- batched multi-view rendering -------------------------------------------
 * Many views rendered by one persistent launch replayed from a CUDA graph.
 * The reference renders one view per Raycaster pass (raycaster.hpp:32-54,
 * called per frame from BasicRenderer::offline_render, basic_renderer.hpp:
 * 134-142); a batch gives images identical to hy_render per view. */
typedef struct hy_batch hy_batch;

typedef struct hy_batch_view {
    hy_view view;          /* ViewArgs of this camera */
    int32_t width;
    int32_t height;
    int64_t rgba_offset;   /* byte offset of this view's RGBA8 image in the output (4-aligned) */
    float eye_pos[3];      /* Isosurface lighting of this camera (see hy_iso_lighting) */
    float light_pos[3];
} hy_batch_view;

typedef struct hy_batch_config {
    int32_t tile_w;        /* warp ray tile width: 4, 8, 16 or 32 (height 32/tile_w) */
    int32_t grab;          /* warp tiles taken per queue access, 1..16 */
    int32_t block_warps;   /* warps per block, 1..8 */
    int32_t blocks_per_sm; /* persistent blocks per SM; 0 = as many as fit */
    int32_t block_queue;   /* 0: each warp takes warp tiles; 1: each block takes a block
                              tile and its warps shade neighbouring warp tiles */
    int32_t steps_per_iter; /* lean Volume march: samples per loop iteration, 1 or 2
                               (0 = 1); the same samples either way */
} hy_batch_config;

/* The batch keeps `vol`, which must outlive it; every render uses the
 * context's transfer function as set at that time (hy_tf_set). */
int hy_batch_create(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *params,
                    const hy_batch_view *views, int32_t nviews, hy_batch **out);
int hy_batch_destroy(hy_batch *batch);
/* Bytes the output buffer must hold (max over views of offset + W*H*4). */
int hy_batch_output_bytes(const hy_batch *batch, int64_t *bytes);
int hy_batch_set_config(hy_batch *batch, const hy_batch_config *cfg);
int hy_batch_get_config(const hy_batch *batch, hy_batch_config *out);
/* 1: count brick samples of each launch into hy_render_stats. */
int hy_batch_set_counting(hy_batch *batch, int32_t count_samples);
/* New cameras for the following renders, as a frame loop supplies them (the
 * reference builds ViewArgs from the camera for every frame,
 * raycaster.hpp:126-135): `views` must keep the batch's number of views and
 * each view's size and output offset; ViewArgs and lighting may change.  The
 * captured graph is kept: the descriptors are copied to the device on the
 * context's stream (hy_batch_view_bytes bytes), ordered before the next
 * render.  Returns without waiting for the copy; `views` may be reused at once. */
int hy_batch_update_views(hy_batch *batch, const hy_batch_view *views, int32_t nviews);
int hy_batch_view_bytes(const hy_batch *batch, int64_t *bytes);
/* Device output, asynchronous on the context's stream. */
int hy_batch_render_device(hy_batch *batch, uint8_t *rgba_dev);
/* Host output; returns when the images are on the host.  rgba_host must
 * hold hy_batch_output_bytes bytes (as a cudaMemcpy destination must: a
 * short pinned buffer would be overrun by the device).  A pinned host
 * buffer mapped into the device's address space (cudaHostAlloc, or
 * cudaHostRegister with mapping) is written by the kernel itself, with no
 * staging copy; any other buffer receives one copy from device memory. */
int hy_batch_render(hy_batch *batch, uint8_t *rgba_host);
/* Times every launch shape (queue per warp or per block, tile 8x4/4x8/16x2,
 * grab 1/2/4, 2/4/8 warps per block), then 1 or 2 march steps per loop
 * iteration on the fastest shape, on this batch and keeps the fastest;
 * it is returned in *best.  For the Isosurface shader, params->to_world must
 * be set (hy_iso_lighting) when the batch is created. */
int hy_batch_autotune(hy_batch *batch, uint8_t *rgba_dev, int32_t reps, hy_batch_config *best);

/* Renders up to 256 views into rgba_dev like hy_batch_render_device (default
 * launch shape, same images), allocating nothing.  No counterpart in the
 * reference.  For callers that may not allocate device memory while they
 * render -- a host application that owns the GPU memory budget and only
 * lends its inputs and outputs, or a frame loop that cannot take the
 * synchronisation cost of cudaMalloc/cudaFree mid-frame.  Scratch lives in a
 * fixed ~33 KiB static device array that every GPU loading the library keeps
 * until exit.  The view descriptors are copied from host stack memory, so a
 * call on a stream that is capturing returns HY_ERR_STATE (capture the batch
 * path, hy_batch_*, instead).  Calls share that array: calls that overlap
 * on the GPU race.  More than 256 views is rejected with HY_ERR_INVALID.
 * rgba_dev must hold at least max over views of rgba_offset + width*height*4
 * bytes (there is no size argument to check it against).
 * Asynchronous on the context's stream; count_samples is ignored. */
int hy_render_views_noalloc(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *params,
                            const hy_batch_view *views, int32_t nviews, uint8_t *rgba_dev);

#ifdef __cplusplus
}
#endif

#endif /* HYDRANT_GB300_H */
