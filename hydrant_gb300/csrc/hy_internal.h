// hy_internal.h -- shared host/device declarations of libhydrant_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/hydrant_gb300.h"

namespace hy {

// One registry entry: the BlockSampler of block_paging.hpp:24-36 (a storage
// slot plus its BlockSamplerMapping {k, b}, block_paging.hpp:11-22).
struct __align__(16) RegEntry {
    float k, bx, by, bz;   // mapped(x) = k * x + b
    long long offset;      // byte offset of the slot in the brick pool
    int pad_[2];
};
static_assert(sizeof(RegEntry) == 32, "RegEntry is two 16-byte loads");

// Where a resident u8 brick also sits in a 2-D gather texture: its P
// slices stacked as P x P tiles in one column of texels, slice z at rows
// y0 + z * P, columns x0 .. x0 + P - 1, in texture `which` (0 or 1) of the
// volume.  The texture returns a u8 texel u as the float u / 255
// (normalised read), so one gather fetches four normalised taps of the
// trilinear footprint.
struct __align__(16) TexEntry {
    float x0, y0;
    int which;
    int pad_;
};
static_assert(sizeof(TexEntry) == 16, "TexEntry is one 16-byte load");
// A volume's bricks go in at most this many gather textures; the handles
// travel in the kernel parameters, so every gather names a warp-uniform
// texture (a per-brick handle in a register would make the compiler
// serialise the gather over the distinct handles of a warp).
constexpr int kMaxGatherTextures = 16;  // a power of two
// A resident volume uses at most two of them (its march selects between two
// textures by a warp vote); a paged cache in gather textures up to all.
constexpr int kResidentGatherTextures = 2;
#ifdef __CUDACC__
// One gather of component 0 (texture unit tld4): the four texels of the
// footprint (x - 1/2 .. x + 1/2, y - 1/2 .. y + 1/2) in the order
// w = (x0, y0), z = (x1, y0), x = (x0, y1), y = (x1, y1).  The march and the
// per-device gather check both call this, so the order they rely on is the
// order checked.  Written as the PTX instruction: through tex2Dgather the
// compiler kept a march's two textures as divergent branches around their
// gathers; with the bare instruction it predicates both (64-view step
// 156.9 vs 170.1 ms).
__device__ __forceinline__ float4 gather_r(unsigned long long t, float x, float y) {
    float4 g;
    asm("tld4.r.2d.v4.f32.f32 {%0, %1, %2, %3}, [%4, {%5, %6}];"
        : "=f"(g.x), "=f"(g.y), "=f"(g.z), "=f"(g.w)
        : "l"(t), "f"(x), "f"(y));
    return g;
}
#endif

// Device view of a volume: the brick pool, the page table + chebyshev
// thumbnail packed per brick as int2 {chebyshev, registry id or -1}, the
// registry, and the mean thumbnail; `tex` (per registry id, or null) places
// each brick in a gather texture.
struct DevVolume {
    const unsigned char *pool;
    const int2 *info;
    const RegEntry *reg;
    const float *mean;
    int gx, gy, gz;
    int P;      // padded brick edge
    int dtype;  // HY_DTYPE_*
    int pad;    // apron width
    const TexEntry *tex;
    unsigned long long gtex[kMaxGatherTextures];  // cudaTextureObject_t
    float map_k, map_b;  // BlockSamplerMapping of every resident brick (with `tex`)
    // with `tex`: per brick {chebyshev, registry id or -1, x0 + 1, y0 + 1}
    // (texel column and row of the brick's origin plus one, as float bits;
    // the row negated in texture 1): the page table and the brick's place in
    // its gather texture in one 16-byte load
    const int4 *info4;
    // the thumbnail grid as floats: g - 1 per axis (the clamp bounds) and
    // gx, gy (the index strides); exact, nbricks <= 2^24
    float gmx, gmy, gmz, fgx, fgy;
    // a paged cache in gather textures (registry entries carry texel origins)
    int paged_gather;
};

// Per-view inputs: ViewArgs (shader.hpp:63-68) plus the image size and the
// camera-dependent isosurface lighting (isosurface.cc:108-113).
struct ViewArgs {
    float trans[16];
    float ctg;
    float ray_o[3];
    float eye[3];
    float light[3];
    int W, H;
};

// Everything one shading launch reads; passed as a __grid_constant__ kernel
// parameter (the reference copies its shader struct into a 16 KiB
// __constant__ buffer per launch, cuda_shading.cu:5-10).
struct ShadeArgs {
    DevVolume vol;
    // IShaderTypeErased (shader.hpp:16-22)
    float bbox_max[3];
    float step, du;
    int max_steps;
    // shader parameters
    int shader, mode;
    float density, isovalue;
    float surface[3];
    float rank;
    int lowest_blkcnt;
    float to_world[16];
    int composite, srgb, count;
    float ert;  // early ray termination opacity (lean Volume march; 0 = off)
    unsigned char clear_u8[4];
    ViewArgs view;
    const float4 *tf;
    int ntf;
    // outputs
    uchar4 *rgba;
    float4 *vout;
    float4 *aux;
    void *film;
    void *dst;
    unsigned long long *counter;
};

}  // namespace hy

struct hy_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    float4 *tf_dev = nullptr;
    int ntf = 0;
    int tf_cap = 0;
    unsigned long long *counter_dev = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    hy_render_stats stats{};
    bool stats_pending = false;   // a launch whose events/counter are not read yet
    int pend_count = 0;
    int64_t pend_pixels = 0;
    // device staging for the host-pointer entry points, grown on demand
    void *stage = nullptr;
    size_t stage_bytes = 0;
    // the differentiable path's volume as a gather texture (hy_diff.cu)
    void *diff_gather = nullptr;
};
// Frees ctx->diff_gather (hy_diff.cu).
void hy_diff_release(hy_ctx *ctx);

struct hy_volume {
    hy_ctx *ctx = nullptr;
    hy_volume_desc desc{};
    int grid[3] = {0, 0, 0};
    int nbricks = 0;
    int P = 0;
    int nonempty = 0;
    int resident = 0;
    size_t elem = 1;
    size_t slot_stride = 0;
    unsigned char *pool = nullptr;
    size_t pool_bytes = 0;
    int2 *info_dev = nullptr;
    hy::RegEntry *reg_dev = nullptr;
    float *mean_dev = nullptr;
    std::vector<int> cheb;
    std::vector<float> mean;
    std::vector<int> reg_of_brick;
    float k = 0.f, b = 0.f;   // uniform mapping of full-resolution bricks
    float bbox_max[3] = {0, 0, 0};
    float du = 0.f;
    bool uploaded = false;
    bool paged = false;       // pool is a brick cache owned by a hy_pager
    // gather textures of the resident bricks (u8 with an apron; see TexEntry)
    std::vector<cudaArray_t> atlas;
    std::vector<unsigned long long> atlas_tex;
    hy::TexEntry *tex_dev = nullptr;
    int4 *info4_dev = nullptr;
    bool tex_sampling = true;  // hy_volume_set_gather_sampling
    bool paged_gather = false;  // a pager's cache held in atlas (gather textures)
};

// Brick store: every non-empty padded brick in pinned host memory, laid out
// like device slots (slot_stride apart), plus the thumbnails.
struct hy_store {
    hy_ctx *ctx = nullptr;
    hy_volume_desc desc{};
    int grid[3] = {0, 0, 0};
    int nbricks = 0;
    int P = 0;
    size_t slot_stride = 0;
    std::vector<int> cheb;
    std::vector<float> mean;
    std::vector<long long> offset;  // brick -> byte offset in `host`, -1 if empty
    unsigned char *host = nullptr;  // pinned, mapped into the device address space
    const unsigned char *host_dev = nullptr;  // the same memory as the device sees it
    size_t host_bytes = 0;
    int nonempty = 0;
    // coarse level (0: none): every coarse brick, slot_stride apart
    int coarse_level = 0;
    int coarse_grid[3] = {0, 0, 0};
    int ncoarse = 0;
    std::vector<unsigned char> coarse;
};

int hy_volume_init(hy_ctx *ctx, const hy_volume_desc *desc, hy_volume *v);
// The gather-texture table of a volume's bricks when they have one and
// sampling through it is on, else null (hy_volume.cu).
const hy::TexEntry *hy_volume_gather_table(const hy_volume *v);
// Fills the gather fields of a device view of the volume (table and handles,
// or null and zeros).
void hy_volume_gather_view(const hy_volume *v, hy::DevVolume *dv);
// Gather textures on this device: *ok when the texture unit's gather order and
// u8 normalisation pass the check; *cols x *rowblocks bricks of edge P fit
// one texture (0 when a brick does not).
int hy_gather_layout(hy_ctx *ctx, int P, bool *ok, int *cols, int *rowblocks);
// A u8 array made for gather (width x height texels) and its texture object;
// with `surf`, also writable by kernels through the surface object *surf.
int hy_gather_texture_create(hy_ctx *ctx, size_t width, size_t height, cudaArray_t *arr,
                             unsigned long long *tex, unsigned long long *surf = nullptr);
void hy_volume_free_gather(hy_volume *v);
// HY_OK unless the arguments' volume is a pager's cache in gather textures
// and the launch would read its voxels other than by the lean Volume march
// of the fused per-view kernel (`fused`: that kernel is the launch); the
// Blocks and Paging shaders read no voxels.
int hy_check_paged_gather(hy_ctx *ctx, const hy::ShadeArgs &a, bool fused);
// store helpers (hy_page.cu): grid / padded edge / slot stride from a
// descriptor, and the pinned allocation for `nonempty` bricks
void hy_store_geometry(hy_store *s, const hy_volume_desc &d);
int hy_store_alloc(hy_store *s, int nonempty);
// Chebyshev distance over the brick grid (hy_page.cu)
void hy_chebyshev_transform(const std::vector<unsigned char> &nonempty, const int grid[3],
                            std::vector<int> &out);

// error helpers (hy_api.cc)
int hy_fail(hy_ctx *ctx, int code, const std::string &msg);
int hy_cuda_fail(hy_ctx *ctx, cudaError_t e, const char *what);
// The kernels store RGBA8 pixels as uchar4 and float images, films and
// transfer functions as float4: device buffers a caller passes must be 4- or
// 16-byte aligned, and the entry points check that before anything else.
inline bool hy_aligned(const void *p, uintptr_t a) {
    return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0;
}
// The device address of a pinned host buffer mapped into the device's
// address space (cudaHostAlloc, cudaHostRegister with mapping) when it is
// `align`-byte aligned, else null.
uint8_t *hy_mapped_device_ptr(void *host, uintptr_t align);

#define HY_CUDA(ctx, call)                                   \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return hy_cuda_fail(ctx, e_, #call); \
    } while (0)

// staging buffer (hy_api.cc)
int hy_stage(hy_ctx *ctx, size_t bytes, void **out);

// launchers (hy_render.cu)
int hy_launch_render(hy_ctx *ctx, const hy::ShadeArgs &args);
// reset_counter = false: the sample counter keeps counting from the previous
// passes (a pager frame made of several passes)
int hy_launch_pass(hy_ctx *ctx, const hy::ShadeArgs &args, int pass, bool reset_counter = true);
int hy_finish_stats(hy_ctx *ctx);
int hy_fill_args(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *p, const hy_view *view,
                 int W, int H, hy::ShadeArgs *a);
