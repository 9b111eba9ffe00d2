// hy_render.cu -- shading kernels and the rendering entry points.
//
// Two ways in:
//  * hy_render / hy_render_device: one fused kernel per view does ray
//    generation, the march and the write_to quantisation; no film goes
//    through HBM.  A warp shades an 8x4 ray tile, a 128-thread block a 16x8
//    pixel tile; the transfer function and the u8 normalisation table sit in
//    shared memory.
//  * hy_shade_pass: the four passes of the reference (cuda_shading.cu:14-96)
//    over a caller-owned film in the reference's pixel layout, so a renderer
//    can swap its ShaderMeta.devices[Cuda] entry for this one.

#include <algorithm>
#include <cstring>

#include "hy_shade.cuh"

using namespace hy;
using namespace hy::dev;

namespace {

constexpr int kTileW = 16, kTileH = 8, kThreads = 128;

__device__ __forceinline__ void load_shared(const ShadeArgs &A, float4 *tf, float *lut) {
    stage_tf(A.tf, A.ntf, tf);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = float(i) / 255.f;
    __syncthreads();
}

__device__ __forceinline__ void tile_xy(int &x, int &y) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    x = blockIdx.x * kTileW + (warp & 1) * 8 + (lane & 7);
    y = blockIdx.y * kTileH + (warp >> 1) * 4 + (lane >> 3);
}

__device__ __forceinline__ void count_samples(const ShadeArgs &A, long long samples) {
    if (!A.count) return;
    unsigned long long s = (unsigned long long)samples;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(A.counter, s);
}

// StdVec4Pixel::write_to (pixel_template.hpp:11-20), RGBA: alpha = saturate(v.a).
__device__ __forceinline__ uchar4 quantise(const ShadeArgs &A, float4 v) {
    if (v.w != 0.f)
        return make_uchar4(saturate_u8(v.x), saturate_u8(v.y), saturate_u8(v.z), saturate_u8(v.w));
    return make_uchar4(A.clear_u8[0], A.clear_u8[1], A.clear_u8[2], 0);
}

// LEAN: Volume shader, Default mode, no compositing and no aux output
// (theta / phi are not computed; see VolumeMarch::step).
template <int SHADER, int PC, int DT, bool PADDED, int COMPOSITE, bool LEAN, int GATHER = 0,
          int LOOP = kLoopOne>
__device__ __forceinline__ void render_body(const ShadeArgs &A) {
    extern __shared__ float4 smem[];
    float4 *tf = smem;
    float *lut = reinterpret_cast<float *>(smem + A.ntf + kTfPad);
    load_shared(A, tf, lut);
    const Shared S = make_shared(tf, A.ntf, lut);
    int x, y;
    tile_xy(x, y);
    unsigned int samples = 0;  // one ray: at most max_steps (+ 6 at a hit) samples
    if (x < A.view.W && y < A.view.H) {
        float ox, oy, oz, dx, dy, dz;
        gen_ray(A.view, x, y, ox, oy, oz, dx, dy, dz);
        float4 v, aux;
        if (COMPOSITE) {
            samples = unsigned(
                composite_ray<SHADER, PC, DT, PADDED, GATHER>(A, A.view, S, ox, oy, oz, dx, dy, dz, v, aux));
        } else {
            Px p;
            samples = unsigned(emit<SHADER, PC, DT, PADDED, LEAN, GATHER, LOOP>(
                p, A, A.view, S, ox, oy, oz, dx, dy, dz, 0.f, 0.f, 0.f, A.bbox_max[0],
                A.bbox_max[1], A.bbox_max[2]));
            v = make_float4(p.vx, p.vy, p.vz, p.vw);
            if (SHADER == HY_SHADER_VOLUME)
                aux = make_float4(p.e0, p.e1, p.e2, p.e3);
            else if (SHADER == HY_SHADER_ISOSURFACE)
                aux = make_float4(p.e3, 0.f, 0.f, 0.f);
            else
                aux = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        if constexpr (LEAN) {
            // the pixel again from the thread's index, not held through the
            // march (the memory clobber keeps the compiler from carrying it)
            asm volatile("" ::: "memory");
            tile_xy(x, y);
        }
        const size_t idx = size_t(y) * A.view.W + x;
        A.rgba[idx] = quantise(A, v);
        if (A.vout) A.vout[idx] = v;
        if (!LEAN && A.aux) A.aux[idx] = aux;
    }
    count_samples(A, samples);
}

template <int SHADER, int PC, int DT, bool PADDED, int COMPOSITE, bool LEAN, int LOOP = kLoopOne>
__global__ void __launch_bounds__(kThreads) render_kernel(const __grid_constant__ ShadeArgs A) {
    render_body<SHADER, PC, DT, PADDED, COMPOSITE, LEAN, false, LOOP>(A);
}

// The lean march of the per-view path by loads (f32 volumes, volumes without
// an apron or gather textures) with its own register budget
// (HY_RENDER_LEAN_REGS, 0: the compiler's choice, 56 registers).  64-view
// step of u8 bricks by loads, one launch per view: 56 registers 199.7 ms, 48
// (8 bytes spilled) 211.7 ms, 40 269.0 ms.
#ifndef HY_RENDER_LEAN_REGS
#define HY_RENDER_LEAN_REGS 0
#endif
#if HY_RENDER_LEAN_REGS > 0
#define HY_RENDER_LEAN_BOUNDS __maxnreg__(HY_RENDER_LEAN_REGS)
#else
#define HY_RENDER_LEAN_BOUNDS __launch_bounds__(kThreads)
#endif
template <int SHADER, int PC, int DT, bool PADDED, int LOOP>
__global__ void HY_RENDER_LEAN_BOUNDS render_lean_kernel(const __grid_constant__ ShadeArgs A) {
    render_body<SHADER, PC, DT, PADDED, 0, true, false, LOOP>(A);
}
// The same march sampling by texture gathers (u8 bricks with an apron in
// the volume's gather textures): 64-view step, one launch per view, 169.6
// ms at 48 registers against 172.4 at 56, 173.1 at 64 and 198.8 for the
// loads (HY_RENDER_GATHER=0 builds the per-view path without it).
#ifndef HY_RENDER_GATHER
#define HY_RENDER_GATHER 1
#endif
#ifndef HY_RENDER_GATHER_REGS
#define HY_RENDER_GATHER_REGS 48
#endif
// The paged cache's march (each brick's own mapping, up to 16 textures):
// 56 registers -- 21.2 ms per out-of-core frame against 24.6 at 48 (64 bytes
// spilled) and 22.5 at 64.
#ifndef HY_RENDER_PAGED_GATHER_REGS
#define HY_RENDER_PAGED_GATHER_REGS 56
#endif
template <int SHADER, int PC, int DT, bool PADDED, int GATHER, int LOOP>
__global__ void __maxnreg__(GATHER == kGatherPaged ? HY_RENDER_PAGED_GATHER_REGS
                                                   : HY_RENDER_GATHER_REGS)
    render_lean_gather_kernel(const __grid_constant__ ShadeArgs A) {
    render_body<SHADER, PC, DT, PADDED, 0, true, GATHER, LOOP>(A);
}


// The per-brick compositing variants of the Volume and Isosurface shaders,
// held to 64 registers (8 resident blocks): on the 512^3 tubes at 1024^2,
// Volume 147 -> 163 and Isosurface 231 -> 237 Gsamples/s against 80
// registers and 6 blocks unbounded (Blocks is 3 % faster unbounded and keeps
// render_kernel).
template <int SHADER, int PC, int DT, bool PADDED>
__global__ void __launch_bounds__(kThreads, 8)
    render_composite_kernel(const __grid_constant__ ShadeArgs A) {
    render_body<SHADER, PC, DT, PADDED, 1, false>(A);
}
// The Volume shader's per-brick compositing sampling by gathers (u8 bricks
// with an apron), 64 registers (8 blocks): 64-view step of per-view launches
// 309.2 ms, against 320.7 at 10 blocks, 319.8 at 12 and 334.6 for the loads.
#ifndef HY_RENDER_COMPOSITE_GATHER
#define HY_RENDER_COMPOSITE_GATHER 1
#endif
#ifndef HY_RENDER_COMPOSITE_GATHER_BLOCKS
#define HY_RENDER_COMPOSITE_GATHER_BLOCKS 8
#endif
template <int SHADER, int PC, int DT, bool PADDED>
__global__ void __launch_bounds__(kThreads, HY_RENDER_COMPOSITE_GATHER_BLOCKS)
    render_composite_gather_kernel(const __grid_constant__ ShadeArgs A) {
    render_body<SHADER, PC, DT, PADDED, 1, false, true>(A);
}

// ---- reference-layout film passes ------------------------------------------

template <int SHADER>
__device__ __forceinline__ size_t film_bytes() {
    return (SHADER == HY_SHADER_BLOCKS || SHADER == HY_SHADER_PAGING) ? 48 : 64;
}

template <int SHADER>
__device__ __forceinline__ void store_film(void *film, size_t idx, const Px &p) {
    float4 *q = reinterpret_cast<float4 *>(static_cast<char *>(film) + idx * film_bytes<SHADER>());
    q[0] = make_float4(p.ox, p.oy, p.oz, p.dx);
    q[1] = make_float4(p.dy, p.dz, __int_as_float(p.nsteps), __int_as_float(p.step_size));
    q[2] = make_float4(p.vx, p.vy, p.vz, p.vw);
    if (SHADER != HY_SHADER_BLOCKS && SHADER != HY_SHADER_PAGING)
        q[3] = make_float4(p.e0, p.e1, p.e2, p.e3);
}

template <int SHADER>
__device__ __forceinline__ Px load_film(const void *film, size_t idx) {
    const float4 *q =
        reinterpret_cast<const float4 *>(static_cast<const char *>(film) + idx * film_bytes<SHADER>());
    Px p;
    float4 a = q[0], b = q[1], c = q[2];
    p.ox = a.x;
    p.oy = a.y;
    p.oz = a.z;
    p.dx = a.w;
    p.dy = b.x;
    p.dz = b.y;
    p.nsteps = __float_as_int(b.z);
    p.step_size = __float_as_int(b.w);
    p.vx = c.x;
    p.vy = c.y;
    p.vz = c.z;
    p.vw = c.w;
    if (SHADER != HY_SHADER_BLOCKS && SHADER != HY_SHADER_PAGING) {
        float4 d = q[3];
        p.e0 = d.x;
        p.e1 = d.y;
        p.e2 = d.z;
        p.e3 = d.w;
    } else {
        p.e0 = p.e1 = p.e2 = p.e3 = 0.f;
    }
    return p;
}

// ray_emit_kernel_impl (cuda_shading.cu:14-35)
template <int SHADER, int DT>
__global__ void __launch_bounds__(kThreads) emit_pass_kernel(const __grid_constant__ ShadeArgs A) {
    extern __shared__ float4 smem[];
    float4 *tf = smem;
    float *lut = reinterpret_cast<float *>(smem + A.ntf + kTfPad);
    load_shared(A, tf, lut);
    const Shared S = make_shared(tf, A.ntf, lut);
    int x, y;
    tile_xy(x, y);
    long long samples = 0;
    if (x < A.view.W && y < A.view.H) {
        float ox, oy, oz, dx, dy, dz;
        gen_ray(A.view, x, y, ox, oy, oz, dx, dy, dz);
        Px p;
        samples = emit<SHADER, 0, DT, false>(p, A, A.view, S, ox, oy, oz, dx, dy, dz, 0.f, 0.f, 0.f,
                                             A.bbox_max[0], A.bbox_max[1], A.bbox_max[2]);
        store_film<SHADER>(A.film, size_t(y) * A.view.W + x, p);
    }
    count_samples(A, samples);
}

// ray_march_kernel_impl (cuda_shading.cu:41-54): resumes every pixel.
template <int SHADER, int DT>
__global__ void __launch_bounds__(kThreads) march_pass_kernel(const __grid_constant__ ShadeArgs A) {
    extern __shared__ float4 smem[];
    float4 *tf = smem;
    float *lut = reinterpret_cast<float *>(smem + A.ntf + kTfPad);
    load_shared(A, tf, lut);
    const Shared S = make_shared(tf, A.ntf, lut);
    int x, y;
    tile_xy(x, y);
    long long samples = 0;
    if (x < A.view.W && y < A.view.H) {
        const size_t idx = size_t(y) * A.view.W + x;
        Px p = load_film<SHADER>(A.film, idx);
        samples = run_main<SHADER, 0, DT, false>(p, A, A.view, S);
        store_film<SHADER>(A.film, idx, p);
    }
    count_samples(A, samples);
}

// pixel_kernel_impl (cuda_shading.cu:60-74): film -> uchar3 via write_to.
template <int SHADER>
__global__ void __launch_bounds__(kThreads) pixel_pass_kernel(const __grid_constant__ ShadeArgs A) {
    int x, y;
    tile_xy(x, y);
    if (x >= A.view.W || y >= A.view.H) return;
    const size_t idx = size_t(y) * A.view.W + x;
    Px p = load_film<SHADER>(A.film, idx);
    unsigned char *d = static_cast<unsigned char *>(A.dst) + idx * 3;
    if (p.vw != 0.f) {
        d[0] = saturate_u8(p.vx);
        d[1] = saturate_u8(p.vy);
        d[2] = saturate_u8(p.vz);
    } else {
        d[0] = A.clear_u8[0];
        d[1] = A.clear_u8[1];
        d[2] = A.clear_u8[2];
    }
}

// fetch_kernel_impl (cuda_shading.cu:80-94): VolumeShaderKernel::fetch
// (volume_shader.cu:23-30), IsosurfaceShaderKernel::fetch
// (isosurface_shader.cu:41-48) and PagingShaderKernel::fetch
// (paging_shader.cu:16-22, uchar3 pixels).  The Blocks shader has no fetch.
template <int SHADER>
__global__ void __launch_bounds__(kThreads) fetch_pass_kernel(const __grid_constant__ ShadeArgs A) {
    int x, y;
    tile_xy(x, y);
    if (x >= A.view.W || y >= A.view.H) return;
    const size_t idx = size_t(y) * A.view.W + x;
    Px p = load_film<SHADER>(A.film, idx);
    if (SHADER == HY_SHADER_VOLUME) {
        float4 *d = reinterpret_cast<float4 *>(static_cast<char *>(A.dst) + idx * 32);
        d[0] = make_float4(p.e0, p.e1, p.e2, p.e3);
        d[1] = make_float4(p.vx, p.vy, p.vz, p.vw);
    } else if (SHADER == HY_SHADER_ISOSURFACE) {
        unsigned char *d = static_cast<unsigned char *>(A.dst) + idx * 8;
        d[0] = saturate_u8(p.vx);
        d[1] = saturate_u8(p.vy);
        d[2] = saturate_u8(p.vz);
        d[3] = 0;
        *reinterpret_cast<float *>(d + 4) = p.e3;
    } else if (SHADER == HY_SHADER_PAGING) {
        unsigned char *d = static_cast<unsigned char *>(A.dst) + idx * 3;
        d[0] = saturate_u8(p.vx);
        d[1] = saturate_u8(p.vy);
        d[2] = saturate_u8(p.vz);
    }
}

size_t smem_bytes(const ShadeArgs &a) {
    return size_t(a.ntf + kTfPad) * sizeof(float4) + 256 * sizeof(float);
}

dim3 grid_of(const ShadeArgs &a) {
    return dim3((a.view.W + kTileW - 1) / kTileW, (a.view.H + kTileH - 1) / kTileH);
}

template <int SHADER, int PC, int DT, bool PADDED>
void launch_fused(const ShadeArgs &a, cudaStream_t s) {
    if (a.composite) {
        if constexpr (SHADER == HY_SHADER_BLOCKS)
            render_kernel<SHADER, PC, DT, PADDED, 1, false><<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
        else if constexpr (HY_RENDER_COMPOSITE_GATHER && SHADER == HY_SHADER_VOLUME &&
                           DT == HY_DTYPE_U8 && PADDED) {
            if (a.vol.tex)
                render_composite_gather_kernel<SHADER, PC, DT, PADDED>
                    <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
            else
                render_composite_kernel<SHADER, PC, DT, PADDED>
                    <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
        } else
            render_composite_kernel<SHADER, PC, DT, PADDED><<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
        return;
    }
    if constexpr (SHADER == HY_SHADER_VOLUME) {
        if (a.mode == HY_VOLUME_DEFAULT && !a.aux) {
            const bool ert = a.ert > 0.f;
            if constexpr (DT == HY_DTYPE_U8 && PADDED) {
                if (a.vol.paged_gather) {  // a pager's cache in gather textures
                    if (ert)
                        render_lean_gather_kernel<SHADER, PC, DT, PADDED, kGatherPaged, kLoopErt>
                            <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
                    else
                        render_lean_gather_kernel<SHADER, PC, DT, PADDED, kGatherPaged, kLoopOne>
                            <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
                    return;
                }
            }
            if constexpr (HY_RENDER_GATHER && DT == HY_DTYPE_U8 && PADDED) {
                if (a.vol.tex) {  // bricks in gather textures
                    if (ert)
                        render_lean_gather_kernel<SHADER, PC, DT, PADDED, kGatherResident, kLoopErt>
                            <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
                    else
                        render_lean_gather_kernel<SHADER, PC, DT, PADDED, kGatherResident, kLoopOne>
                            <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
                    return;
                }
            }
            if (ert)
                render_lean_kernel<SHADER, PC, DT, PADDED, kLoopErt>
                    <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
            else
                render_lean_kernel<SHADER, PC, DT, PADDED, kLoopOne>
                    <<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
            return;
        }
    }
    render_kernel<SHADER, PC, DT, PADDED, 0, false><<<grid_of(a), kThreads, smem_bytes(a), s>>>(a);
}

// Instantiations: Blocks reads no bricks; u8 volumes with a 1-voxel apron and
// 64^3 or 128^3 bricks get a compile-time brick edge (immediate offsets).
template <int SHADER>
int dispatch_fused(const ShadeArgs &a, cudaStream_t s) {
    if constexpr (SHADER == HY_SHADER_BLOCKS || SHADER == HY_SHADER_PAGING) {
        launch_fused<SHADER, 0, HY_DTYPE_U8, false>(a, s);
    } else {
        const bool padded = a.vol.pad > 0;
        if (a.vol.dtype == HY_DTYPE_F32) {
            if (padded)
                launch_fused<SHADER, 0, HY_DTYPE_F32, true>(a, s);
            else
                launch_fused<SHADER, 0, HY_DTYPE_F32, false>(a, s);
        } else if (padded && a.vol.P == 66) {
            launch_fused<SHADER, 66, HY_DTYPE_U8, true>(a, s);
        } else if (padded && a.vol.P == 130) {
            launch_fused<SHADER, 130, HY_DTYPE_U8, true>(a, s);
        } else if (padded) {
            launch_fused<SHADER, 0, HY_DTYPE_U8, true>(a, s);
        } else {
            launch_fused<SHADER, 0, HY_DTYPE_U8, false>(a, s);
        }
    }
    return HY_OK;
}

template <int SHADER>
void dispatch_pass(const ShadeArgs &a, int pass, cudaStream_t s) {
    const dim3 g = grid_of(a);
    const size_t sm = smem_bytes(a);
    const bool f32 = a.vol.dtype == HY_DTYPE_F32;
    switch (pass) {
        case HY_PASS_RAY_EMIT:
            if (f32)
                emit_pass_kernel<SHADER, HY_DTYPE_F32><<<g, kThreads, sm, s>>>(a);
            else
                emit_pass_kernel<SHADER, HY_DTYPE_U8><<<g, kThreads, sm, s>>>(a);
            break;
        case HY_PASS_RAY_MARCH:
            if (f32)
                march_pass_kernel<SHADER, HY_DTYPE_F32><<<g, kThreads, sm, s>>>(a);
            else
                march_pass_kernel<SHADER, HY_DTYPE_U8><<<g, kThreads, sm, s>>>(a);
            break;
        case HY_PASS_PIXEL:
            pixel_pass_kernel<SHADER><<<g, kThreads, 0, s>>>(a);
            break;
        default:
            fetch_pass_kernel<SHADER><<<g, kThreads, 0, s>>>(a);
            break;
    }
}

unsigned char sat_host(float f) {
    float x = f * 255.f;
    x = (x < 0.f) ? 0.f : x;
    x = (255.f < x) ? 255.f : x;
    return (unsigned char)x;
}

}  // namespace

int hy_fill_args(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *p, const hy_view *view,
                 int W, int H, ShadeArgs *a) {
    if (!vol || !p) return hy_fail(ctx, HY_ERR_INVALID, "render: null volume or params");
    if (vol->ctx != ctx) return hy_fail(ctx, HY_ERR_INVALID, "render: volume of another context");
    if (!vol->uploaded) return hy_fail(ctx, HY_ERR_STATE, "render: volume not uploaded");
    // the launch grid is W/16 x H/8 tiles (at most 65535 tile rows)
    if (W <= 0 || H <= 0 || (long long)W * H > (1ll << 31) || (H + kTileH - 1) / kTileH > 65535)
        return hy_fail(ctx, HY_ERR_INVALID, "render: bad resolution");
    if (p->shader < HY_SHADER_VOLUME || p->shader > HY_SHADER_PAGING)
        return hy_fail(ctx, HY_ERR_INVALID, "render: unknown shader");
    if (p->shader == HY_SHADER_PAGING && p->composite)
        return hy_fail(ctx, HY_ERR_UNSUPPORTED, "render: the Paging shader has no compositing");
    if (!(p->sample_rate > 0.f)) return hy_fail(ctx, HY_ERR_INVALID, "render: sample_rate <= 0");
    if (p->shader == HY_SHADER_VOLUME && ctx->ntf <= 0)
        return hy_fail(ctx, HY_ERR_STATE, "render: Volume shader needs a transfer function");
    std::memset(a, 0, sizeof(*a));
    a->vol = DevVolume{vol->pool, vol->info_dev, vol->reg_dev, vol->mean_dev, vol->grid[0],
                       vol->grid[1], vol->grid[2], vol->P, vol->desc.dtype, vol->desc.padding,
                       nullptr, {0ull, 0ull}, vol->k, vol->b, nullptr};
    a->vol.gmx = float(vol->grid[0] - 1);
    a->vol.gmy = float(vol->grid[1] - 1);
    a->vol.gmz = float(vol->grid[2] - 1);
    a->vol.fgx = float(vol->grid[0]);
    a->vol.fgy = float(vol->grid[1]);
    hy_volume_gather_view(vol, &a->vol);
    for (int i = 0; i < 3; ++i) a->bbox_max[i] = vol->bbox_max[i];
    a->du = vol->du;
    a->step = vol->du / 4.f / p->sample_rate;  // basic_renderer.hpp:129
    a->max_steps = p->max_steps;
    a->shader = p->shader;
    a->mode = p->mode;
    a->density = p->density;
    a->isovalue = p->isovalue;
    for (int i = 0; i < 3; ++i) {
        a->surface[i] = p->surface_color[i];
        a->view.eye[i] = p->eye_pos[i];
        a->view.light[i] = p->light_pos[i];
        a->clear_u8[i] = sat_host(p->clear_color[i]);  // raycaster.hpp:211
    }
    a->rank = p->rank;
    a->lowest_blkcnt = p->lowest_blkcnt;
    std::memcpy(a->to_world, p->to_world, sizeof(a->to_world));
    a->composite = p->composite;
    a->srgb = p->srgb;
    a->count = p->count_samples;
    // early ray termination: the lean march only (Volume, Default mode, one
    // march through the volume box; films and compositing need full rays)
    if (!(p->early_termination >= 0.f) || p->early_termination > 1.f)
        return hy_fail(ctx, HY_ERR_INVALID, "render: early_termination must be 0 (off) or in (0, 1]");
    a->ert = (p->shader == HY_SHADER_VOLUME && p->mode == HY_VOLUME_DEFAULT && !p->composite)
                 ? p->early_termination
                 : 0.f;
    if (view) {
        std::memcpy(a->view.trans, view->trans, sizeof(a->view.trans));
        a->view.ctg = view->ctg_fovy_2;
        for (int i = 0; i < 3; ++i) a->view.ray_o[i] = view->ray_o[i];
    }
    a->view.W = W;
    a->view.H = H;
    a->tf = ctx->tf_dev;
    a->ntf = ctx->ntf;
    a->counter = ctx->counter_dev;
    return HY_OK;
}

int hy_check_paged_gather(hy_ctx *ctx, const ShadeArgs &a, bool fused) {
    if (!a.vol.paged_gather || a.shader == HY_SHADER_BLOCKS || a.shader == HY_SHADER_PAGING)
        return HY_OK;
    const bool lean = a.shader == HY_SHADER_VOLUME && a.mode == HY_VOLUME_DEFAULT &&
                      !a.composite && !a.aux && a.vol.dtype == HY_DTYPE_U8 && a.vol.pad > 0;
    if (fused && lean) return HY_OK;
    return hy_fail(ctx, HY_ERR_UNSUPPORTED,
                   "a pager's cache in gather textures serves the Volume shader's lean per-view "
                   "march (Default mode, no compositing, no aux output) and the Blocks and "
                   "Paging shaders; create the pager with HY_PAGER_LOADS for this use");
}

int hy_launch_render(hy_ctx *ctx, const ShadeArgs &a) {
    int rc = hy_check_paged_gather(ctx, a, true);
    if (rc) return rc;
    if (a.count) HY_CUDA(ctx, cudaMemsetAsync(ctx->counter_dev, 0, sizeof(unsigned long long), ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    switch (a.shader) {
        case HY_SHADER_VOLUME:
            dispatch_fused<HY_SHADER_VOLUME>(a, ctx->stream);
            break;
        case HY_SHADER_BLOCKS:
            dispatch_fused<HY_SHADER_BLOCKS>(a, ctx->stream);
            break;
        case HY_SHADER_PAGING:
            dispatch_fused<HY_SHADER_PAGING>(a, ctx->stream);
            break;
        default:
            dispatch_fused<HY_SHADER_ISOSURFACE>(a, ctx->stream);
            break;
    }
    HY_CUDA(ctx, cudaGetLastError());
    HY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->stats_pending = true;
    ctx->pend_count = a.count;
    ctx->pend_pixels = (int64_t)a.view.W * a.view.H;
    return HY_OK;
}

int hy_launch_pass(hy_ctx *ctx, const ShadeArgs &a, int pass, bool reset_counter) {
    int rc = hy_check_paged_gather(ctx, a, false);
    if (rc) return rc;
    if (reset_counter && a.count && pass <= HY_PASS_RAY_MARCH)
        HY_CUDA(ctx, cudaMemsetAsync(ctx->counter_dev, 0, sizeof(unsigned long long), ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    switch (a.shader) {
        case HY_SHADER_VOLUME:
            dispatch_pass<HY_SHADER_VOLUME>(a, pass, ctx->stream);
            break;
        case HY_SHADER_BLOCKS:
            dispatch_pass<HY_SHADER_BLOCKS>(a, pass, ctx->stream);
            break;
        case HY_SHADER_PAGING:
            dispatch_pass<HY_SHADER_PAGING>(a, pass, ctx->stream);
            break;
        default:
            dispatch_pass<HY_SHADER_ISOSURFACE>(a, pass, ctx->stream);
            break;
    }
    HY_CUDA(ctx, cudaGetLastError());
    HY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->stats_pending = true;
    ctx->pend_count = a.count && pass <= HY_PASS_RAY_MARCH;
    ctx->pend_pixels = (int64_t)a.view.W * a.view.H;
    return HY_OK;
}

int hy_finish_stats(hy_ctx *ctx) {
    HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!ctx->stats_pending) return HY_OK;
    ctx->stats_pending = false;
    float ms = 0.f;
    HY_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    ctx->stats.ms = ms;
    ctx->stats.pixels = ctx->pend_pixels;
    ctx->stats.samples = -1;
    if (ctx->pend_count) {
        unsigned long long n = 0;
        HY_CUDA(ctx, cudaMemcpy(&n, ctx->counter_dev, sizeof(n), cudaMemcpyDeviceToHost));
        ctx->stats.samples = (int64_t)n;
    }
    return HY_OK;
}

extern "C" int hy_render_device(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *p,
                                const hy_view *view, int32_t W, int32_t H, uint8_t *rgba_dev,
                                float *v_dev, float *aux_dev) {
    if (!ctx) return HY_ERR_INVALID;
    if (!hy_aligned(rgba_dev, 4) || !hy_aligned(v_dev, 16) || !hy_aligned(aux_dev, 16))
        return hy_fail(ctx, HY_ERR_INVALID,
                       "render: misaligned output (rgba 4-byte, float images 16-byte)");
    if (!view || !rgba_dev) return hy_fail(ctx, HY_ERR_INVALID, "render: null view or output");
    ShadeArgs a;
    int rc = hy_fill_args(ctx, vol, p, view, W, H, &a);
    if (rc) return rc;
    a.rgba = reinterpret_cast<uchar4 *>(rgba_dev);
    a.vout = reinterpret_cast<float4 *>(v_dev);
    a.aux = reinterpret_cast<float4 *>(aux_dev);
    return hy_launch_render(ctx, a);
}

uint8_t *hy_mapped_device_ptr(void *host, uintptr_t align) {
    if (!host || !hy_aligned(host, align)) return nullptr;
    cudaPointerAttributes pa{};
    if (cudaPointerGetAttributes(&pa, host) != cudaSuccess) {
        cudaGetLastError();  // not a pointer the runtime knows
        return nullptr;
    }
    if (pa.type != cudaMemoryTypeHost || !hy_aligned(pa.devicePointer, align)) return nullptr;
    return static_cast<uint8_t *>(pa.devicePointer);
}

extern "C" int hy_render(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *p,
                         const hy_view *view, int32_t W, int32_t H, uint8_t *rgba_out,
                         float *v_out, float *aux_out) {
    if (!ctx) return HY_ERR_INVALID;
    if (!view || !rgba_out) return hy_fail(ctx, HY_ERR_INVALID, "render: null view or output");
    ShadeArgs a;
    int rc = hy_fill_args(ctx, vol, p, view, W, H, &a);
    if (rc) return rc;
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    // outputs in pinned, mapped host memory are written by the kernel itself
    // (as in hy_batch_render); the others are staged in device memory and
    // copied once
    uint8_t *rgba_d = hy_mapped_device_ptr(rgba_out, 4);
    uint8_t *v_d = v_out ? hy_mapped_device_ptr(v_out, 16) : nullptr;
    uint8_t *aux_d = aux_out ? hy_mapped_device_ptr(aux_out, 16) : nullptr;
    const size_t npx = size_t(W) * H;
    const size_t rgba_b = (npx * 4 + 255) / 256 * 256, f4_b = npx * 16;
    const size_t total =
        (rgba_d ? 0 : rgba_b) + (v_out && !v_d ? f4_b : 0) + (aux_out && !aux_d ? f4_b : 0);
    char *base = nullptr;
    if (total) {
        void *stage = nullptr;
        rc = hy_stage(ctx, total, &stage);
        if (rc) return rc;
        base = static_cast<char *>(stage);
    }
    size_t off = 0;
    auto place = [&](uint8_t *direct, size_t bytes) -> char * {
        if (direct) return reinterpret_cast<char *>(direct);
        char *q = base + off;
        off += bytes;
        return q;
    };
    a.rgba = reinterpret_cast<uchar4 *>(place(rgba_d, rgba_b));
    if (v_out) a.vout = reinterpret_cast<float4 *>(place(v_d, f4_b));
    if (aux_out) a.aux = reinterpret_cast<float4 *>(place(aux_d, f4_b));
    rc = hy_launch_render(ctx, a);
    if (rc) return rc;
    if (!rgba_d)
        HY_CUDA(ctx, cudaMemcpyAsync(rgba_out, a.rgba, npx * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (v_out && !v_d)
        HY_CUDA(ctx, cudaMemcpyAsync(v_out, a.vout, f4_b, cudaMemcpyDeviceToHost, ctx->stream));
    if (aux_out && !aux_d)
        HY_CUDA(ctx, cudaMemcpyAsync(aux_out, a.aux, f4_b, cudaMemcpyDeviceToHost, ctx->stream));
    return hy_finish_stats(ctx);
}

extern "C" int hy_shade_pass(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *p,
                             int32_t pass, const hy_view *view, void *film_dev, int32_t W,
                             int32_t H, void *dst_dev, const uint8_t clear_rgb[3]) {
    if (!ctx) return HY_ERR_INVALID;
    // films hold float4 records; the Volume fetch pixel is two float4, the
    // Isosurface one stores a float at byte 4 (16 covers both)
    if (!hy_aligned(film_dev, 16) || (pass == HY_PASS_FETCH && !hy_aligned(dst_dev, 16)))
        return hy_fail(ctx, HY_ERR_INVALID,
                       "pass: misaligned film or fetch destination (16-byte)");
    if (pass < HY_PASS_RAY_EMIT || pass > HY_PASS_FETCH)
        return hy_fail(ctx, HY_ERR_INVALID, "pass: unknown pass");
    if (!film_dev) return hy_fail(ctx, HY_ERR_INVALID, "pass: null film");
    if (pass == HY_PASS_RAY_EMIT && !view) return hy_fail(ctx, HY_ERR_INVALID, "pass: emit needs a view");
    if (pass >= HY_PASS_PIXEL && !dst_dev) return hy_fail(ctx, HY_ERR_INVALID, "pass: null destination");
    if (p && p->composite) return hy_fail(ctx, HY_ERR_UNSUPPORTED, "pass: composite is fused-only");
    ShadeArgs a;
    int rc = hy_fill_args(ctx, vol, p, view, W, H, &a);
    if (rc) return rc;
    a.film = film_dev;
    a.dst = dst_dev;
    if (clear_rgb)
        for (int i = 0; i < 3; ++i) a.clear_u8[i] = clear_rgb[i];
    return hy_launch_pass(ctx, a, pass);
}
