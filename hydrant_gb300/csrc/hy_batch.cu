// hy_batch.cu -- many views, one persistent launch, replayed from a CUDA graph.
//
// The reference renders one view per Raycaster pass (raycaster.hpp:32-54):
// each view is its own launch, and small views leave most SMs idle while the
// last wave of a big view drains.  Here every view of a batch is cut into
// warp ray tiles (32 rays: 8x4, 4x8, 16x2 or 32x1 pixels), all tiles of all
// views form one queue, and a persistent grid sized to the GPU takes tiles
// from it (one atomicAdd per `grab` units) until it is empty -- per warp, or
// per block with the block's warps on neighbouring warp tiles.  A
// tile's rays are shaded exactly as in the single-view kernel, so images are
// identical to the per-view path.  The queue head is the only scratch memory;
// the {queue reset, kernel} pair is captured once into a CUDA graph and
// replayed per batch.

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "hy_shade.cuh"

using namespace hy;
using namespace hy::dev;

namespace {

struct BatchView {
    ViewArgs view;
    long long out_off;  // byte offset of the view's RGBA8 image
    int tiles_x;
    int tile0;          // first queue index of this view
};

struct BatchArgs {
    ShadeArgs A;
    const BatchView *views;
    const int *starts;  // tile0 of every view, ascending
    int nviews;
    int total_tiles;
    int tile_w, tile_h, grab;
    int block_queue, bx, by;  // per-block queue units of bx x by warp tiles
    unsigned int *queue;
    unsigned char *out;
};

constexpr int kMaxViews = 2048;
constexpr int kMaxBlockThreads = 256;
// Resident 256-thread blocks per SM the compiler is asked to fit (a register
// budget of 65536 / (256 * n) per thread).
#ifndef HY_BATCH_MIN_BLOCKS
#define HY_BATCH_MIN_BLOCKS 4
#endif

__device__ __forceinline__ int find_view(const int *starts, int n, int t) {
    int lo = 0, hi = n - 1;  // last view with starts[v] <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= t)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// The view and pixel of this thread in queue unit t (see batch_body).
struct UnitPixel {
    const BatchView *bv;
    int x, y;
};
__device__ __forceinline__ UnitPixel unit_pixel(const BatchArgs &B, const int *starts, int t) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int lx = lane % B.tile_w, ly = lane / B.tile_w;
    const int vi = find_view(starts, B.nviews, t);
    const BatchView *bv = B.views + vi;
    const int local = t - starts[vi];
    const int uy = local / bv->tiles_x, ux = local - uy * bv->tiles_x;
    if (B.block_queue) {
        const int wx = warp % B.bx, wy = warp / B.bx;
        return UnitPixel{bv, (ux * B.bx + wx) * B.tile_w + lx, (uy * B.by + wy) * B.tile_h + ly};
    }
    return UnitPixel{bv, ux * B.tile_w + lx, uy * B.tile_h + ly};
}

// Adds a unit's samples of the warp to the launch's counter (every lane of
// the warp comes here together: the queue loops are warp-uniform).
__device__ __forceinline__ void count_unit(const ShadeArgs &A, unsigned int n) {
    unsigned long long s = n;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(A.counter, s);
}

// Shades this thread's pixel of queue unit t and stores its RGBA8 value.
// LEAN: the unit's view and pixel are found again after the march (the empty
// asm with a memory clobber makes the compiler re-read them rather than hold
// the view pointer and pixel coordinates in registers through the march):
// measured when it was introduced, the lean march then fitted 56 registers
// without spilling (171.5 vs 175.4 ms per 64-view step).  The per-brick
// compositing march keeps them (re-deriving measured slower there: 340.3 vs
// 312.6 ms).
template <int SHADER, int PC, int DT, bool PADDED, int COMPOSITE, bool LEAN, int GATHER, int LOOP>
__device__ __forceinline__ unsigned int shade_batch_unit(const BatchArgs &B, const Shared &S,
                                                         const int *starts, int t) {
    const ShadeArgs &A = B.A;
    unsigned int samples;
    float4 v;
    UnitPixel u = unit_pixel(B, starts, t);
    {
        const BatchView &bv = *u.bv;
        if (u.x >= bv.view.W || u.y >= bv.view.H) return 0;
        float ox, oy, oz, dx, dy, dz;
        gen_ray(bv.view, u.x, u.y, ox, oy, oz, dx, dy, dz);
        if (COMPOSITE) {
            float4 aux;
            samples = unsigned(composite_ray<SHADER, PC, DT, PADDED, GATHER>(A, bv.view, S, ox, oy, oz, dx,
                                                                    dy, dz, v, aux));
        } else {
            Px p;
            samples = unsigned(emit<SHADER, PC, DT, PADDED, LEAN, GATHER, LOOP>(
                p, A, bv.view, S, ox, oy, oz, dx, dy, dz, 0.f, 0.f, 0.f, A.bbox_max[0],
                A.bbox_max[1], A.bbox_max[2]));
            v = make_float4(p.vx, p.vy, p.vz, p.vw);
        }
    }
    if constexpr (LEAN) {
        asm volatile("" ::: "memory");
        u = unit_pixel(B, starts, t);
    }
    uchar4 q;
    if (v.w != 0.f)
        q = make_uchar4(saturate_u8(v.x), saturate_u8(v.y), saturate_u8(v.z), saturate_u8(v.w));
    else
        q = make_uchar4(A.clear_u8[0], A.clear_u8[1], A.clear_u8[2], 0);
    *reinterpret_cast<uchar4 *>(B.out + u.bv->out_off + (size_t(u.y) * u.bv->view.W + u.x) * 4) = q;
    return samples;
}

// Queue units: one warp tile per unit (block_queue == 0, each warp takes its
// own units), or one block tile of bx x by warp tiles per unit (block_queue
// == 1, the block takes a unit and warp w shades its w-th warp tile, so the
// warps of an SM work on neighbouring rays and share L1 lines).
// LEAN: Volume shader in Default mode without compositing (theta / phi are
// not needed for an RGBA image; see VolumeMarch::step).
template <int SHADER, int PC, int DT, bool PADDED, int COMPOSITE, bool LEAN, int GATHER = 0,
          int LOOP = kLoopOne>
__device__ __forceinline__ void batch_body(const BatchArgs &B) {
    extern __shared__ float4 smem[];
    __shared__ unsigned int s_t0;
    const ShadeArgs &A = B.A;
    float4 *tf = smem;
    float *lut = reinterpret_cast<float *>(smem + A.ntf + kTfPad);
    int *starts = reinterpret_cast<int *>(lut + 256);
    stage_tf(A.tf, A.ntf, tf);
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = float(i) / 255.f;
    for (int i = threadIdx.x; i < B.nviews; i += blockDim.x) starts[i] = B.starts[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const Shared S = make_shared(tf, A.ntf, lut);
    if (B.block_queue) {
        for (;;) {
            if (threadIdx.x == 0) s_t0 = atomicAdd(B.queue, unsigned(B.grab));
            __syncthreads();
            const unsigned int t0 = s_t0;
            __syncthreads();
            if (t0 >= unsigned(B.total_tiles)) break;
            for (int g = 0; g < B.grab; ++g) {
                const int t = int(t0) + g;
                if (t >= B.total_tiles) break;
                const unsigned int n =
                    shade_batch_unit<SHADER, PC, DT, PADDED, COMPOSITE, LEAN, GATHER, LOOP>(B, S, starts, t);
                if (A.count) count_unit(A, n);
            }
        }
    } else {
        for (;;) {
            unsigned int t0 = 0;
            if (lane == 0) t0 = atomicAdd(B.queue, unsigned(B.grab));
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            if (t0 >= unsigned(B.total_tiles)) break;
            for (int g = 0; g < B.grab; ++g) {
                const int t = int(t0) + g;
                if (t >= B.total_tiles) break;
                const unsigned int n =
                    shade_batch_unit<SHADER, PC, DT, PADDED, COMPOSITE, LEAN, GATHER, LOOP>(B, S, starts, t);
                if (A.count) count_unit(A, n);
            }
        }
    }
}

// The per-brick compositing march sampling by gathers: five 256-thread
// blocks (48 registers, 256 bytes spilled) -- 64-view composite step 293.1
// ms, against 304.9 at four blocks (64 registers) and 298.6 for the loads at
// four (which spill 304 bytes at five, 327.9 ms).
#ifndef HY_BATCH_COMPOSITE_GATHER_MIN_BLOCKS
#define HY_BATCH_COMPOSITE_GATHER_MIN_BLOCKS 5
#endif
template <int SHADER, int PC, int DT, bool PADDED, int COMPOSITE, int GATHER = 0>
__global__ void __launch_bounds__(kMaxBlockThreads,
                                  (COMPOSITE && GATHER) ? HY_BATCH_COMPOSITE_GATHER_MIN_BLOCKS
                                                        : HY_BATCH_MIN_BLOCKS)
    batch_kernel(const __grid_constant__ BatchArgs B) {
    batch_body<SHADER, PC, DT, PADDED, COMPOSITE, false, GATHER>(B);
}

// The lean march over u8 bricks with an apron holds its state in 56
// registers (40 bytes spill), so nine 4-warp blocks fit on an SM: 36
// resident warps hide more of the L1 latency of the tap loads than 32 do
// (64-view step: 178.2 vs 182.0 ms).  f32 and apron-less volumes spill far
// more at 56 and keep 64.  (__maxnreg__ excludes __launch_bounds__; the
// batch launches at most kMaxBlockThreads threads per block.)
#ifndef HY_BATCH_LEAN_REGS
#define HY_BATCH_LEAN_REGS 56
#endif
// The lean march sampling by texture gathers: 48 registers (8 bytes spill)
// for 40 resident warps.  64-view step: 148.2 ms, against 151.1 at 56
// registers (no spills, 36 warps) and 173.1 at 40 (168 bytes spill, 48
// warps).
// The Volume shader's per-brick compositing in the batch samples by
// gathers (1) or loads (0).
#ifndef HY_BATCH_COMPOSITE_GATHER
#define HY_BATCH_COMPOSITE_GATHER 1
#endif
#ifndef HY_BATCH_GATHER_REGS
#define HY_BATCH_GATHER_REGS 48
#endif
template <int DT, bool PADDED, int GATHER>
constexpr int lean_regs() {
    return GATHER ? HY_BATCH_GATHER_REGS : (DT == HY_DTYPE_U8 && PADDED) ? HY_BATCH_LEAN_REGS : 64;
}
template <int SHADER, int PC, int DT, bool PADDED, int GATHER, int LOOP>
__global__ void __maxnreg__((lean_regs<DT, PADDED, GATHER>()))
    batch_lean_kernel(const __grid_constant__ BatchArgs B) {
    batch_body<SHADER, PC, DT, PADDED, 0, true, GATHER, LOOP>(B);
}

template <int SHADER, int PC, int DT, bool PADDED, int GATHER>
const void *pick_lean(const ShadeArgs &a, int steps_per_iter) {
    if (a.ert > 0.f)
        return reinterpret_cast<const void *>(
            &batch_lean_kernel<SHADER, PC, DT, PADDED, GATHER, kLoopErt>);
    if (steps_per_iter == 2)
        return reinterpret_cast<const void *>(
            &batch_lean_kernel<SHADER, PC, DT, PADDED, GATHER, kLoopTwo>);
    return reinterpret_cast<const void *>(&batch_lean_kernel<SHADER, PC, DT, PADDED, GATHER, kLoopOne>);
}

template <int SHADER, int PC, int DT, bool PADDED>
const void *pick_c(const ShadeArgs &a, int steps_per_iter) {
    if (a.composite) {
        // the Volume shader's per-brick segments sample by gathers too
        if constexpr (SHADER == HY_SHADER_VOLUME && DT == HY_DTYPE_U8 && PADDED) {
            if (a.vol.tex && HY_BATCH_COMPOSITE_GATHER)
                return reinterpret_cast<const void *>(&batch_kernel<SHADER, PC, DT, PADDED, 1, true>);
        }
        return reinterpret_cast<const void *>(&batch_kernel<SHADER, PC, DT, PADDED, 1>);
    }
    if constexpr (SHADER == HY_SHADER_VOLUME) {
        if (a.mode == HY_VOLUME_DEFAULT) {
            if constexpr (DT == HY_DTYPE_U8 && PADDED) {
                if (a.vol.tex)  // bricks in gather textures
                    return pick_lean<SHADER, PC, DT, PADDED, true>(a, steps_per_iter);
            }
            return pick_lean<SHADER, PC, DT, PADDED, false>(a, steps_per_iter);
        }
    }
    return reinterpret_cast<const void *>(&batch_kernel<SHADER, PC, DT, PADDED, 0>);
}

template <int SHADER>
const void *pick_shader(const ShadeArgs &a, int spi) {
    if constexpr (SHADER == HY_SHADER_BLOCKS || SHADER == HY_SHADER_PAGING) {
        return pick_c<SHADER, 0, HY_DTYPE_U8, false>(a, spi);
    } else {
        const bool padded = a.vol.pad > 0;
        if (a.vol.dtype == HY_DTYPE_F32) {
            return padded ? pick_c<SHADER, 0, HY_DTYPE_F32, true>(a, spi)
                          : pick_c<SHADER, 0, HY_DTYPE_F32, false>(a, spi);
        }
        if (padded && a.vol.P == 66) return pick_c<SHADER, 66, HY_DTYPE_U8, true>(a, spi);
        if (padded && a.vol.P == 130) return pick_c<SHADER, 130, HY_DTYPE_U8, true>(a, spi);
        return padded ? pick_c<SHADER, 0, HY_DTYPE_U8, true>(a, spi)
                      : pick_c<SHADER, 0, HY_DTYPE_U8, false>(a, spi);
    }
}

// steps_per_iter: march steps per loop iteration of the lean Volume march
// (1 or 2; early termination keeps 1)
const void *pick_kernel(const ShadeArgs &a, int steps_per_iter = 1) {
    switch (a.shader) {
        case HY_SHADER_VOLUME:
            return pick_shader<HY_SHADER_VOLUME>(a, steps_per_iter);
        case HY_SHADER_BLOCKS:
            return pick_shader<HY_SHADER_BLOCKS>(a, steps_per_iter);
        case HY_SHADER_PAGING:
            return pick_shader<HY_SHADER_PAGING>(a, steps_per_iter);
        default:
            return pick_shader<HY_SHADER_ISOSURFACE>(a, steps_per_iter);
    }
}

}  // namespace

struct hy_batch {
    hy_ctx *ctx = nullptr;
    const hy_volume *vol = nullptr;
    hy_shader_params params{};
    std::vector<hy_batch_view> in;
    std::vector<BatchView> views;
    std::vector<int> starts;
    BatchView *views_dev = nullptr;
    int *starts_dev = nullptr;
    unsigned int *queue_dev = nullptr;
    int total_tiles = 0;
    int64_t out_bytes = 0;
    hy_batch_config cfg{8, 1, 4, 0, 1};
    ShadeArgs base{};
    const void *kernel = nullptr;
    size_t smem = 0;
    int grid = 0;
    cudaGraphExec_t exec = nullptr;
    uint8_t *graph_out = nullptr;
    int graph_count = -1;
    // new cameras between renders (hy_batch_update_views): descriptors staged
    // in pinned host memory, copied to views_dev on the stream; the event
    // marks when the staging buffer may be rewritten
    BatchView *views_pinned = nullptr;
    cudaEvent_t upd_ev = nullptr;
    bool upd_pending = false;
};

namespace {

// Dynamic shared memory above the default 48 KiB needs an opt-in per kernel.
// (The CUDA runtime's default L1 / shared-memory split is kept: asking for the
// largest L1 left too little shared memory for the resident blocks.)
cudaError_t allow_smem(const void *kernel, size_t smem) {
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
}

bool valid_config(const hy_batch_config &c) {
    const bool tw = c.tile_w == 4 || c.tile_w == 8 || c.tile_w == 16 || c.tile_w == 32;
    return tw && c.grab >= 1 && c.grab <= 16 && c.block_warps >= 1 &&
           c.block_warps * 32 <= kMaxBlockThreads && c.blocks_per_sm >= 0 &&
           c.blocks_per_sm <= 32 && (c.block_queue == 0 || c.block_queue == 1) &&
           c.steps_per_iter >= 0 && c.steps_per_iter <= 2;
}

void drop_graph(hy_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->graph_out = nullptr;
    b->graph_count = -1;
}

void unit_shape(const hy_batch_config &c, int &bx, int &by) {
    if (!c.block_queue) {
        bx = by = 1;
        return;
    }
    bx = (c.block_warps >= 4 && c.block_warps % 2 == 0) ? 2 : c.block_warps;
    by = c.block_warps / bx;
}

// One view's device descriptor: camera, lighting, size, output offset and
// its place in the tile queue.
void fill_view(BatchView &d, const hy_batch_view &v, int tiles_x, int tile0) {
    std::memset(&d, 0, sizeof(d));
    std::memcpy(d.view.trans, v.view.trans, sizeof(d.view.trans));
    d.view.ctg = v.view.ctg_fovy_2;
    for (int k = 0; k < 3; ++k) {
        d.view.ray_o[k] = v.view.ray_o[k];
        d.view.eye[k] = v.eye_pos[k];
        d.view.light[k] = v.light_pos[k];
    }
    d.view.W = v.width;
    d.view.H = v.height;
    d.out_off = v.rgba_offset;
    d.tiles_x = tiles_x;
    d.tile0 = tile0;
}

// (Re)build the tile layout for the current config and the persistent grid.
int layout(hy_batch *b) {
    hy_ctx *ctx = b->ctx;
    b->kernel = pick_kernel(b->base, b->cfg.steps_per_iter == 2 ? 2 : 1);
    int bx, by;
    unit_shape(b->cfg, bx, by);
    const int tw = b->cfg.tile_w * bx, th = (32 / b->cfg.tile_w) * by;
    b->views.resize(b->in.size());
    b->starts.resize(b->in.size());
    long long tile = 0;
    for (size_t i = 0; i < b->in.size(); ++i) {
        const hy_batch_view &v = b->in[i];
        BatchView &d = b->views[i];
        fill_view(d, v, (v.width + tw - 1) / tw, int(tile));
        b->starts[i] = int(tile);
        tile += (long long)d.tiles_x * ((v.height + th - 1) / th);
    }
    if (tile >= (1ll << 31) - 64) return hy_fail(ctx, HY_ERR_INVALID, "batch: too many ray tiles");
    b->total_tiles = int(tile);
    HY_CUDA(ctx, cudaMemcpyAsync(b->views_dev, b->views.data(), b->views.size() * sizeof(BatchView),
                                 cudaMemcpyHostToDevice, ctx->stream));
    HY_CUDA(ctx, cudaMemcpyAsync(b->starts_dev, b->starts.data(), b->starts.size() * sizeof(int),
                                 cudaMemcpyHostToDevice, ctx->stream));
    HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    b->smem = size_t(b->base.ntf + kTfPad) * sizeof(float4) + 256 * sizeof(float) +
              b->in.size() * sizeof(int);
    HY_CUDA(ctx, allow_smem(b->kernel, b->smem));
    const int threads = b->cfg.block_warps * 32;
    int per_sm = b->cfg.blocks_per_sm;
    if (per_sm == 0) {
        HY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->kernel, threads,
                                                                   b->smem));
        per_sm = std::max(per_sm, 1);
    }
    int sms = 0;
    HY_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    b->grid = sms * per_sm;
    drop_graph(b);
    return HY_OK;
}

int launch(hy_batch *b, uint8_t *out) {
    hy_ctx *ctx = b->ctx;
    // the batch renders with the context's current transfer function: a new
    // table (hy_tf_set may have reallocated it) or knot count means new
    // kernel arguments, shared-memory size and graph
    if (b->base.tf != ctx->tf_dev || b->base.ntf != ctx->ntf) {
        if (b->params.shader == HY_SHADER_VOLUME && ctx->ntf <= 0)
            return hy_fail(ctx, HY_ERR_STATE, "batch: Volume shader needs a transfer function");
        b->base.tf = ctx->tf_dev;
        b->base.ntf = ctx->ntf;
        int rc = layout(b);
        if (rc) return rc;
    }
    const int count = b->params.count_samples ? 1 : 0;
    if (!b->exec || b->graph_out != out || b->graph_count != count) {
        drop_graph(b);
        BatchArgs args;
        args.A = b->base;
        args.A.count = count;
        args.views = b->views_dev;
        args.starts = b->starts_dev;
        args.nviews = int(b->views.size());
        args.total_tiles = b->total_tiles;
        args.tile_w = b->cfg.tile_w;
        args.tile_h = 32 / b->cfg.tile_w;
        args.grab = b->cfg.grab;
        args.block_queue = b->cfg.block_queue;
        unit_shape(b->cfg, args.bx, args.by);
        args.queue = b->queue_dev;
        args.out = out;
        void *kargs[] = {&args};
        cudaGraph_t graph = nullptr;
        HY_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(b->queue_dev, 0, sizeof(unsigned int), ctx->stream);
        if (count) cudaMemsetAsync(ctx->counter_dev, 0, sizeof(unsigned long long), ctx->stream);
        cudaError_t le = cudaLaunchKernel(b->kernel, dim3(b->grid), dim3(b->cfg.block_warps * 32),
                                          kargs, b->smem, ctx->stream);
        cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (le != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return hy_cuda_fail(ctx, le, "batch: kernel launch during capture");
        }
        HY_CUDA(ctx, ce);
        cudaError_t ie = cudaGraphInstantiate(&b->exec, graph, 0);
        cudaGraphDestroy(graph);
        HY_CUDA(ctx, ie);
        b->graph_out = out;
        b->graph_count = count;
    }
    HY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    HY_CUDA(ctx, cudaGraphLaunch(b->exec, ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->stats_pending = true;
    ctx->pend_count = count;
    int64_t px = 0;
    for (auto &v : b->in) px += (int64_t)v.width * v.height;
    ctx->pend_pixels = px;
    return HY_OK;
}

}  // namespace

extern "C" int hy_batch_create(hy_ctx *ctx, const hy_volume *vol, const hy_shader_params *params,
                               const hy_batch_view *views, int32_t nviews, hy_batch **out) {
    if (!ctx || !out) return HY_ERR_INVALID;
    *out = nullptr;
    if (!views || nviews <= 0 || nviews > kMaxViews)
        return hy_fail(ctx, HY_ERR_INVALID, "batch: need 1..2048 views");
    if (params && params->composite && params->shader == HY_SHADER_VOLUME && params->srgb) {
        // supported: sRGB is applied per ray after compositing
    }
    hy::ShadeArgs base;
    int rc = hy_fill_args(ctx, vol, params, nullptr, 1, 1, &base);
    if (rc) return rc;
    rc = hy_check_paged_gather(ctx, base, false);
    if (rc) return rc;
    for (int i = 0; i < nviews; ++i) {
        const hy_batch_view &v = views[i];
        if (v.width <= 0 || v.height <= 0 || v.rgba_offset < 0 || (v.rgba_offset & 3))
            return hy_fail(ctx, HY_ERR_INVALID, "batch: bad view size or output offset");
    }
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    hy_batch *b = new hy_batch();
    b->ctx = ctx;
    b->vol = vol;
    b->params = *params;
    b->in.assign(views, views + nviews);
    b->base = base;
    b->kernel = pick_kernel(base);
    for (auto &v : b->in)
        b->out_bytes = std::max<int64_t>(b->out_bytes, v.rgba_offset + (int64_t)v.width * v.height * 4);
    cudaError_t e = cudaMalloc(&b->views_dev, sizeof(BatchView) * nviews);
    if (e == cudaSuccess) e = cudaMalloc(&b->starts_dev, sizeof(int) * nviews);
    if (e == cudaSuccess) e = cudaMalloc(&b->queue_dev, sizeof(unsigned int));
    if (e == cudaSuccess)
        e = cudaHostAlloc(&b->views_pinned, sizeof(BatchView) * nviews, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->upd_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        hy_batch_destroy(b);
        return hy_cuda_fail(ctx, e, "batch: allocation");
    }
    rc = layout(b);
    if (rc) {
        hy_batch_destroy(b);
        return rc;
    }
    *out = b;
    return HY_OK;
}

extern "C" int hy_batch_destroy(hy_batch *b) {
    if (!b) return HY_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    drop_graph(b);
    if (b->views_dev) cudaFree(b->views_dev);
    if (b->starts_dev) cudaFree(b->starts_dev);
    if (b->queue_dev) cudaFree(b->queue_dev);
    if (b->views_pinned) cudaFreeHost(b->views_pinned);
    if (b->upd_ev) cudaEventDestroy(b->upd_ev);
    delete b;
    return HY_OK;
}

// New cameras for the next renders: the views keep their sizes and output
// offsets (so the tile queue, the launch and the captured graph stay), only
// the ViewArgs and lighting change.  The descriptors go through a pinned
// staging buffer and one copy on the context's stream, ordered before the
// next render; the call returns without waiting for it (it waits only for
// the previous update's copy before rewriting the staging buffer).
extern "C" int hy_batch_update_views(hy_batch *b, const hy_batch_view *views, int32_t nviews) {
    if (!b) return HY_ERR_INVALID;
    hy_ctx *ctx = b->ctx;
    if (!views || nviews != int32_t(b->in.size()))
        return hy_fail(ctx, HY_ERR_INVALID, "batch: update needs the batch's number of views");
    for (int i = 0; i < nviews; ++i)
        if (views[i].width != b->in[i].width || views[i].height != b->in[i].height ||
            views[i].rgba_offset != b->in[i].rgba_offset)
            return hy_fail(ctx, HY_ERR_INVALID,
                           "batch: an update keeps every view's size and output offset");
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    if (b->upd_pending) HY_CUDA(ctx, cudaEventSynchronize(b->upd_ev));
    for (int i = 0; i < nviews; ++i) {
        b->in[i] = views[i];
        fill_view(b->views[i], views[i], b->views[i].tiles_x, b->views[i].tile0);
    }
    std::memcpy(b->views_pinned, b->views.data(), sizeof(BatchView) * size_t(nviews));
    HY_CUDA(ctx, cudaMemcpyAsync(b->views_dev, b->views_pinned, sizeof(BatchView) * size_t(nviews),
                                 cudaMemcpyHostToDevice, ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(b->upd_ev, ctx->stream));
    b->upd_pending = true;
    return HY_OK;
}

extern "C" int hy_batch_view_bytes(const hy_batch *b, int64_t *bytes) {
    if (!b || !bytes) return HY_ERR_INVALID;
    *bytes = int64_t(sizeof(BatchView)) * int64_t(b->in.size());
    return HY_OK;
}

extern "C" int hy_batch_output_bytes(const hy_batch *b, int64_t *bytes) {
    if (!b || !bytes) return HY_ERR_INVALID;
    *bytes = b->out_bytes;
    return HY_OK;
}

extern "C" int hy_batch_set_config(hy_batch *b, const hy_batch_config *cfg) {
    if (!b || !cfg) return HY_ERR_INVALID;
    if (!valid_config(*cfg)) return hy_fail(b->ctx, HY_ERR_INVALID, "batch: bad config");
    b->cfg = *cfg;
    return layout(b);
}

extern "C" int hy_batch_get_config(const hy_batch *b, hy_batch_config *out) {
    if (!b || !out) return HY_ERR_INVALID;
    *out = b->cfg;
    return HY_OK;
}

extern "C" int hy_batch_set_counting(hy_batch *b, int32_t count_samples) {
    if (!b) return HY_ERR_INVALID;
    b->params.count_samples = count_samples ? 1 : 0;
    return HY_OK;
}

extern "C" int hy_batch_render_device(hy_batch *b, uint8_t *rgba_dev) {
    if (!b) return HY_ERR_INVALID;
    if (!hy_aligned(rgba_dev, 4)) return hy_fail(b->ctx, HY_ERR_INVALID, "batch: misaligned output (4-byte)");
    if (!rgba_dev) return hy_fail(b->ctx, HY_ERR_INVALID, "batch: null output");
    return launch(b, rgba_dev);
}

// A host buffer that is pinned and mapped into the device's address space
// (cudaHostAlloc, or cudaHostRegister with mapping -- what a serving process
// allocates for its frames) is written by the kernel itself: the pixels
// cross the host link while the march runs, with no staging copy after it.
// Any other host buffer (or one not 4-byte aligned) gets the image through a
// device staging buffer and one copy.

extern "C" int hy_batch_render(hy_batch *b, uint8_t *rgba_host) {
    if (!b) return HY_ERR_INVALID;
    if (!rgba_host) return hy_fail(b->ctx, HY_ERR_INVALID, "batch: null output");
    hy_ctx *ctx = b->ctx;
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    if (uint8_t *direct = hy_mapped_device_ptr(rgba_host, 4)) {
        int rc = launch(b, direct);
        if (rc) return rc;
        return hy_finish_stats(ctx);
    }
    void *stage = nullptr;
    int rc = hy_stage(ctx, size_t(b->out_bytes), &stage);
    if (rc) return rc;
    rc = launch(b, static_cast<uint8_t *>(stage));
    if (rc) return rc;
    HY_CUDA(ctx, cudaMemcpyAsync(rgba_host, stage, size_t(b->out_bytes), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    return hy_finish_stats(ctx);
}

// Times every candidate launch shape on this batch and keeps the fastest.
extern "C" int hy_batch_autotune(hy_batch *b, uint8_t *rgba_dev, int32_t reps,
                                 hy_batch_config *best_out) {
    if (!b || !rgba_dev) return HY_ERR_INVALID;
    hy_ctx *ctx = b->ctx;
    if (!hy_aligned(rgba_dev, 4)) return hy_fail(ctx, HY_ERR_INVALID, "batch: misaligned output (4-byte)");
    if (reps <= 0) reps = 3;
    const int tws[] = {8, 4, 16};
    const int grabs[] = {1, 2, 4};
    const int warps[] = {2, 4, 8};
    const int count = b->params.count_samples;
    b->params.count_samples = 0;
    hy_batch_config best = b->cfg;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    HY_CUDA(ctx, cudaEventCreate(&e0));
    HY_CUDA(ctx, cudaEventCreate(&e1));
    int rc = HY_OK;
    for (int bq = 0; bq < 2; ++bq)
    for (int tw : tws)
        for (int g : grabs)
            for (int w : warps) {
                hy_batch_config c{tw, g, w, 0, bq, 1};
                b->cfg = c;
                if ((rc = layout(b))) goto done;
                if ((rc = launch(b, rgba_dev))) goto done;  // warm-up and graph build
                HY_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
                for (int r = 0; r < reps; ++r)
                    if ((rc = launch(b, rgba_dev))) goto done;
                HY_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
                HY_CUDA(ctx, cudaEventSynchronize(e1));
                float ms = 0.f;
                HY_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
            }
    // samples per loop iteration on the fastest shape
    if (b->base.shader == HY_SHADER_VOLUME && b->base.mode == HY_VOLUME_DEFAULT &&
        !b->base.composite && !(b->base.ert > 0.f)) {
        hy_batch_config c = best;
        c.steps_per_iter = 2;
        b->cfg = c;
        if ((rc = layout(b))) goto done;
        if ((rc = launch(b, rgba_dev))) goto done;
        HY_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        for (int r = 0; r < reps; ++r)
            if ((rc = launch(b, rgba_dev))) goto done;
        HY_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        HY_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.f;
        HY_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
done:
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->params.count_samples = count;
    ctx->stats_pending = false;
    if (rc) return rc;
    b->cfg = best;
    rc = layout(b);
    if (rc) return rc;
    if (best_out) *best_out = best;
    return HY_OK;
}

// ---- rendering a batch of views without allocating ---------------------------
//
// hy_render_views_noalloc is for callers that may not allocate device memory
// while they render: a host application that owns the GPU's memory budget and
// only lends this library its inputs and outputs, or a real-time frame loop
// that cannot afford the implicit synchronisation and fragmentation of
// cudaMalloc/cudaFree in the middle of a frame.  It renders like
// hy_batch_render_device with the default launch shape, but keeps its scratch
// -- the work-queue head, the first tile of each view and the per-view
// descriptors -- in the file-scope array below instead of device allocations.
//
// The array is a fixed kNoAllocScratchBytes (about 33 KiB) that every GPU
// which loads this library holds until the process exits.  Its device address
// is looked up once per device, on the first call made on that device (with
// the device made current), so that first call should come before any stream
// capture.  All calls share the array and it keeps the last call's contents:
// each call rewrites the descriptors and clears the queue head on its stream
// before launching, and calls whose work overlaps on the GPU (other streams,
// other host threads, several contexts on one device) race on it.

constexpr int kNoAllocMaxViews = 256;
constexpr size_t kNoAllocQueueBytes = 256;
constexpr size_t kNoAllocStartsBytes = (kNoAllocMaxViews * sizeof(int) + 255) / 256 * 256;
constexpr size_t kNoAllocScratchBytes =
    kNoAllocQueueBytes + kNoAllocStartsBytes + kNoAllocMaxViews * sizeof(BatchView);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on ctx's device (host code cannot use
// the symbol itself: on the host it names a stand-in, not device memory).
int noalloc_scratch(hy_ctx *ctx, unsigned char **out) {
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return hy_fail(ctx, HY_ERR_INVALID, "noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[ctx->device]) {
        HY_CUDA(ctx, cudaSetDevice(ctx->device));
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return hy_cuda_fail(ctx, e, "noalloc: cudaGetSymbolAddress(scratch)");
        g_noalloc_addr[ctx->device] = static_cast<unsigned char *>(p);
    }
    *out = g_noalloc_addr[ctx->device];
    return HY_OK;
}

}  // namespace

extern "C" int hy_render_views_noalloc(hy_ctx *ctx, const hy_volume *vol,
                                       const hy_shader_params *params,
                                       const hy_batch_view *views, int32_t nviews,
                                       uint8_t *rgba_dev) {
    if (!ctx) return HY_ERR_INVALID;
    if (!hy_aligned(rgba_dev, 4))
        return hy_fail(ctx, HY_ERR_INVALID, "noalloc: misaligned output (4-byte)");
    if (!views || !rgba_dev) return hy_fail(ctx, HY_ERR_INVALID, "noalloc: null views or output");
    if (nviews <= 0 || nviews > kNoAllocMaxViews)
        return hy_fail(ctx, HY_ERR_INVALID,
                       "noalloc: nviews must be 1..256 (the static scratch holds 256 views)");
    ShadeArgs base;
    int rc = hy_fill_args(ctx, vol, params, nullptr, 1, 1, &base);
    if (rc) return rc;
    rc = hy_check_paged_gather(ctx, base, false);
    if (rc) return rc;
    base.count = 0;  // sample counting is not available on this entry point
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    // The descriptors are copied from this call's stack: a captured copy
    // would replay from a dead address, so capture is refused.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    HY_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cap));
    if (cap != cudaStreamCaptureStatusNone)
        return hy_fail(ctx, HY_ERR_STATE,
                       "noalloc: the stream is capturing (view descriptors are copied from "
                       "host stack memory; call it outside capture)");
    unsigned char *scratch = nullptr;
    rc = noalloc_scratch(ctx, &scratch);
    if (rc) return rc;

    // default launch shape: 8x4 warp tiles, block tiles of 2x2 warp tiles,
    // one block tile per queue access
    const hy_batch_config cfg{8, 1, 4, 0, 1};
    int bx, by;
    unit_shape(cfg, bx, by);
    const int uw = cfg.tile_w * bx, uh = (32 / cfg.tile_w) * by;
    BatchView hv[kNoAllocMaxViews];
    int hs[kNoAllocMaxViews];
    long long tile = 0;
    for (int i = 0; i < nviews; ++i) {
        const hy_batch_view &v = views[i];
        if (v.width <= 0 || v.height <= 0 || v.rgba_offset < 0 || (v.rgba_offset & 3))
            return hy_fail(ctx, HY_ERR_INVALID, "noalloc: bad view size or output offset");
        BatchView &d = hv[i];
        std::memset(&d, 0, sizeof(d));
        std::memcpy(d.view.trans, v.view.trans, sizeof(d.view.trans));
        d.view.ctg = v.view.ctg_fovy_2;
        for (int k = 0; k < 3; ++k) {
            d.view.ray_o[k] = v.view.ray_o[k];
            d.view.eye[k] = v.eye_pos[k];
            d.view.light[k] = v.light_pos[k];
        }
        d.view.W = v.width;
        d.view.H = v.height;
        d.out_off = v.rgba_offset;
        d.tiles_x = (v.width + uw - 1) / uw;
        d.tile0 = int(tile);
        hs[i] = int(tile);
        tile += (long long)d.tiles_x * ((v.height + uh - 1) / uh);
        if (tile >= (1ll << 31) - 64) return hy_fail(ctx, HY_ERR_INVALID, "noalloc: too many tiles");
    }
    unsigned int *queue = reinterpret_cast<unsigned int *>(scratch);
    int *starts = reinterpret_cast<int *>(scratch + kNoAllocQueueBytes);
    BatchView *vdev = reinterpret_cast<BatchView *>(scratch + kNoAllocQueueBytes + kNoAllocStartsBytes);
    HY_CUDA(ctx, cudaMemcpyAsync(vdev, hv, size_t(nviews) * sizeof(BatchView),
                                 cudaMemcpyHostToDevice, ctx->stream));
    HY_CUDA(ctx, cudaMemcpyAsync(starts, hs, size_t(nviews) * sizeof(int), cudaMemcpyHostToDevice,
                                 ctx->stream));
    HY_CUDA(ctx, cudaMemsetAsync(queue, 0, sizeof(unsigned int), ctx->stream));

    BatchArgs args;
    args.A = base;
    args.views = vdev;
    args.starts = starts;
    args.nviews = nviews;
    args.total_tiles = int(tile);
    args.tile_w = cfg.tile_w;
    args.tile_h = 32 / cfg.tile_w;
    args.grab = cfg.grab;
    args.block_queue = cfg.block_queue;
    args.bx = bx;
    args.by = by;
    args.queue = queue;
    args.out = rgba_dev;
    const void *kernel = pick_kernel(base);
    const int threads = cfg.block_warps * 32;
    const size_t smem = size_t(base.ntf + kTfPad) * sizeof(float4) + 256 * sizeof(float) +
                        size_t(nviews) * sizeof(int);
    int per_sm = 0, sms = 0;
    HY_CUDA(ctx, allow_smem(kernel, smem));
    HY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
    HY_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    void *kargs[] = {&args};
    HY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    HY_CUDA(ctx, cudaLaunchKernel(kernel, dim3(sms * std::max(per_sm, 1)), dim3(threads), kargs,
                                  smem, ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->stats_pending = true;
    ctx->pend_count = 0;
    int64_t px = 0;
    for (int i = 0; i < nviews; ++i) px += (int64_t)views[i].width * views[i].height;
    ctx->pend_pixels = px;
    return HY_OK;
}
