// hy_page.cu -- out-of-core volumes: a pinned host brick store, visible-brick
// culling on the GPU, and a pager that keeps a fixed HBM brick cache filled.
//
// Reference: LosslessBlockPagingServer (src/slave/paging/
// lossless_block_paging.cc:116-174) renders a frame in batches of resident
// bricks, nearest first, re-emitting nothing: rays that reach an absent brick
// stop (volume_shader.cu:49-50) and the next batch's march pass resumes them.
// RtBlockPagingServer (src/slave/paging/rt_block_paging.cc:249-326) keeps the
// nearest visible bricks resident across frames, replacing bricks that left
// the visible set.  Both take the visible set from OctreeCuller::cull
// (include/hydrant/octree_culler.hpp:121-161).
//
// Here the bricks live in one pinned host allocation (the "store"), laid out
// exactly like device slots, so a brick upload is a single DMA
// (cudaMemcpyAsync) on a copy stream; the page table (int2 per brick) is
// rewritten on the render stream after an event says the bricks arrived.  In
// lossless mode the cache is double-buffered: batch k+1 uploads into the
// other half while batch k marches.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <numeric>
#include <thread>
#include <vector>

#include "hy_shade.cuh"

using namespace hy;
using namespace hy::dev;

// ---------------------------------------------------------------------------
// Brick store
// ---------------------------------------------------------------------------

// Chebyshev distance transform over the brick grid (26-neighbour dilation).
void hy_chebyshev_transform(const std::vector<unsigned char> &ne, const int g[3],
                            std::vector<int> &out) {
    const int n = g[0] * g[1] * g[2];
    const int cap = std::max(g[0], std::max(g[1], g[2]));
    out.assign(n, -1);
    std::vector<int> frontier;
    for (int i = 0; i < n; ++i)
        if (ne[i]) {
            out[i] = 0;
            frontier.push_back(i);
        }
    for (int r = 1; r <= cap && !frontier.empty(); ++r) {
        std::vector<int> next;
        for (int id : frontier) {
            const int x = id % g[0], y = (id / g[0]) % g[1], z = id / (g[0] * g[1]);
            for (int k = 0; k < 27; ++k) {
                const int X = x + k % 3 - 1, Y = y + (k / 3) % 3 - 1, Z = z + k / 9 - 1;
                if (X < 0 || Y < 0 || Z < 0 || X >= g[0] || Y >= g[1] || Z >= g[2]) continue;
                const int j = (Z * g[1] + Y) * g[0] + X;
                if (out[j] < 0) {
                    out[j] = r;
                    next.push_back(j);
                }
            }
        }
        frontier.swap(next);
    }
    for (int i = 0; i < n; ++i)
        if (out[i] < 0) out[i] = cap;
}

int hy_store_alloc(hy_store *s, int nonempty) {
    s->nonempty = nonempty;
    s->host_bytes = std::max<size_t>(1, size_t(nonempty)) * s->slot_stride;
    HY_CUDA(s->ctx, cudaHostAlloc(reinterpret_cast<void **>(&s->host), s->host_bytes,
                                  cudaHostAllocMapped | cudaHostAllocPortable));
    void *dev = nullptr;
    HY_CUDA(s->ctx, cudaHostGetDevicePointer(&dev, s->host, 0));
    s->host_dev = static_cast<const unsigned char *>(dev);
    return HY_OK;
}

namespace {

// ---- procedural value noise (the 32 GiB paging workload) --------------------

__device__ __forceinline__ unsigned int mix32(unsigned int h) {
    h ^= h >> 16;
    h *= 0x7feb352dU;
    h ^= h >> 15;
    h *= 0x846ca68bU;
    h ^= h >> 16;
    return h;
}

__device__ __forceinline__ float lattice(unsigned int seed, int o, int x, int y, int z) {
    unsigned int h = mix32(seed ^ mix32(unsigned(o) * 0x9E3779B9U ^ mix32(unsigned(x) ^
                                         mix32(unsigned(y) * 0x85EBCA6BU ^ mix32(unsigned(z))))));
    return float(h >> 8) * (1.f / 16777216.f);
}

// one octave of lattice value noise with smoothstep weights at p (cells)
__device__ __forceinline__ float value_noise(unsigned int seed, int o, float px, float py, float pz) {
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const int ix = int(fx), iy = int(fy), iz = int(fz);
    float tx = px - fx, ty = py - fy, tz = pz - fz;
    tx = tx * tx * (3.f - 2.f * tx);
    ty = ty * ty * (3.f - 2.f * ty);
    tz = tz * tz * (3.f - 2.f * tz);
    float c[2][2];
    for (int k = 0; k < 2; ++k)
        for (int j = 0; j < 2; ++j) {
            const float a = lattice(seed, o, ix, iy + j, iz + k);
            const float b = lattice(seed, o, ix + 1, iy + j, iz + k);
            c[k][j] = a + (b - a) * tx;
        }
    const float y0 = c[0][0] + (c[0][1] - c[0][0]) * ty;
    const float y1 = c[1][0] + (c[1][1] - c[1][0]) * ty;
    return y0 + (y1 - y0) * tz;
}

// 3 octaves (cell, cell/2, cell/4; amplitudes 1, 1/2, 1/4), normalised to [0,1)
__device__ __forceinline__ float noise3(unsigned int seed, float inv_cell, int x, int y, int z) {
    const float px = (float(x) + 0.5f) * inv_cell, py = (float(y) + 0.5f) * inv_cell,
                pz = (float(z) + 0.5f) * inv_cell;
    float n = value_noise(seed, 0, px, py, pz);
    n += 0.5f * value_noise(seed, 1, 2.f * px, 2.f * py, 2.f * pz);
    n += 0.25f * value_noise(seed, 2, 4.f * px, 4.f * py, 4.f * pz);
    return n * (1.f / 1.75f);
}

__device__ __forceinline__ unsigned char noise_voxel(unsigned int seed, float inv_cell, float thr,
                                                     int x, int y, int z) {
    const float n = noise3(seed, inv_cell, x, y, z);
    if (!(n > thr)) return 0;
    const float v = 1.f + floorf(254.f * (n - thr) / (1.f - thr));
    return (unsigned char)fminf(255.f, v);
}

// noise at hashed sample positions, for the occupancy threshold
__global__ void noise_sample_kernel(unsigned int seed, float inv_cell, int dx, int dy, int dz,
                                    int n, float *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned int h1 = mix32(unsigned(i) * 2654435761U ^ 0x1234567U);
    const unsigned int h2 = mix32(h1 ^ 0x9E3779B9U), h3 = mix32(h2 ^ 0x7F4A7C15U);
    out[i] = noise3(seed, inv_cell, int(h1 % unsigned(dx)), int(h2 % unsigned(dy)),
                    int(h3 % unsigned(dz)));
}

struct NoiseChunk {
    unsigned int seed;
    float inv_cell, thr;
    int dx, dy, dz, bs, pad, gx, gy;
    int brick0;
    long long slot_stride;
    unsigned char *out;         // chunk of padded bricks (nullptr: flags only)
    unsigned int *nonempty;     // per brick of the chunk
    unsigned long long *sum;    // per brick: sum of core voxels
};

// One block per brick of the chunk: padded voxels (apron clamped at the
// volume border), emptiness and the core sum.
__global__ void noise_brick_kernel(const __grid_constant__ NoiseChunk a) {
    const int bid = a.brick0 + blockIdx.x;
    const int bx = bid % a.gx, by = (bid / a.gx) % a.gy, bz = bid / (a.gx * a.gy);
    const int P = a.bs + 2 * a.pad;
    const long long P3 = (long long)P * P * P;
    unsigned int any = 0;
    unsigned long long sum = 0;
    unsigned char *dst = a.out ? a.out + (long long)blockIdx.x * a.slot_stride : nullptr;
    for (long long i = threadIdx.x; i < P3; i += blockDim.x) {
        const int x = int(i % P), y = int((i / P) % P), z = int(i / ((long long)P * P));
        const int X = min(max(bx * a.bs + x - a.pad, 0), a.dx - 1);
        const int Y = min(max(by * a.bs + y - a.pad, 0), a.dy - 1);
        const int Z = min(max(bz * a.bs + z - a.pad, 0), a.dz - 1);
        const unsigned char v = noise_voxel(a.seed, a.inv_cell, a.thr, X, Y, Z);
        if (dst) dst[i] = v;
        any |= v != 0;
        const bool core = x >= a.pad && x < a.pad + a.bs && y >= a.pad && y < a.pad + a.bs &&
                          z >= a.pad && z < a.pad + a.bs;
        if (core) sum += v;
    }
    __shared__ unsigned long long ssum[32];
    __shared__ unsigned int sany[32];
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        any |= __shfl_down_sync(0xffffffffu, any, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        ssum[warp] = sum;
        sany[warp] = any;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long s = 0;
        unsigned int an = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) {
            s += ssum[w];
            an |= sany[w];
        }
        a.nonempty[blockIdx.x] = an;
        a.sum[blockIdx.x] = s;
    }
}



}  // namespace

void hy_store_geometry(hy_store *s, const hy_volume_desc &d) {
    s->desc = d;
    for (int i = 0; i < 3; ++i) s->grid[i] = (d.dim[i] + d.block_size - 1) / d.block_size;
    s->nbricks = s->grid[0] * s->grid[1] * s->grid[2];
    s->P = d.block_size + 2 * d.padding;
    const size_t elem = d.dtype == HY_DTYPE_U8 ? 1 : 4;
    s->slot_stride = (size_t(s->P) * s->P * s->P * elem + 255) / 256 * 256;
}

extern "C" int hy_store_from_volume(const hy_volume *vol, hy_store **out) {
    if (!vol || !out) return HY_ERR_INVALID;
    *out = nullptr;
    hy_ctx *ctx = vol->ctx;
    if (!vol->uploaded || vol->paged)
        return hy_fail(ctx, HY_ERR_STATE, "store: needs a resident, uploaded volume");
    hy_store *s = new hy_store();
    s->ctx = ctx;
    hy_store_geometry(s, vol->desc);
    s->cheb = vol->cheb;
    s->mean = vol->mean;
    s->offset.assign(s->nbricks, -1);
    int rc = hy_store_alloc(s, vol->resident);
    if (rc) {
        delete s;
        return rc;
    }
    for (int b = 0; b < s->nbricks; ++b)
        if (vol->reg_of_brick[b] >= 0) s->offset[b] = (long long)vol->reg_of_brick[b] * s->slot_stride;
    cudaError_t e = cudaMemcpyAsync(s->host, vol->pool, size_t(vol->resident) * s->slot_stride,
                                    cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        hy_store_destroy(s);
        return hy_cuda_fail(ctx, e, "store: copy bricks to host");
    }
    *out = s;
    return HY_OK;
}

extern "C" int hy_store_create_noise(hy_ctx *ctx, const hy_volume_desc *desc, uint64_t seed,
                                     float cell_voxels, float occupancy, hy_store **out) {
    if (!ctx || !desc || !out) return HY_ERR_INVALID;
    *out = nullptr;
    if (desc->dtype != HY_DTYPE_U8) return hy_fail(ctx, HY_ERR_INVALID, "noise store: u8 only");
    if (!(cell_voxels >= 1.f) || !(occupancy > 0.f && occupancy < 1.f))
        return hy_fail(ctx, HY_ERR_INVALID, "noise store: bad cell size or occupancy");
    hy_volume tmp;
    int rc = hy_volume_init(ctx, desc, &tmp);
    if (rc) return rc;
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    hy_store *s = new hy_store();
    s->ctx = ctx;
    hy_store_geometry(s, *desc);
    const unsigned int sd = unsigned(seed ^ (seed >> 32));
    const float inv_cell = 1.f / cell_voxels;
    // occupancy threshold: the (1 - occupancy) quantile of 2^22 sampled voxels
    const int ns = 1 << 22;
    float *samp = nullptr;
    unsigned char *chunk = nullptr;
    unsigned int *ne_dev = nullptr;
    unsigned long long *sum_dev = nullptr;
    const int CH = 512;
    auto fail = [&](cudaError_t e, const char *what) {
        if (samp) cudaFree(samp);
        if (chunk) cudaFree(chunk);
        if (ne_dev) cudaFree(ne_dev);
        if (sum_dev) cudaFree(sum_dev);
        hy_store_destroy(s);
        return hy_cuda_fail(ctx, e, what);
    };
    cudaError_t e = cudaMalloc(&samp, ns * sizeof(float));
    if (e != cudaSuccess) return fail(e, "noise store: sample buffer");
    noise_sample_kernel<<<(ns + 255) / 256, 256, 0, ctx->stream>>>(sd, inv_cell, desc->dim[0],
                                                                   desc->dim[1], desc->dim[2], ns,
                                                                   samp);
    std::vector<float> hs(ns);
    e = cudaMemcpyAsync(hs.data(), samp, ns * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(e, "noise store: threshold samples");
    const size_t q = size_t(double(ns) * (1.0 - double(occupancy)));
    std::nth_element(hs.begin(), hs.begin() + q, hs.end());
    const float thr = hs[q];
    e = cudaMalloc(&chunk, size_t(CH) * s->slot_stride);
    if (e == cudaSuccess) e = cudaMalloc(&ne_dev, CH * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMalloc(&sum_dev, CH * sizeof(unsigned long long));
    if (e != cudaSuccess) return fail(e, "noise store: chunk buffers");
    NoiseChunk a{sd, inv_cell, thr, desc->dim[0], desc->dim[1], desc->dim[2], desc->block_size,
                 desc->padding, s->grid[0], s->grid[1], 0, (long long)s->slot_stride, nullptr,
                 ne_dev, sum_dev};
    // pass 1: emptiness and means
    std::vector<unsigned char> ne(s->nbricks);
    std::vector<unsigned long long> sums(s->nbricks);
    std::vector<unsigned int> nb(CH);
    for (int b0 = 0; b0 < s->nbricks; b0 += CH) {
        const int n = std::min(CH, s->nbricks - b0);
        a.brick0 = b0;
        a.out = nullptr;
        noise_brick_kernel<<<n, 256, 0, ctx->stream>>>(a);
        e = cudaMemcpyAsync(nb.data(), ne_dev, n * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                            ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&sums[b0], sum_dev, n * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return fail(e, "noise store: emptiness pass");
        for (int i = 0; i < n; ++i) ne[b0 + i] = nb[i] ? 1 : 0;
    }
    hy_chebyshev_transform(ne, s->grid, s->cheb);
    const double ncore = double(desc->block_size) * desc->block_size * desc->block_size;
    s->mean.resize(s->nbricks);
    s->offset.assign(s->nbricks, -1);
    int nonempty = 0;
    for (int b = 0; b < s->nbricks; ++b) {
        s->mean[b] = float(double(sums[b]) / 255.0 / ncore);
        if (ne[b]) s->offset[b] = (long long)(nonempty++) * s->slot_stride;
    }
    rc = hy_store_alloc(s, nonempty);
    if (rc) {
        cudaFree(samp);
        cudaFree(chunk);
        cudaFree(ne_dev);
        cudaFree(sum_dev);
        hy_store_destroy(s);
        return rc;
    }
    // pass 2: generate and copy the non-empty bricks into the pinned store
    for (int b0 = 0; b0 < s->nbricks; b0 += CH) {
        const int n = std::min(CH, s->nbricks - b0);
        bool any = false;
        for (int i = 0; i < n; ++i) any |= ne[b0 + i] != 0;
        if (!any) continue;
        a.brick0 = b0;
        a.out = chunk;
        noise_brick_kernel<<<n, 256, 0, ctx->stream>>>(a);
        for (int i = 0; i < n; ++i)
            if (ne[b0 + i]) {
                e = cudaMemcpyAsync(s->host + s->offset[b0 + i], chunk + size_t(i) * s->slot_stride,
                                    s->slot_stride, cudaMemcpyDeviceToHost, ctx->stream);
                if (e != cudaSuccess) return fail(e, "noise store: brick copy");
            }
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return fail(e, "noise store: generation pass");
    }
    cudaFree(samp);
    cudaFree(chunk);
    cudaFree(ne_dev);
    cudaFree(sum_dev);
    *out = s;
    return HY_OK;
}

namespace {

// fn(i) for i in [0, n) over the host's cores
template <typename F>
void parallel_for(int n, F fn) {
    const int nt = std::max(1, std::min<int>(n, int(std::thread::hardware_concurrency())));
    std::atomic<int> next{0};
    std::vector<std::thread> ts;
    for (int t = 0; t < nt; ++t)
        ts.emplace_back([&]() {
            for (int i = next++; i < n; i = next++) fn(i);
        });
    for (auto &t : ts) t.join();
}

// Coarse voxels of one fine brick: with bs a multiple of sc, the sc^3 cube of
// every coarse voxel lies inside a single fine brick.
template <typename T, typename Acc>
void coarse_of_brick(const hy_store *s, int b, int sc, const int cdim[3], T *cvol) {
    const int bs = s->desc.block_size, pad = s->desc.padding, P = s->P;
    const int *dim = s->desc.dim;
    const int bx = b % s->grid[0], by = (b / s->grid[0]) % s->grid[1],
              bz = b / (s->grid[0] * s->grid[1]);
    const T *src = reinterpret_cast<const T *>(s->host + s->offset[b]);
    const int cpb = bs / sc;
    for (int cz = 0; cz < cpb; ++cz)
        for (int cy = 0; cy < cpb; ++cy)
            for (int cx = 0; cx < cpb; ++cx) {
                const int X = bx * cpb + cx, Y = by * cpb + cy, Z = bz * cpb + cz;
                if (X >= cdim[0] || Y >= cdim[1] || Z >= cdim[2]) continue;
                Acc sum = 0;
                long long cnt = 0;
                for (int z = Z * sc; z < std::min(Z * sc + sc, dim[2]); ++z)
                    for (int y = Y * sc; y < std::min(Y * sc + sc, dim[1]); ++y)
                        for (int x = X * sc; x < std::min(X * sc + sc, dim[0]); ++x) {
                            const int lx = x - bx * bs + pad, ly = y - by * bs + pad,
                                      lz = z - bz * bs + pad;
                            sum += Acc(src[(size_t(lz) * P + ly) * P + lx]);
                            ++cnt;
                        }
                T out;
                if constexpr (sizeof(T) == 1)
                    out = T((sum + Acc(cnt / 2)) / Acc(cnt));  // round half up
                else
                    out = T(double(sum) / double(cnt));
                cvol[(size_t(Z) * cdim[1] + Y) * cdim[0] + X] = out;
            }
}

template <typename T>
void build_coarse(hy_store *s, int sc, const int cdim[3]) {
    const size_t nc = size_t(cdim[0]) * cdim[1] * cdim[2];
    std::vector<T> cvol(nc, T(0));  // empty fine bricks stay 0
    parallel_for(s->nbricks, [&](int b) {
        if (s->offset[b] < 0) return;
        if constexpr (sizeof(T) == 1)
            coarse_of_brick<T, unsigned long long>(s, b, sc, cdim, cvol.data());
        else
            coarse_of_brick<T, double>(s, b, sc, cdim, cvol.data());
    });
    // brick the coarse volume like the fine one: apron clamped at its border
    const int bs = s->desc.block_size, pad = s->desc.padding, P = s->P;
    const int *g = s->coarse_grid;
    s->coarse.assign(size_t(s->ncoarse) * s->slot_stride, 0);
    parallel_for(s->ncoarse, [&](int cb) {
        const int bx = cb % g[0], by = (cb / g[0]) % g[1], bz = cb / (g[0] * g[1]);
        T *dst = reinterpret_cast<T *>(s->coarse.data() + size_t(cb) * s->slot_stride);
        for (int k = 0; k < P; ++k)
            for (int j = 0; j < P; ++j)
                for (int i = 0; i < P; ++i) {
                    const int x = std::min(std::max(bx * bs + i - pad, 0), cdim[0] - 1);
                    const int y = std::min(std::max(by * bs + j - pad, 0), cdim[1] - 1);
                    const int z = std::min(std::max(bz * bs + k - pad, 0), cdim[2] - 1);
                    dst[(size_t(k) * P + j) * P + i] = cvol[(size_t(z) * cdim[1] + y) * cdim[0] + x];
                }
    });
}

}  // namespace

extern "C" int hy_store_build_coarse(hy_store *s, int32_t level) {
    if (!s) return HY_ERR_INVALID;
    hy_ctx *ctx = s->ctx;
    const int bs = s->desc.block_size;
    if (level < 1 || level > 12 || bs % (1 << level) != 0)
        return hy_fail(ctx, HY_ERR_INVALID,
                       "store: coarse level must be >= 1 with block_size a multiple of 2^level");
    const int sc = 1 << level;
    int cdim[3];
    for (int i = 0; i < 3; ++i) {
        cdim[i] = (s->desc.dim[i] + sc - 1) / sc;
        s->coarse_grid[i] = (cdim[i] + bs - 1) / bs;
    }
    s->ncoarse = s->coarse_grid[0] * s->coarse_grid[1] * s->coarse_grid[2];
    s->coarse_level = level;
    if (s->desc.dtype == HY_DTYPE_U8)
        build_coarse<unsigned char>(s, sc, cdim);
    else
        build_coarse<float>(s, sc, cdim);
    return HY_OK;
}

extern "C" int hy_store_coarse_grid(const hy_store *s, int32_t grid[3]) {
    if (!s || !grid) return HY_ERR_INVALID;
    for (int i = 0; i < 3; ++i) grid[i] = s->coarse_grid[i];
    return HY_OK;
}

extern "C" int hy_store_coarse_brick(const hy_store *s, int32_t brick, void *out) {
    if (!s || !out || brick < 0 || brick >= s->ncoarse) return HY_ERR_INVALID;
    const size_t bytes = size_t(s->P) * s->P * s->P * (s->desc.dtype == HY_DTYPE_U8 ? 1 : 4);
    std::memcpy(out, s->coarse.data() + size_t(brick) * s->slot_stride, bytes);
    return HY_OK;
}

extern "C" int hy_store_destroy(hy_store *s) {
    if (!s) return HY_OK;
    if (s->host) cudaFreeHost(s->host);
    delete s;
    return HY_OK;
}

extern "C" int hy_store_get_info(const hy_store *s, hy_volume_info *out) {
    if (!s || !out) return HY_ERR_INVALID;
    for (int i = 0; i < 3; ++i) {
        out->grid[i] = s->grid[i];
        out->bbox_max[i] = float(s->desc.dim[i]) / float(s->desc.block_size);
    }
    out->nbricks = s->nbricks;
    out->nonempty = s->nonempty;
    out->resident = 0;
    out->padded = s->P;
    out->slot_bytes = (int64_t)s->slot_stride;
    out->pool_bytes = (int64_t)s->host_bytes;
    return HY_OK;
}

extern "C" int hy_store_thumbnails(const hy_store *s, int32_t *chebyshev, float *mean) {
    if (!s) return HY_ERR_INVALID;
    for (int i = 0; i < s->nbricks; ++i) {
        if (chebyshev) chebyshev[i] = s->cheb[i];
        if (mean) mean[i] = s->mean[i];
    }
    return HY_OK;
}

extern "C" int hy_store_brick(const hy_store *s, int32_t brick, void *out) {
    if (!s || !out || brick < 0 || brick >= s->nbricks) return HY_ERR_INVALID;
    const size_t bytes = size_t(s->P) * s->P * s->P * (s->desc.dtype == HY_DTYPE_U8 ? 1 : 4);
    if (s->offset[brick] < 0)
        std::memset(out, 0, bytes);
    else
        std::memcpy(out, s->host + s->offset[brick], bytes);
    return HY_OK;
}

// ---------------------------------------------------------------------------
// Visible-brick culling (OctreeCuller::cull, octree_culler.hpp:121-161).
// Frustum: border rays at (+-1, +-1, -ctg) in camera space; plane normals
// cross(border[i], border[i+1]) and the origin are taken to object space, the
// border directions are used untransformed (octree_culler.hpp:324-345, as in
// the reference).  A brick is visible if it is non-empty and contains_fast()
// accepts its box: a corner inside all four planes, or a border ray from the
// origin that hits the box with tfar > 0 (octree_culler.hpp:162-183).
// ---------------------------------------------------------------------------
namespace {

struct CullArgs {
    float norm[4][3];
    float rdir[4][3];  // 1 / normalize(border[i])
    float orig[3];
    const int *cheb;  // chebyshev value of brick b at cheb[b * cheb_stride]
    int cheb_stride;
    int gx, gy, gz;
    int *ids;
    float *d2;
    unsigned int *count;
};

__device__ __forceinline__ bool frustum_contains(const CullArgs &a, float x, float y, float z) {
    const float px = x - a.orig[0], py = y - a.orig[1], pz = z - a.orig[2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        if (!(a.norm[i][0] * px + a.norm[i][1] * py + a.norm[i][2] * pz > 0.f)) return false;
    return true;
}

__global__ void cull_kernel(const __grid_constant__ CullArgs a) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= a.gx * a.gy * a.gz) return;
    if (a.cheb[size_t(id) * a.cheb_stride] != 0) return;
    const int x = id % a.gx, y = (id / a.gx) % a.gy, z = id / (a.gx * a.gy);
    const float x0 = float(x), y0 = float(y), z0 = float(z);
    const float x1 = float(x + 1), y1 = float(y + 1), z1 = float(z + 1);
    const float vx[2] = {x0, x1}, vy[2] = {y0, y1}, vz[2] = {z0, z1};
    bool hit = false;
    for (int i = 0; i < 2 && !hit; ++i)
        for (int j = 0; j < 2 && !hit; ++j)
            for (int k = 0; k < 2 && !hit; ++k) hit = frustum_contains(a, vx[i], vy[j], vz[k]);
    for (int i = 0; i < 4 && !hit; ++i) {
        float tnear, tfar;
        if (intersect(a.orig[0], a.orig[1], a.orig[2], a.rdir[i][0], a.rdir[i][1], a.rdir[i][2], x0,
                      y0, z0, x1, y1, z1, tnear, tfar) &&
            tfar > 0.f)
            hit = true;
    }
    if (!hit) return;
    const float cx = x0 + .5f - a.orig[0], cy = y0 + .5f - a.orig[1], cz = z0 + .5f - a.orig[2];
    const unsigned int slot = atomicAdd(a.count, 1u);
    a.ids[slot] = id;
    a.d2[slot] = cx * cx + cy * cy + cz * cz;
}

void hcross(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - b[1] * a[2];
    o[1] = a[2] * b[0] - b[2] * a[0];
    o[2] = a[0] * b[1] - b[0] * a[1];
}

void host_frustum(const hy_view &v, const float rect[4], CullArgs &a) {
    const float ctg = v.ctg_fovy_2;
    const float border[4][3] = {{rect[2], rect[3], -ctg},
                                {rect[2], rect[1], -ctg},
                                {rect[0], rect[1], -ctg},
                                {rect[0], rect[3], -ctg}};
    const float *m = v.trans;
    for (int i = 0; i < 4; ++i) {
        float n[3];
        hcross(border[i], border[(i + 1) % 4], n);
        for (int r = 0; r < 3; ++r)
            a.norm[i][r] = m[r] * n[0] + m[4 + r] * n[1] + m[8 + r] * n[2] + m[12 + r] * 0.f;
        const float s = 1.f / std::sqrt(border[i][0] * border[i][0] + border[i][1] * border[i][1] +
                                        border[i][2] * border[i][2]);
        for (int r = 0; r < 3; ++r) a.rdir[i][r] = 1.f / (border[i][r] * s);
    }
    for (int r = 0; r < 3; ++r)
        a.orig[r] = m[r] * 0.f + m[4 + r] * 0.f + m[8 + r] * 0.f + m[12 + r] * 1.f;
}

struct CullScratch {
    int *ids = nullptr;
    float *d2 = nullptr;
    unsigned int *count = nullptr;
    int cap = 0;
};

// Culls on `stream` (default: the context's); the chebyshev values come
// from the volume's page table unless `cheb` (one int per brick) is given.
int run_cull(hy_ctx *ctx, const hy_volume *vol, const hy_view &view, const float rect_in[4],
             int limit, CullScratch &cs, std::vector<int> &ids, std::vector<float> &d2,
             std::vector<int> *all_visible = nullptr, cudaStream_t stream = nullptr,
             const int *cheb = nullptr) {
    if (!stream) stream = ctx->stream;
    const float def_rect[4] = {-1.f, -1.f, 1.f, 1.f};
    const float *rect = rect_in ? rect_in : def_rect;
    if (cs.cap < vol->nbricks) {
        if (cs.ids) cudaFree(cs.ids);
        if (cs.d2) cudaFree(cs.d2);
        if (cs.count) cudaFree(cs.count);
        cs = CullScratch{};
        HY_CUDA(ctx, cudaMalloc(&cs.ids, vol->nbricks * sizeof(int)));
        HY_CUDA(ctx, cudaMalloc(&cs.d2, vol->nbricks * sizeof(float)));
        HY_CUDA(ctx, cudaMalloc(&cs.count, sizeof(unsigned int)));
        cs.cap = vol->nbricks;
    }
    CullArgs a;
    host_frustum(view, rect, a);
    a.cheb = cheb ? cheb : reinterpret_cast<const int *>(vol->info_dev);
    a.cheb_stride = cheb ? 1 : 2;
    a.gx = vol->grid[0];
    a.gy = vol->grid[1];
    a.gz = vol->grid[2];
    a.ids = cs.ids;
    a.d2 = cs.d2;
    a.count = cs.count;
    HY_CUDA(ctx, cudaMemsetAsync(cs.count, 0, sizeof(unsigned int), stream));
    cull_kernel<<<(vol->nbricks + 255) / 256, 256, 0, stream>>>(a);
    HY_CUDA(ctx, cudaGetLastError());
    unsigned int n = 0;
    HY_CUDA(ctx, cudaMemcpyAsync(&n, cs.count, sizeof(n), cudaMemcpyDeviceToHost, stream));
    HY_CUDA(ctx, cudaStreamSynchronize(stream));
    std::vector<int> hid(n);
    std::vector<float> hd(n);
    if (n) {
        HY_CUDA(ctx, cudaMemcpyAsync(hid.data(), cs.ids, n * sizeof(int), cudaMemcpyDeviceToHost,
                                     stream));
        HY_CUDA(ctx, cudaMemcpyAsync(hd.data(), cs.d2, n * sizeof(float), cudaMemcpyDeviceToHost,
                                     stream));
        HY_CUDA(ctx, cudaStreamSynchronize(stream));
    }
    if (all_visible) *all_visible = hid;
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    size_t keep = n;
    if (limit >= 0 && size_t(limit) < n) {
        // nearest `limit` by (distance^2, index)
        std::nth_element(idx.begin(), idx.begin() + limit, idx.end(), [&](int x, int y) {
            return hd[x] < hd[y] || (hd[x] == hd[y] && hid[x] < hid[y]);
        });
        keep = size_t(limit);
        idx.resize(keep);
    }
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return hid[x] < hid[y]; });
    ids.resize(keep);
    d2.resize(keep);
    for (size_t i = 0; i < keep; ++i) {
        ids[i] = hid[idx[i]];
        d2[i] = hd[idx[i]];
    }
    return HY_OK;
}

}  // namespace

extern "C" int hy_cull(const hy_volume *vol, const hy_view *view, const float rect[4],
                       int32_t limit, int32_t *ids_out, float *dist2_out, int32_t *n_out) {
    if (!vol || !view || !n_out) return HY_ERR_INVALID;
    hy_ctx *ctx = vol->ctx;
    if (!vol->info_dev) return hy_fail(ctx, HY_ERR_STATE, "cull: volume has no page table");
    CullScratch cs;
    std::vector<int> ids;
    std::vector<float> d2;
    int rc = run_cull(ctx, vol, *view, rect, limit, cs, ids, d2);
    if (cs.ids) cudaFree(cs.ids);
    if (cs.d2) cudaFree(cs.d2);
    if (cs.count) cudaFree(cs.count);
    if (rc) return rc;
    for (size_t i = 0; i < ids.size(); ++i) {
        if (ids_out) ids_out[i] = ids[i];
        if (dist2_out) dist2_out[i] = d2[i];
    }
    *n_out = int32_t(ids.size());
    return HY_OK;
}

// ---------------------------------------------------------------------------
// Pager
// ---------------------------------------------------------------------------
namespace {

// One brick move of a realtime frame: store bytes at `src` -> cache slot `dst`.
struct GatherItem {
    long long src;
    int dst;
    int pad_;
};

// One block per brick: the slot is filled straight from the mapped pinned
// store (the GPU reads host memory over the C2C link), 16 bytes per thread
// and iteration; slot_stride is a multiple of 256 bytes.
__global__ void gather_bricks_kernel(const unsigned char *__restrict__ store,
                                     const GatherItem *__restrict__ items,
                                     unsigned char *__restrict__ pool, long long slot0,
                                     long long stride) {
    const GatherItem it = items[blockIdx.x];
    const uint4 *src = reinterpret_cast<const uint4 *>(store + it.src);
    uint4 *dst = reinterpret_cast<uint4 *>(pool + (slot0 + it.dst) * stride);
    const int n = int(stride / 16);
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// The same moves into a cache held in gather textures: one block per brick
// reads the record from the mapped pinned store (16 bytes per thread and
// iteration) and writes it through the texture's surface, two texels per
// write (P is even and every brick's column origin a multiple of P, so a
// pair never straddles a row): record byte r = row * P + col lands at
// texel (x0 + col, y0 + row).  Writes outside the array are dropped.
struct GatherSurfaces {
    unsigned long long s[hy::kMaxGatherTextures];
};
__global__ void fill_textures_kernel(const unsigned char *__restrict__ store,
                                     const GatherItem *__restrict__ items, GatherSurfaces surf,
                                     int P, int gper, int gcols, int slot0) {
    const GatherItem it = items[blockIdx.x];
    const int g = slot0 + it.dst;
    const int t = g / gper, i = g % gper;
    const int x0 = (i % gcols) * P, y0 = (i / gcols) * P * P;
    const cudaSurfaceObject_t so = cudaSurfaceObject_t(surf.s[t & (hy::kMaxGatherTextures - 1)]);
    const uint4 *src = reinterpret_cast<const uint4 *>(store + it.src);
    const int nbytes = P * P * P;
    const int nchunks = (nbytes + 15) / 16;
    for (int j = threadIdx.x; j < nchunks; j += blockDim.x) {
        const uint4 q = src[j];
        const unsigned int w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int r = j * 16 + 2 * k;
            if (r >= nbytes) break;
            const unsigned int v = (w[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
            const int row = r / P, col = r - row * P;
            surf2Dwrite(make_uchar2((unsigned char)(v & 0xff), (unsigned char)(v >> 8)), so,
                        x0 + col, y0 + row, cudaBoundaryModeZero);
        }
    }
}

}  // namespace

struct hy_pager {
    hy_ctx *ctx = nullptr;
    hy_store *store = nullptr;
    hy_volume *vol = nullptr;    // paged volume: pool = cache slots
    hy_pager_desc desc{};
    int nslots = 0;              // device slots (2 x batch in lossless mode)
    cudaStream_t copy = nullptr;
    cudaEvent_t copied = nullptr;
    cudaEvent_t marched[2] = {nullptr, nullptr};  // last pass that used each cache half
    cudaEvent_t staged[2] = {nullptr, nullptr};   // page-table copy out of each staging buffer
    std::vector<int> page;       // brick -> slot, -1 absent
    std::vector<int> owner;      // slot -> brick, -1 free
    // realtime with the store's coarse level: the coarse bricks occupy the
    // first `ncoarse` pool slots, registry ids [0, nbricks) sample them and
    // cache slot i is registry id reg_base + i
    bool coarse = false;
    int ncoarse = 0;
    int reg_base = 0;
    int next_free = 0;           // realtime: slots never used yet
    // realtime, LRU: per slot the last frame its brick was visible
    std::vector<int64_t> stamp;
    // realtime prefetch (hy_pager_prefetch): the next camera's missing bricks
    // move on the copy stream while the current frame renders, into slots
    // that no page table of a frame still in flight references -- never-used
    // slots, or spares: slots evicted a frame early and kept out of the page
    // table.  Arrived bricks enter the page table at the next frame.
    bool prefetching = false;
    int reserve = 0;                           // spare slots kept while prefetching
    std::vector<int> spare;
    std::vector<std::pair<int, int>> arrived;  // (brick, slot)
    cudaEvent_t rendered[2] = {nullptr, nullptr};  // realtime frames' renders, alternating
    int rendered_i = 0;                            // the last frame's event
    bool rendered_rec[2] = {false, false};
    cudaEvent_t prefetch_ev = nullptr;
    int2 *info_stage[2] = {nullptr, nullptr};  // pinned staging of the page table
    // realtime frames overlap: a frame culls on its own stream, from a copy
    // of the chebyshev values, while the previous frame still renders
    cudaStream_t cull_stream = nullptr;
    int *cheb_dev = nullptr;
    int frame_buf = 0;           // page-table staging buffer of the next frame
    // brick moves: two pinned staging lists, their device copies (nslots
    // items each) and the event after each list's upload
    GatherItem *gather_stage[2] = {nullptr, nullptr};
    GatherItem *gather_dev = nullptr;
    cudaEvent_t gathered[2] = {nullptr, nullptr};
    CullScratch cs;
    void *film = nullptr;
    size_t film_bytes = 0;
    hy_pager_stats stats{};
    // HY_PAGER_GATHERS: pool slot g (the coarse bricks, then the cache) sits
    // in gather texture g / gper, column block (g % gper) % gcols, row block
    // (g % gper) / gcols of the volume's atlas
    bool gathers = false;
    int gcols = 0, gper = 0;
    unsigned long long surf[hy::kMaxGatherTextures] = {};  // the textures' surfaces
    void texel_origin(int g, int &t, int &x0, int &y0) const {
        const int P = vol->P;
        t = g / gper;
        const int i = g % gper;
        x0 = (i % gcols) * P;
        y0 = (i / gcols) * P * P;
    }
};

namespace {

// film -> RGBA8 with the write_to rule (pixel_template.hpp:11-20)
__global__ void film_rgba_kernel(const float4 *__restrict__ film, int stride_f4, int n,
                                 uchar4 *__restrict__ out, uchar4 clear) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = film[size_t(i) * stride_f4 + 2];
    out[i] = v.w != 0.f ? make_uchar4(saturate_u8(v.x), saturate_u8(v.y), saturate_u8(v.z),
                                      saturate_u8(v.w))
                        : clear;
}

// Rewrites the device page table on the render stream from staging buffer
// `buf` (0 or 1); the buffer is reused only after its previous copy ran.
int upload_page_table(hy_pager *pg, int buf = 0) {
    hy_ctx *ctx = pg->ctx;
    hy_volume *v = pg->vol;
    HY_CUDA(ctx, cudaEventSynchronize(pg->staged[buf]));
    int2 *st = pg->info_stage[buf];
    for (int b = 0; b < v->nbricks; ++b) {
        const int slot = pg->page[b];
        const int id = slot >= 0 ? pg->reg_base + slot : (pg->coarse && v->cheb[b] == 0 ? b : -1);
        st[b] = make_int2(v->cheb[b], id);
    }
    HY_CUDA(ctx, cudaMemcpyAsync(v->info_dev, st, v->nbricks * sizeof(int2),
                                 cudaMemcpyHostToDevice, ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(pg->staged[buf], ctx->stream));
    return HY_OK;
}

// Upload bricks into slots on the copy stream; returns after queuing.
// Moves n bricks from the store into cache slots with one gather kernel on
// `stream`: the list goes through staging list `buf` (reused only after its
// previous upload ran), the kernel reads the mapped pinned store directly.
int move_bricks(hy_pager *pg, const int *bricks, const int *slots, int n, cudaStream_t stream,
                int buf) {
    if (n == 0) return HY_OK;
    hy_ctx *ctx = pg->ctx;
    hy_volume *v = pg->vol;
    if (n > pg->nslots) return hy_fail(ctx, HY_ERR_STATE, "pager: more moves than slots");
    HY_CUDA(ctx, cudaEventSynchronize(pg->gathered[buf]));
    GatherItem *items = pg->gather_stage[buf];
    for (int i = 0; i < n; ++i) {
        const long long off = pg->store->offset[bricks[i]];
        if (off < 0) return hy_fail(ctx, HY_ERR_INVALID, "pager: empty brick requested");
        if (off + (long long)v->slot_stride > (long long)pg->store->host_bytes || slots[i] < 0 ||
            slots[i] >= pg->nslots)
            return hy_fail(ctx, HY_ERR_STATE, "pager: brick move out of range");
        items[i] = GatherItem{off, slots[i], 0};
    }
    GatherItem *dev = pg->gather_dev + size_t(buf) * pg->nslots;
    HY_CUDA(ctx, cudaMemcpyAsync(dev, items, n * sizeof(GatherItem), cudaMemcpyHostToDevice,
                                 stream));
    HY_CUDA(ctx, cudaEventRecord(pg->gathered[buf], stream));
    if (pg->gathers) {
        GatherSurfaces gs;
        for (int t = 0; t < hy::kMaxGatherTextures; ++t)
            gs.s[t] = pg->surf[t] ? pg->surf[t] : pg->surf[0];
        fill_textures_kernel<<<n, 256, 0, stream>>>(pg->store->host_dev, dev, gs, v->P, pg->gper,
                                                     pg->gcols, pg->ncoarse);
    } else {
        gather_bricks_kernel<<<n, 256, 0, stream>>>(pg->store->host_dev, dev, v->pool, pg->ncoarse,
                                                    (long long)v->slot_stride);
    }
    HY_CUDA(ctx, cudaGetLastError());
    pg->stats.uploads += n;
    pg->stats.upload_bytes += (int64_t)n * (int64_t)pg->store->slot_stride;
    return HY_OK;
}

}  // namespace

namespace {
// A registry entry of a cache in gather textures: pool offset 0 (the one
// zero slot) and the slot's texel origin + 1 in the last two words,
// (texture << 16 | x0 + 1, y0 + 1), as the march reads them.
void set_texel_origin(const hy_pager *pg, RegEntry &r, int g) {
    int t, x0, y0;
    pg->texel_origin(g, t, x0, y0);
    r.offset = 0;
    r.pad_[0] = (t << 16) | (x0 + 1);
    r.pad_[1] = y0 + 1;
}
}  // namespace

extern "C" int hy_pager_create(hy_ctx *ctx, hy_store *store, const hy_pager_desc *desc,
                               hy_pager **out) {
    if (!ctx || !store || !desc || !out) return HY_ERR_INVALID;
    *out = nullptr;
    if (store->ctx != ctx) return hy_fail(ctx, HY_ERR_INVALID, "pager: store of another context");
    if (desc->slots <= 0) return hy_fail(ctx, HY_ERR_INVALID, "pager: slots must be > 0");
    if (desc->mode != HY_PAGER_LOSSLESS && desc->mode != HY_PAGER_REALTIME)
        return hy_fail(ctx, HY_ERR_INVALID, "pager: unknown mode");
    if (desc->eviction != HY_EVICT_LRU && desc->eviction != HY_EVICT_REFERENCE)
        return hy_fail(ctx, HY_ERR_INVALID, "pager: unknown eviction policy");
    if (desc->sampler != HY_PAGER_LOADS && desc->sampler != HY_PAGER_GATHERS)
        return hy_fail(ctx, HY_ERR_INVALID, "pager: unknown sampler");
    // (an even brick edge P: the fill writes texel pairs at multiples of P)
    if (desc->sampler == HY_PAGER_GATHERS &&
        (desc->mode != HY_PAGER_REALTIME || store->desc.dtype != HY_DTYPE_U8 ||
         store->desc.padding < 1 || (store->P & 1)))
        return hy_fail(ctx, HY_ERR_UNSUPPORTED,
                       "pager: gather textures hold a realtime cache of u8 bricks with an apron "
                       "and an even edge");
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    hy_pager *pg = new hy_pager();
    pg->ctx = ctx;
    pg->store = store;
    pg->desc = *desc;
    pg->nslots = desc->mode == HY_PAGER_LOSSLESS ? 2 * desc->slots : desc->slots;
    hy_volume *v = new hy_volume();
    pg->vol = v;
    int rc = hy_volume_init(ctx, &store->desc, v);
    auto fail = [&](int code) {
        hy_pager_destroy(pg);
        return code;
    };
    if (rc) return fail(rc);
    v->paged = true;
    v->cheb = store->cheb;
    v->mean = store->mean;
    v->nonempty = store->nonempty;
    v->resident = 0;
    v->reg_of_brick.assign(v->nbricks, -1);
    pg->coarse = desc->mode == HY_PAGER_REALTIME && store->coarse_level > 0;
    pg->ncoarse = pg->coarse ? store->ncoarse : 0;
    pg->reg_base = pg->coarse ? v->nbricks : 0;
    const int nreg = pg->reg_base + pg->nslots;
    const int ntotal = pg->ncoarse + pg->nslots;
    if (desc->sampler == HY_PAGER_GATHERS) {
        bool ok = false;
        int rows = 0;
        rc = hy_gather_layout(ctx, v->P, &ok, &pg->gcols, &rows);
        if (rc) return fail(rc);
        pg->gper = pg->gcols * rows;
        if (!ok || pg->gper <= 0 ||
            (long long)pg->gper * hy::kMaxGatherTextures < (long long)ntotal)
            return fail(hy_fail(ctx, HY_ERR_UNSUPPORTED,
                                "pager: this device's gather textures cannot hold the cache"));
        pg->gathers = true;
        v->paged_gather = true;
        // the textures, each exactly as large as its bricks need
        for (int first = 0; first < ntotal; first += pg->gper) {
            const int cnt = std::min(pg->gper, ntotal - first);
            const int ucols = std::min(pg->gcols, cnt), urows = (cnt + pg->gcols - 1) / pg->gcols;
            cudaArray_t arr = nullptr;
            unsigned long long tex = 0;
            unsigned long long sf = 0;
            rc = hy_gather_texture_create(ctx, size_t(ucols) * v->P,
                                          size_t(urows) * v->P * v->P, &arr, &tex, &sf);
            if (rc) return fail(rc);
            pg->surf[v->atlas.size()] = sf;
            v->atlas.push_back(arr);
            v->atlas_tex.push_back(tex);
        }
    }
    // with gathers the pool is one slot of zeros: every registry entry points
    // there, so no launch can read outside memory it owns
    v->pool_bytes = size_t(pg->gathers ? 1 : ntotal) * v->slot_stride;
    cudaError_t e = cudaMalloc(&v->pool, v->pool_bytes);
    if (e == cudaSuccess && pg->gathers) e = cudaMemset(v->pool, 0, v->pool_bytes);
    if (e == cudaSuccess) e = cudaMalloc(&v->info_dev, v->nbricks * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc(&v->reg_dev, nreg * sizeof(RegEntry));
    if (e == cudaSuccess) e = cudaMalloc(&v->mean_dev, v->nbricks * sizeof(float));
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaHostAlloc(reinterpret_cast<void **>(&pg->info_stage[i]), v->nbricks * sizeof(int2),
                          cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pg->marched[i], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pg->staged[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&pg->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pg->copied, cudaEventDisableTiming);
    // the cull runs while the previous frame's render grid still has blocks
    // waiting; the highest priority lets its few blocks go first
    int prio_low = 0, prio_high = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithPriority(&pg->cull_stream, cudaStreamNonBlocking, prio_high);
    if (e == cudaSuccess) e = cudaMalloc(&pg->cheb_dev, v->nbricks * sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemcpy(pg->cheb_dev, v->cheb.data(), v->nbricks * sizeof(int),
                       cudaMemcpyHostToDevice);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
        e = cudaHostAlloc(reinterpret_cast<void **>(&pg->gather_stage[i]),
                          pg->nslots * sizeof(GatherItem), cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaMalloc(&pg->gather_dev, 2 * pg->nslots * sizeof(GatherItem));
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&pg->gathered[i], cudaEventDisableTiming);
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&pg->rendered[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pg->prefetch_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return fail(hy_cuda_fail(ctx, e, "pager: allocation"));
    std::vector<RegEntry> reg(nreg);
    if (pg->coarse) {
        // LowestLevelBlock samplers (rt_block_paging.cc:141-188): fine brick
        // b = base * s + d reads its sub-box of coarse brick `base`
        const int sc = 1 << store->coarse_level;
        const int P = v->P, bs = store->desc.block_size, pad = store->desc.padding;
        const float kc = float(bs) / float(P) / float(sc);
        const float b0 = float(pad) / float(P);
        const int *cg = store->coarse_grid;
        for (int b = 0; b < v->nbricks; ++b) {
            const int x = b % v->grid[0], y = (b / v->grid[0]) % v->grid[1],
                      z = b / (v->grid[0] * v->grid[1]);
            const int cid = ((z / sc) * cg[1] + y / sc) * cg[0] + x / sc;
            reg[b] = RegEntry{kc, b0 + float(x % sc) * kc, b0 + float(y % sc) * kc,
                              b0 + float(z % sc) * kc, (long long)cid * (long long)v->slot_stride,
                              {0, 0}};
            if (pg->gathers) set_texel_origin(pg, reg[b], cid);
        }
        if (pg->gathers) {
            const int P = v->P;
            for (int c = 0; c < pg->ncoarse && e == cudaSuccess; ++c) {
                int t, x0, y0;
                pg->texel_origin(c, t, x0, y0);
                e = cudaMemcpy2DToArray(v->atlas[t], size_t(x0), size_t(y0),
                                        store->coarse.data() + size_t(c) * v->slot_stride,
                                        size_t(P), size_t(P), size_t(P) * P,
                                        cudaMemcpyHostToDevice);
            }
        } else {
            e = cudaMemcpyAsync(v->pool, store->coarse.data(), store->coarse.size(),
                                cudaMemcpyHostToDevice, ctx->stream);
        }
        if (e != cudaSuccess) return fail(hy_cuda_fail(ctx, e, "pager: coarse level upload"));
    }
    for (int s = 0; s < pg->nslots; ++s) {
        reg[pg->reg_base + s] =
            RegEntry{v->k, v->b, v->b, v->b,
                     (long long)(pg->ncoarse + s) * (long long)v->slot_stride, {0, 0}};
        if (pg->gathers) set_texel_origin(pg, reg[pg->reg_base + s], pg->ncoarse + s);
    }
    e = cudaMemcpyAsync(v->reg_dev, reg.data(), reg.size() * sizeof(RegEntry),
                        cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(v->mean_dev, v->mean.data(), v->nbricks * sizeof(float),
                            cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return fail(hy_cuda_fail(ctx, e, "pager: registry upload"));
    pg->page.assign(v->nbricks, -1);
    pg->owner.assign(pg->nslots, -1);
    pg->stamp.assign(pg->nslots, -1);
    rc = upload_page_table(pg);
    if (rc) return fail(rc);
    v->uploaded = true;
    *out = pg;
    return HY_OK;
}

extern "C" int hy_pager_destroy(hy_pager *pg) {
    if (!pg) return HY_OK;
    hy_ctx *ctx = pg->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (pg->copy) {
        cudaStreamSynchronize(pg->copy);
        cudaStreamDestroy(pg->copy);
    }
    if (pg->copied) cudaEventDestroy(pg->copied);
    if (pg->cull_stream) {
        cudaStreamSynchronize(pg->cull_stream);
        cudaStreamDestroy(pg->cull_stream);
    }
    if (pg->cheb_dev) cudaFree(pg->cheb_dev);
    for (int i = 0; i < 2; ++i)
        if (pg->gather_stage[i]) cudaFreeHost(pg->gather_stage[i]);
    if (pg->gather_dev) cudaFree(pg->gather_dev);
    for (int i = 0; i < 2; ++i)
        if (pg->gathered[i]) cudaEventDestroy(pg->gathered[i]);
    for (int i = 0; i < 2; ++i)
        if (pg->rendered[i]) cudaEventDestroy(pg->rendered[i]);
    if (pg->prefetch_ev) cudaEventDestroy(pg->prefetch_ev);
    for (int i = 0; i < 2; ++i) {
        if (pg->marched[i]) cudaEventDestroy(pg->marched[i]);
        if (pg->staged[i]) cudaEventDestroy(pg->staged[i]);
        if (pg->info_stage[i]) cudaFreeHost(pg->info_stage[i]);
    }
    if (pg->cs.ids) cudaFree(pg->cs.ids);
    if (pg->cs.d2) cudaFree(pg->cs.d2);
    if (pg->cs.count) cudaFree(pg->cs.count);
    if (pg->film) cudaFree(pg->film);
    for (auto sf : pg->surf)
        if (sf) cudaDestroySurfaceObject(cudaSurfaceObject_t(sf));
    if (pg->vol) {
        hy_volume *v = pg->vol;
        hy_volume_free_gather(v);
        if (v->pool) cudaFree(v->pool);
        if (v->info_dev) cudaFree(v->info_dev);
        if (v->reg_dev) cudaFree(v->reg_dev);
        if (v->mean_dev) cudaFree(v->mean_dev);
        delete v;
    }
    delete pg;
    return HY_OK;
}

// Cache size for a camera path: the most bricks any of the cameras sees
// (the GPU cull over the store's chebyshev thumbnail), with 10 % headroom
// for the bricks the next frames bring into view, within the byte budget
// and never more than the store holds.  The reference sizes its cache from
// a fixed mem_limit_mb alone (rt_block_paging.cc:230-236).
extern "C" int hy_pager_tune_slots(hy_ctx *ctx, const hy_store *store, const hy_camera *cams,
                                   int32_t ncams, int64_t budget_bytes, int32_t *slots_out,
                                   int32_t *visible_max_out) {
    if (!ctx || !store || !cams || ncams <= 0 || !slots_out) return HY_ERR_INVALID;
    if (store->ctx != ctx) return hy_fail(ctx, HY_ERR_INVALID, "tune: store of another context");
    if (budget_bytes < (int64_t)store->slot_stride)
        return hy_fail(ctx, HY_ERR_INVALID, "tune: the budget holds no brick");
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    hy_volume v;
    int rc = hy_volume_init(ctx, &store->desc, &v);
    if (rc) return rc;
    int *cheb_dev = nullptr;
    HY_CUDA(ctx, cudaMalloc(&cheb_dev, size_t(v.nbricks) * sizeof(int)));
    CullScratch cs;
    size_t most = 0;
    cudaError_t e = cudaMemcpyAsync(cheb_dev, store->cheb.data(), size_t(v.nbricks) * sizeof(int),
                                    cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) rc = hy_cuda_fail(ctx, e, "tune: chebyshev upload");
    for (int i = 0; i < ncams && rc == HY_OK; ++i) {
        hy_view view;
        rc = hy_camera_view(&v, &cams[i], &view);
        std::vector<int> ids;
        std::vector<float> d2;
        if (rc == HY_OK)
            rc = run_cull(ctx, &v, view, nullptr, -1, cs, ids, d2, nullptr, ctx->stream, cheb_dev);
        most = std::max(most, ids.size());
    }
    if (cs.ids) cudaFree(cs.ids);
    if (cs.d2) cudaFree(cs.d2);
    if (cs.count) cudaFree(cs.count);
    cudaFree(cheb_dev);
    if (rc) return rc;
    const long long budget = budget_bytes / (long long)store->slot_stride;
    long long want = (long long)(most + (most + 9) / 10);
    want = std::min(want, (long long)store->nonempty);
    want = std::min(want, budget);
    *slots_out = int32_t(std::max(want, 1ll));
    if (visible_max_out) *visible_max_out = int32_t(most);
    return HY_OK;
}

extern "C" int hy_pager_volume(hy_pager *pg, hy_volume **out) {
    if (!pg || !out) return HY_ERR_INVALID;
    *out = pg->vol;
    return HY_OK;
}

extern "C" int hy_pager_stats_get(const hy_pager *pg, hy_pager_stats *out) {
    if (!pg || !out) return HY_ERR_INVALID;
    *out = pg->stats;
    return HY_OK;
}

namespace {

// LosslessBlockPagingServer::start + next (lossless_block_paging.cc:116-174):
// visible bricks by distance to inverse(iet) * eye, in batches of
// desc.slots; batch k marches while batch k+1 uploads into the other half.
int render_lossless(hy_pager *pg, const hy_shader_params *p, const hy_camera *cam,
                    const hy_view &view, int W, int H, uint8_t *rgba_dev) {
    hy_ctx *ctx = pg->ctx;
    hy_volume *v = pg->vol;
    std::vector<int> ids;
    std::vector<float> d2;
    int rc = run_cull(ctx, v, view, nullptr, -1, pg->cs, ids, d2);
    if (rc) return rc;
    // order: distance of brick centres to cp = inverse(iet) * eye, ties by
    // index; inverse(iet) is the to_world matrix of hy_iso_lighting
    hy_shader_params tmp;
    std::memset(&tmp, 0, sizeof(tmp));
    rc = hy_iso_lighting(v, cam, &tmp);
    if (rc) return rc;
    const float *et = tmp.to_world;
    float cp[3];
    for (int r = 0; r < 3; ++r)
        cp[r] = et[r] * cam->position[0] + et[4 + r] * cam->position[1] +
                et[8 + r] * cam->position[2] + et[12 + r] * 1.f;
    std::vector<std::pair<float, int>> order(ids.size());
    for (size_t i = 0; i < ids.size(); ++i) {
        const int id = ids[i];
        const int x = id % v->grid[0], y = (id / v->grid[0]) % v->grid[1],
                  z = id / (v->grid[0] * v->grid[1]);
        const float dx = cp[0] - (float(x) + 0.5f), dy = cp[1] - (float(y) + 0.5f),
                    dz = cp[2] - (float(z) + 0.5f);
        order[i] = {std::sqrt(dx * dx + dy * dy + dz * dz), id};
    }
    std::sort(order.begin(), order.end());
    const int B = pg->desc.slots;
    const int nbatch = std::max(1, int((order.size() + B - 1) / B));
    const size_t need = size_t(W) * H * 64;
    if (need > pg->film_bytes) {
        if (pg->film) cudaFree(pg->film);
        pg->film = nullptr;
        pg->film_bytes = 0;
        HY_CUDA(ctx, cudaMalloc(&pg->film, need));
        pg->film_bytes = need;
    }
    ShadeArgs a;
    rc = hy_fill_args(ctx, v, p, &view, W, H, &a);
    if (rc) return rc;
    a.film = pg->film;
    // samples of the whole frame: the counter is cleared once, the passes add
    a.count = p->count_samples ? 1 : 0;
    if (a.count)
        HY_CUDA(ctx, cudaMemsetAsync(ctx->counter_dev, 0, sizeof(unsigned long long), ctx->stream));
    std::vector<int> bricks, slots;
    auto queue_batch = [&](int k) -> int {
        bricks.clear();
        slots.clear();
        const int half = k & 1;
        for (int j = k * B; j < std::min<int>((k + 1) * B, int(order.size())); ++j) {
            bricks.push_back(order[j].second);
            slots.push_back(half * B + (j - k * B));
        }
        // this half of the cache is free once the pass of batch k-2 has run
        HY_CUDA(ctx, cudaStreamWaitEvent(pg->copy, pg->marched[half], 0));
        int r = move_bricks(pg, bricks.data(), slots.data(), int(bricks.size()), pg->copy, half);
        if (r) return r;
        HY_CUDA(ctx, cudaEventRecord(pg->copied, pg->copy));
        return HY_OK;
    };
    HY_CUDA(ctx, cudaEventRecord(pg->marched[0], ctx->stream));
    HY_CUDA(ctx, cudaEventRecord(pg->marched[1], ctx->stream));
    std::vector<int> prev;
    rc = queue_batch(0);
    if (rc) return rc;
    for (int k = 0; k < nbatch; ++k) {
        const std::vector<int> cur = bricks, cur_slots = slots;
        HY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, pg->copied, 0));
        // page table: only batch k present (lossless_block_paging.cc:147, 163)
        for (int b : prev) pg->page[b] = -1;
        for (size_t i = 0; i < cur.size(); ++i) pg->page[cur[i]] = cur_slots[i];
        rc = upload_page_table(pg, k & 1);
        if (rc) return rc;
        rc = hy_launch_pass(ctx, a, k == 0 ? HY_PASS_RAY_EMIT : HY_PASS_RAY_MARCH, false);
        if (rc) return rc;
        HY_CUDA(ctx, cudaEventRecord(pg->marched[k & 1], ctx->stream));
        ++pg->stats.passes;
        prev = cur;
        if (k + 1 < nbatch) {
            rc = queue_batch(k + 1);
            if (rc) return rc;
        }
    }
    for (int b : prev) pg->page[b] = -1;
    uchar4 clear = make_uchar4(a.clear_u8[0], a.clear_u8[1], a.clear_u8[2], 0);
    const int stride = (p->shader == HY_SHADER_BLOCKS || p->shader == HY_SHADER_PAGING) ? 3 : 4;
    film_rgba_kernel<<<(W * H + 255) / 256, 256, 0, ctx->stream>>>(
        static_cast<const float4 *>(pg->film), stride, W * H, reinterpret_cast<uchar4 *>(rgba_dev),
        clear);
    HY_CUDA(ctx, cudaGetLastError());
    pg->stats.visible = int64_t(order.size());
    v->resident = 0;
    return HY_OK;
}

// RtBlockPagingServer::update (rt_block_paging.cc:296-326) and the brick
// arrival handler (rt_block_paging.cc:246-291): the nearest `slots` visible
// bricks are required; missing ones (nearest first, at most
// max_uploads_per_frame) go to never-used slots, then to slots of bricks that
// are no longer required, chosen by the eviction policy:
//  HY_EVICT_LRU        the least recently visible brick first (a slot's
//                      stamp is the last frame its brick was visible; ties by
//                      brick index), so a brick seen a few frames ago
//                      survives bricks that left the view long before;
//  HY_EVICT_REFERENCE  the highest brick index first (the reference's
//                      redundant set, an ordered std::set popped from the end).
// The whole frame's plan is checked before any page-table entry changes, so
// a refused move leaves the cache as it was; then one frame.
int render_realtime(hy_pager *pg, const hy_shader_params *p, const hy_view &view, int W, int H,
                    uint8_t *rgba_dev) {
    hy_ctx *ctx = pg->ctx;
    hy_volume *v = pg->vol;
    std::vector<int> req, visible;
    std::vector<float> d2;
    // while prefetching, `reserve` slots stay out of the required set (the
    // nearest visible bricks) to serve as the next prefetch's spares
    int rc = run_cull(ctx, v, view, nullptr, pg->nslots - pg->reserve, pg->cs, req, d2, &visible,
                      pg->cull_stream, pg->cheb_dev);
    if (rc) return rc;
    const int64_t frame = pg->stats.frames;
    // bricks a prefetch moved in enter the page table now (the render
    // stream waits for their copies before the page table is uploaded)
    const bool had_arrivals = !pg->arrived.empty();
    for (auto &a : pg->arrived) {
        pg->page[a.first] = a.second;
        pg->owner[a.second] = a.first;
        pg->stamp[a.second] = frame;
    }
    const int64_t accepted = int64_t(pg->arrived.size());
    pg->arrived.clear();
    std::vector<char> required(v->nbricks, 0);
    for (int b : req) required[b] = 1;
    // visible resident bricks are used this frame
    for (int b : visible)
        if (pg->page[b] >= 0) pg->stamp[pg->page[b]] = frame;
    std::vector<std::pair<float, int>> missing;
    int64_t hits = 0;
    for (size_t i = 0; i < req.size(); ++i)
        if (pg->page[req[i]] < 0) missing.push_back({d2[i], req[i]});
        else ++hits;
    std::sort(missing.begin(), missing.end());
    // eviction candidates, the next victim at the back
    std::vector<std::pair<int64_t, int>> victims;  // (key, slot)
    for (int s = 0; s < pg->nslots; ++s) {
        const int b = pg->owner[s];
        if (b < 0 || required[b]) continue;
        if (pg->desc.eviction == HY_EVICT_REFERENCE)
            victims.push_back({int64_t(b), s});  // highest brick index last
        else
            victims.push_back({-(pg->stamp[s] * int64_t(v->nbricks) + b), s});  // oldest last
    }
    std::sort(victims.begin(), victims.end());
    const int budget = pg->desc.max_uploads_per_frame > 0 ? pg->desc.max_uploads_per_frame
                                                           : int(missing.size());
    std::vector<int> move_b, move_s, evicted;
    int next_free = pg->next_free;
    std::vector<int> spare = pg->spare;
    for (int i = 0; i < int(missing.size()) && int(move_b.size()) < budget; ++i) {
        const int b = missing[i].second;
        int slot;
        if (next_free < pg->nslots) {
            slot = next_free++;
        } else if (!spare.empty()) {
            slot = spare.back();
            spare.pop_back();
        } else if (!victims.empty()) {
            slot = victims.back().second;
            victims.pop_back();
            evicted.push_back(pg->owner[slot]);
        } else {
            break;  // no slot: the brick stays absent this frame
        }
        move_b.push_back(b);
        move_s.push_back(slot);
    }
    for (size_t i = 0; i < move_b.size(); ++i) {
        const long long off = pg->store->offset[move_b[i]];
        if (off < 0 || off + (long long)v->slot_stride > (long long)pg->store->host_bytes)
            return hy_fail(ctx, HY_ERR_STATE, "pager: a planned brick is not in the store");
    }
    // commit the plan
    pg->stats.hits += hits;
    pg->stats.misses += int64_t(missing.size());
    pg->next_free = next_free;
    pg->spare = spare;
    for (int old : evicted) {
        pg->page[old] = -1;
        ++pg->stats.evictions;
    }
    for (size_t i = 0; i < move_b.size(); ++i) {
        pg->owner[move_s[i]] = move_b[i];
        pg->page[move_b[i]] = move_s[i];
        pg->stamp[move_s[i]] = frame;
    }
    // prefetching: the next prefetch needs slots that this frame's page table
    // does not reference; as many as this frame brought in (moved plus
    // arrived) are evicted now, in the policy's order, among the bricks this
    // frame does not require
    if (pg->prefetching) {
        // the reserve follows the frames' turnover (twice the bricks this
        // frame brought in, 16 .. slots / 8)
        const int64_t turnover = int64_t(move_b.size()) + accepted;
        pg->reserve = int(std::min<int64_t>(std::max<int64_t>(2 * turnover, 16),
                                            std::max(pg->nslots / 8, 1)));
        const int64_t want = std::min<int64_t>(pg->reserve, int64_t(pg->nslots - int(req.size())));
        while (int64_t(pg->spare.size()) < want && !victims.empty()) {
            const int s = victims.back().second;
            victims.pop_back();
            if (pg->owner[s] < 0) continue;
            pg->page[pg->owner[s]] = -1;
            pg->owner[s] = -1;
            pg->spare.push_back(s);
            ++pg->stats.evictions;
        }
    }
    // one gather kernel on the render stream moves every brick of the frame:
    // it runs after the previous frame's render, so reused slots are free
    // after the prefetch's copies: its bricks are in this frame's page table,
    // and its move list shares the device staging list with this frame's
    if (had_arrivals) HY_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, pg->prefetch_ev, 0));
    rc = move_bricks(pg, move_b.data(), move_s.data(), int(move_b.size()), ctx->stream,
                     pg->frame_buf);
    if (rc) return rc;
    rc = upload_page_table(pg, pg->frame_buf);
    if (rc) return rc;
    pg->frame_buf ^= 1;
    int resident = 0;
    for (int s = 0; s < pg->nslots; ++s) resident += pg->owner[s] >= 0;
    v->resident = resident;
    pg->stats.visible = int64_t(req.size());
    int64_t fallback = 0;
    if (pg->coarse)
        for (int b : visible) fallback += pg->page[b] < 0;
    pg->stats.fallback = fallback;
    ++pg->stats.passes;
    rc = hy_render_device(ctx, v, p, &view, W, H, rgba_dev, nullptr, nullptr);
    if (rc) return rc;
    pg->rendered_i ^= 1;
    HY_CUDA(ctx, cudaEventRecord(pg->rendered[pg->rendered_i], ctx->stream));
    pg->rendered_rec[pg->rendered_i] = true;
    return HY_OK;
}

// hy_pager_prefetch: the next camera's required bricks that are not resident,
// nearest first (within max_uploads_per_frame), moved on the copy stream
// into never-used or spare slots.  A spare slot left the page table at the
// last frame, so only the frame before may still read it: the copy stream
// waits for that frame's render, not for the last one.
int prefetch_realtime(hy_pager *pg, const hy_view &view) {
    hy_ctx *ctx = pg->ctx;
    hy_volume *v = pg->vol;
    pg->prefetching = true;
    std::vector<int> req;
    std::vector<float> d2;
    if (pg->reserve == 0) pg->reserve = std::min(16, std::max(pg->nslots / 8, 1));
    int rc = run_cull(ctx, v, view, nullptr, pg->nslots - pg->reserve, pg->cs, req, d2, nullptr,
                      pg->cull_stream, pg->cheb_dev);
    if (rc) return rc;
    std::vector<char> coming(v->nbricks, 0);
    for (auto &a : pg->arrived) coming[a.first] = 1;
    std::vector<std::pair<float, int>> missing;
    for (size_t i = 0; i < req.size(); ++i)
        if (pg->page[req[i]] < 0 && !coming[req[i]]) missing.push_back({d2[i], req[i]});
    std::sort(missing.begin(), missing.end());
    const int budget = pg->desc.max_uploads_per_frame > 0 ? pg->desc.max_uploads_per_frame
                                                           : int(missing.size());
    std::vector<int> move_b, move_s;
    int next_free = pg->next_free;
    size_t nspare = pg->spare.size();
    for (int i = 0; i < int(missing.size()) && int(move_b.size()) < budget; ++i) {
        int slot;
        if (next_free < pg->nslots) {
            slot = next_free++;
        } else if (nspare > 0) {
            slot = pg->spare[--nspare];
        } else {
            break;
        }
        const long long off = pg->store->offset[missing[i].second];
        if (off < 0 || off + (long long)v->slot_stride > (long long)pg->store->host_bytes)
            return hy_fail(ctx, HY_ERR_STATE, "pager: a planned brick is not in the store");
        move_b.push_back(missing[i].second);
        move_s.push_back(slot);
    }
    if (move_b.empty()) return HY_OK;
    // the frame before the last may still read a spare slot's old brick, and
    // its moves used the device move list this prefetch rewrites
    const int prev = pg->rendered_i ^ 1;
    if (pg->rendered_rec[prev]) HY_CUDA(ctx, cudaStreamWaitEvent(pg->copy, pg->rendered[prev], 0));
    rc = move_bricks(pg, move_b.data(), move_s.data(), int(move_b.size()), pg->copy,
                     pg->frame_buf);
    if (rc) return rc;
    HY_CUDA(ctx, cudaEventRecord(pg->prefetch_ev, pg->copy));
    pg->next_free = next_free;
    pg->spare.resize(nspare);
    for (size_t i = 0; i < move_b.size(); ++i) pg->arrived.push_back({move_b[i], move_s[i]});
    pg->stats.prefetched += int64_t(move_b.size());
    return HY_OK;
}

}  // namespace

extern "C" int hy_pager_render(hy_pager *pg, const hy_shader_params *p, const hy_camera *cam,
                               int32_t W, int32_t H, uint8_t *rgba_dev) {
    if (!pg || !p || !cam || !rgba_dev) return HY_ERR_INVALID;
    hy_ctx *ctx = pg->ctx;
    if (!hy_aligned(rgba_dev, 4)) return hy_fail(ctx, HY_ERR_INVALID, "pager: misaligned output (4-byte)");
    if (p->composite) return hy_fail(ctx, HY_ERR_UNSUPPORTED, "pager: composite not supported");
    if (pg->gathers && !(p->shader == HY_SHADER_BLOCKS || p->shader == HY_SHADER_PAGING ||
                         (p->shader == HY_SHADER_VOLUME && p->mode == HY_VOLUME_DEFAULT)))
        return hy_fail(ctx, HY_ERR_UNSUPPORTED,
                       "pager: a cache in gather textures serves the Volume shader in Default "
                       "mode and the Blocks and Paging shaders (HY_PAGER_LOADS serves all)");
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    hy_view view;
    int rc = hy_camera_view(pg->vol, cam, &view);
    if (rc) return rc;
    ++pg->stats.frames;
    hy_shader_params q = *p;
    q.lowest_blkcnt = pg->reg_base;
    if (pg->desc.mode == HY_PAGER_LOSSLESS)
        return render_lossless(pg, &q, cam, view, W, H, rgba_dev);
    return render_realtime(pg, &q, view, W, H, rgba_dev);
}

extern "C" int hy_pager_prefetch(hy_pager *pg, const hy_camera *next_cam) {
    if (!pg || !next_cam) return HY_ERR_INVALID;
    hy_ctx *ctx = pg->ctx;
    if (pg->desc.mode != HY_PAGER_REALTIME)
        return hy_fail(ctx, HY_ERR_UNSUPPORTED, "pager: prefetch needs the realtime policy");
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    hy_view view;
    int rc = hy_camera_view(pg->vol, next_cam, &view);
    if (rc) return rc;
    return prefetch_realtime(pg, view);
}

extern "C" int hy_pager_render_host(hy_pager *pg, const hy_shader_params *p, const hy_camera *cam,
                                    int32_t W, int32_t H, uint8_t *rgba_host) {
    if (!pg || !p || !cam || !rgba_host || W <= 0 || H <= 0) return HY_ERR_INVALID;
    hy_ctx *ctx = pg->ctx;
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    void *dev = nullptr;
    const size_t bytes = size_t(W) * H * 4;
    int rc = hy_stage(ctx, bytes, &dev);
    if (rc) return rc;
    rc = hy_pager_render(pg, p, cam, W, H, static_cast<uint8_t *>(dev));
    if (rc) return rc;
    HY_CUDA(ctx, cudaMemcpyAsync(rgba_host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HY_OK;
}

extern "C" int hy_pager_present(const hy_pager *pg, uint8_t *mask) {
    if (!pg || !mask) return HY_ERR_INVALID;
    for (int b = 0; b < pg->vol->nbricks; ++b) mask[b] = pg->page[b] >= 0 ? 1 : 0;
    return HY_OK;
}
