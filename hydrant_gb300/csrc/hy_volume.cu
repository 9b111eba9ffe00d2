// hy_volume.cu -- brick pool, page table and thumbnails on the device.
//
// Replaces, for volumes that stay resident, what the reference does per
// frame on the host: decode bricks and upload one 3-D texture per brick,
// write vaddr[brick] = slot and re-upload the registry
// (src/slave/paging/lossless_block_paging.cc:137-174).  Layout in HBM:
//   pool  : resident bricks, (bs+2*pad)^3 voxels each, x fastest, slots
//           256-byte aligned, u8 (1 B/voxel) or f32 (4 B/voxel);
//   info  : int2 per brick {chebyshev distance, registry id or -1}, the
//           chebyshev thumbnail and the vaddr texture read together
//           (volume_shader.cu:45-50);
//   reg   : RegEntry per registry id {k, b, slot offset} (block_paging.hpp:24-36);
//   mean  : float per brick (the "mean" thumbnail read by blocks_shader.cu:33).
// The dataset definition this builds: the apron of a brick holds the
// neighbouring voxels, clamped at the volume border; a brick is non-empty if
// any voxel of core or apron is non-zero; chebyshev = L-infinity distance in
// bricks to the nearest non-empty brick (0 = non-empty, max(grid) if there is
// none); mean = mean of the normalised core voxels.

#include <algorithm>
#include <cstring>
#include <mutex>

#include "hy_internal.h"

namespace {

template <typename T>
__global__ void brick_stats_kernel(const T *__restrict__ raw, int dx, int dy, int dz, int bs,
                                   int pad, int gx, int gy, unsigned int *__restrict__ nonempty,
                                   double *__restrict__ core_sum) {
    const int bid = blockIdx.x;
    const int bx = bid % gx, by = (bid / gx) % gy, bz = bid / (gx * gy);
    const int P = bs + 2 * pad;
    const long long P3 = (long long)P * P * P;
    unsigned int any = 0;
    double sum = 0.0;
    for (long long i = threadIdx.x; i < P3; i += blockDim.x) {
        int x = int(i % P), y = int((i / P) % P), z = int(i / ((long long)P * P));
        int X = min(max(bx * bs + x - pad, 0), dx - 1);
        int Y = min(max(by * bs + y - pad, 0), dy - 1);
        int Z = min(max(bz * bs + z - pad, 0), dz - 1);
        T v = raw[((long long)Z * dy + Y) * dx + X];
        if (v != T(0)) any = 1;
        bool core = x >= pad && x < pad + bs && y >= pad && y < pad + bs && z >= pad && z < pad + bs;
        if (core) sum += double(v);
    }
    // block reduction
    __shared__ double ssum[32];
    __shared__ unsigned int sany[32];
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        any |= __shfl_down_sync(0xffffffffu, any, o);
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        ssum[warp] = sum;
        sany[warp] = any;
    }
    __syncthreads();
    if (warp == 0) {
        int nw = blockDim.x >> 5;
        sum = lane < nw ? ssum[lane] : 0.0;
        any = lane < nw ? sany[lane] : 0u;
        for (int o = 16; o > 0; o >>= 1) {
            sum += __shfl_down_sync(0xffffffffu, sum, o);
            any |= __shfl_down_sync(0xffffffffu, any, o);
        }
        if (lane == 0) {
            nonempty[bid] = any;
            core_sum[bid] = sum;
        }
    }
}

template <typename T>
__global__ void brick_fill_kernel(const T *__restrict__ raw, int dx, int dy, int dz, int bs,
                                  int pad, int gx, int gy, const int *__restrict__ slot_brick,
                                  unsigned char *__restrict__ pool, long long slot_stride,
                                  int slot0) {
    const int slot = slot0 + blockIdx.y;
    const int bid = slot_brick[slot];
    const int bx = bid % gx, by = (bid / gx) % gy, bz = bid / (gx * gy);
    const int P = bs + 2 * pad;
    const long long P3 = (long long)P * P * P;
    T *dst = reinterpret_cast<T *>(pool + (long long)slot * slot_stride);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < P3;
         i += (long long)gridDim.x * blockDim.x) {
        int x = int(i % P), y = int((i / P) % P), z = int(i / ((long long)P * P));
        int X = min(max(bx * bs + x - pad, 0), dx - 1);
        int Y = min(max(by * bs + y - pad, 0), dy - 1);
        int Z = min(max(bz * bs + z - pad, 0), dz - 1);
        dst[i] = raw[((long long)Z * dy + Y) * dx + X];
    }
}

// Chebyshev distance transform over the brick grid by 26-neighbour dilation.
void chebyshev_transform(const std::vector<unsigned int> &nonempty, const int g[3],
                         std::vector<int> &out) {
    const int n = g[0] * g[1] * g[2];
    const int cap = std::max(g[0], std::max(g[1], g[2]));
    out.assign(n, -1);
    for (int i = 0; i < n; ++i)
        if (nonempty[i]) out[i] = 0;
    std::vector<int> next;
    for (int r = 1; r <= cap; ++r) {
        next = out;
        bool changed = false;
        for (int z = 0; z < g[2]; ++z)
            for (int y = 0; y < g[1]; ++y)
                for (int x = 0; x < g[0]; ++x) {
                    int id = (z * g[1] + y) * g[0] + x;
                    if (out[id] >= 0) continue;
                    for (int k = 0; k < 27; ++k) {
                        int X = x + k % 3 - 1, Y = y + (k / 3) % 3 - 1, Z = z + k / 9 - 1;
                        if (X < 0 || Y < 0 || Z < 0 || X >= g[0] || Y >= g[1] || Z >= g[2])
                            continue;
                        if (out[(Z * g[1] + Y) * g[0] + X] == r - 1) {
                            next[id] = r;
                            changed = true;
                            break;
                        }
                    }
                }
        out.swap(next);
        if (!changed) break;
    }
    for (int i = 0; i < n; ++i)
        if (out[i] < 0) out[i] = cap;
}

// ---- gather textures ---------------------------------------------------------
//
// Every resident brick of a u8 volume with an apron is also placed in a 2-D
// u8 texture made for gather: its P slices stacked as P x P tiles in one
// column of texels (slice z at rows y0 + z * P).  The interior sampler then
// fetches the eight taps of a trilinear footprint with two gathers (slices
// z and z + 1), each returning the 2x2 texels at rows y, y + 1 and columns
// x, x + 1 as floats, normalised by the texture unit.  The coordinates are
// whole texel edges (x + 1, y + 1 with x, y integral), so the footprint the
// hardware picks is exactly (x, y) .. (x + 1, y + 1).  Bricks with P^2 rows
// taller than a gather texture allows keep the plain loads.

__global__ void gather_check_kernel(cudaTextureObject_t t, unsigned int *bad) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= 255) return;
    // row 0 holds u = column, row 1 holds 255 - column
    const float4 g = hy::gather_r((unsigned long long)t, float(x) + 1.f, 1.f);
    const float ew = __fdiv_rn(float(x), 255.f), ez = __fdiv_rn(float(x + 1), 255.f);
    const float ex = __fdiv_rn(float(255 - x), 255.f), ey = __fdiv_rn(float(254 - x), 255.f);
    if (__float_as_uint(g.w) != __float_as_uint(ew) || __float_as_uint(g.z) != __float_as_uint(ez) ||
        __float_as_uint(g.x) != __float_as_uint(ex) || __float_as_uint(g.y) != __float_as_uint(ey))
        atomicAdd(bad, 1u);
}

cudaTextureObject_t make_gather_texture(cudaArray_t arr, cudaError_t *err) {
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeNormalizedFloat;
    td.normalizedCoords = 0;
    cudaTextureObject_t t = 0;
    *err = cudaCreateTextureObject(&t, &rd, &td, nullptr);
    return t;
}

// Once per device: the gather order and the u8 -> u / 255 normalisation
// of the texture unit equal what the sampler assumes (for all 256 values,
// against IEEE division).  A device that fails renders with the plain loads.
constexpr int kMaxCheckDevices = 64;
std::mutex g_gather_mu;
int g_gather_ok[kMaxCheckDevices] = {};  // 0 unknown, 1 passed, -1 failed

int gather_check(hy_ctx *ctx, bool *ok) {
    *ok = false;
    if (ctx->device < 0 || ctx->device >= kMaxCheckDevices) return HY_OK;
    std::lock_guard<std::mutex> lock(g_gather_mu);
    if (g_gather_ok[ctx->device] == 0) {
        cudaChannelFormatDesc cd = cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindUnsigned);
        cudaArray_t arr = nullptr;
        unsigned int *bad = nullptr;
        cudaTextureObject_t t = 0;
        unsigned char host[2 * 256];
        for (int c = 0; c < 256; ++c) {
            host[c] = (unsigned char)c;
            host[256 + c] = (unsigned char)(255 - c);
        }
        unsigned int nbad = 1;
        cudaError_t e = cudaMallocArray(&arr, &cd, 256, 2, cudaArrayTextureGather);
        if (e == cudaSuccess)
            e = cudaMemcpy2DToArrayAsync(arr, 0, 0, host, 256, 256, 2, cudaMemcpyHostToDevice,
                                         ctx->stream);
        if (e == cudaSuccess) t = make_gather_texture(arr, &e);
        if (e == cudaSuccess) e = cudaMalloc(&bad, sizeof(unsigned int));
        if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(unsigned int), ctx->stream);
        if (e == cudaSuccess) {
            gather_check_kernel<<<1, 256, 0, ctx->stream>>>(t, bad);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&nbad, bad, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (t) cudaDestroyTextureObject(t);
        if (arr) cudaFreeArray(arr);
        if (bad) cudaFree(bad);
        if (e != cudaSuccess) return hy_cuda_fail(ctx, e, "volume: gather texture check");
        g_gather_ok[ctx->device] = nbad == 0 ? 1 : -1;
    }
    *ok = g_gather_ok[ctx->device] == 1;
    return HY_OK;
}

void free_gather(hy_volume *v) {
    for (auto t : v->atlas_tex) cudaDestroyTextureObject(cudaTextureObject_t(t));
    for (auto a : v->atlas) cudaFreeArray(a);
    if (v->tex_dev) cudaFree(v->tex_dev);
    if (v->info4_dev) cudaFree(v->info4_dev);
    v->atlas_tex.clear();
    v->atlas.clear();
    v->tex_dev = nullptr;
    v->info4_dev = nullptr;
}

int build_gather(hy_volume *vol) {
    hy_ctx *ctx = vol->ctx;
    const int P = vol->P;
    if (vol->desc.dtype != HY_DTYPE_U8 || vol->desc.padding < 1 || vol->resident <= 0) return HY_OK;
    int gw = 0, gh = 0;
    HY_CUDA(ctx, cudaDeviceGetAttribute(&gw, cudaDevAttrMaxTexture2DGatherWidth, ctx->device));
    HY_CUDA(ctx, cudaDeviceGetAttribute(&gh, cudaDevAttrMaxTexture2DGatherHeight, ctx->device));
    const long long brick_rows = (long long)P * P;
    if (P > gw || brick_rows > gh) return HY_OK;  // too tall for a gather texture
    bool ok = false;
    int rc = gather_check(ctx, &ok);
    if (rc || !ok) return rc;
    const int cols = gw / P, rowblocks = int(gh / brick_rows), per = cols * rowblocks;
    const int n = vol->resident;
    if ((long long)per * hy::kResidentGatherTextures < n) return HY_OK;  // more than two textures hold
    std::vector<hy::TexEntry> table(n);
    cudaChannelFormatDesc cd = cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindUnsigned);
    for (int first = 0; first < n; first += per) {
        const int cnt = std::min(per, n - first);
        const int ucols = std::min(cols, cnt), urows = (cnt + cols - 1) / cols;
        cudaArray_t arr = nullptr;
        cudaError_t e = cudaMallocArray(&arr, &cd, size_t(ucols) * P, size_t(urows) * brick_rows,
                                        cudaArrayTextureGather);
        if (e != cudaSuccess) {
            free_gather(vol);
            return hy_cuda_fail(ctx, e, "volume: gather texture allocation");
        }
        vol->atlas.push_back(arr);
        cudaTextureObject_t t = make_gather_texture(arr, &e);
        if (e != cudaSuccess) {
            free_gather(vol);
            return hy_cuda_fail(ctx, e, "volume: gather texture object");
        }
        vol->atlas_tex.push_back((unsigned long long)t);
        for (int i = 0; i < cnt; ++i) {
            const int slot = first + i, cx = i % cols, ry = i / cols;
            e = cudaMemcpy2DToArrayAsync(arr, size_t(cx) * P, size_t(ry) * brick_rows,
                                         vol->pool + size_t(slot) * vol->slot_stride, P, P,
                                         brick_rows, cudaMemcpyDeviceToDevice, ctx->stream);
            if (e != cudaSuccess) {
                free_gather(vol);
                return hy_cuda_fail(ctx, e, "volume: gather texture fill");
            }
            table[slot] = hy::TexEntry{float(cx * P), float(ry * brick_rows),
                                       int(vol->atlas_tex.size()) - 1, 0};
        }
    }
    // the page table with each resident brick's texel origin beside it
    std::vector<int4> info4(vol->nbricks);
    for (int b = 0; b < vol->nbricks; ++b) {
        const int reg = vol->reg_of_brick[b];
        int4 q = make_int4(vol->cheb[b], reg, 0, 0);
        if (reg >= 0) {
            // texel origin + 1 as floats (the sampler's footprint column and
            // row offsets), the texture in the sign of the row (>= 1)
            const float x1 = table[reg].x0 + 1.f, y1 = table[reg].y0 + 1.f;
            const float ys = table[reg].which ? -y1 : y1;
            std::memcpy(&q.z, &x1, 4);
            std::memcpy(&q.w, &ys, 4);
        }
        info4[b] = q;
    }
    cudaError_t e = cudaMalloc(&vol->tex_dev, size_t(n) * sizeof(hy::TexEntry));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(vol->tex_dev, table.data(), size_t(n) * sizeof(hy::TexEntry),
                            cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMalloc(&vol->info4_dev, size_t(vol->nbricks) * sizeof(int4));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(vol->info4_dev, info4.data(), size_t(vol->nbricks) * sizeof(int4),
                            cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        free_gather(vol);
        return hy_cuda_fail(ctx, e, "volume: gather table");
    }
    return HY_OK;
}

void free_volume_device(hy_volume *v) {
    free_gather(v);
    if (v->pool) cudaFree(v->pool);
    if (v->info_dev) cudaFree(v->info_dev);
    if (v->reg_dev) cudaFree(v->reg_dev);
    if (v->mean_dev) cudaFree(v->mean_dev);
    v->pool = nullptr;
    v->info_dev = nullptr;
    v->reg_dev = nullptr;
    v->mean_dev = nullptr;
    v->pool_bytes = 0;
    v->uploaded = false;
}

template <typename T>
int upload_impl(hy_volume *vol, const void *host) {
    hy_ctx *ctx = vol->ctx;
    const hy_volume_desc &d = vol->desc;
    const size_t nvox = size_t(d.dim[0]) * d.dim[1] * d.dim[2];
    T *raw = nullptr;
    unsigned int *ne_dev = nullptr;
    double *sum_dev = nullptr;
    int *slot_brick_dev = nullptr;
    auto cleanup = [&] {
        if (raw) cudaFree(raw);
        if (ne_dev) cudaFree(ne_dev);
        if (sum_dev) cudaFree(sum_dev);
        if (slot_brick_dev) cudaFree(slot_brick_dev);
    };
#define HY_UP(call)                                            \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) {                               \
            cleanup();                                         \
            return hy_cuda_fail(ctx, e_, #call);               \
        }                                                      \
    } while (0)
    free_volume_device(vol);
    HY_UP(cudaMalloc(&raw, nvox * sizeof(T)));
    HY_UP(cudaMemcpyAsync(raw, host, nvox * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    const int nb = vol->nbricks;
    HY_UP(cudaMalloc(&ne_dev, nb * sizeof(unsigned int)));
    HY_UP(cudaMalloc(&sum_dev, nb * sizeof(double)));
    brick_stats_kernel<T><<<nb, 256, 0, ctx->stream>>>(raw, d.dim[0], d.dim[1], d.dim[2],
                                                       d.block_size, d.padding, vol->grid[0],
                                                       vol->grid[1], ne_dev, sum_dev);
    HY_UP(cudaGetLastError());
    std::vector<unsigned int> ne(nb);
    std::vector<double> sums(nb);
    HY_UP(cudaMemcpyAsync(ne.data(), ne_dev, nb * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                          ctx->stream));
    HY_UP(cudaMemcpyAsync(sums.data(), sum_dev, nb * sizeof(double), cudaMemcpyDeviceToHost,
                          ctx->stream));
    HY_UP(cudaStreamSynchronize(ctx->stream));

    chebyshev_transform(ne, vol->grid, vol->cheb);
    const double ncore = double(d.block_size) * d.block_size * d.block_size;
    vol->mean.resize(nb);
    for (int i = 0; i < nb; ++i)
        vol->mean[i] = (sizeof(T) == 1) ? float(sums[i] / 255.0 / ncore) : float(sums[i] / ncore);
    std::vector<int> slot_brick;
    vol->reg_of_brick.assign(nb, -1);
    for (int i = 0; i < nb; ++i)
        if (ne[i]) {
            vol->reg_of_brick[i] = int(slot_brick.size());
            slot_brick.push_back(i);
        }
    vol->nonempty = int(slot_brick.size());
    vol->resident = vol->nonempty;
    const int nslots = std::max(vol->resident, 1);
    vol->pool_bytes = size_t(nslots) * vol->slot_stride;
    HY_UP(cudaMalloc(&vol->pool, vol->pool_bytes));
    HY_UP(cudaMemsetAsync(vol->pool, 0, vol->pool_bytes, ctx->stream));
    if (vol->resident > 0) {
        HY_UP(cudaMalloc(&slot_brick_dev, slot_brick.size() * sizeof(int)));
        HY_UP(cudaMemcpyAsync(slot_brick_dev, slot_brick.data(), slot_brick.size() * sizeof(int),
                              cudaMemcpyHostToDevice, ctx->stream));
        const long long P3 = (long long)vol->P * vol->P * vol->P;
        for (int s0 = 0; s0 < vol->resident; s0 += 65535) {
            const int n = std::min(65535, vol->resident - s0);
            dim3 grid(unsigned((P3 + 255) / 256 < 512 ? (P3 + 255) / 256 : 512), unsigned(n));
            brick_fill_kernel<T><<<grid, 256, 0, ctx->stream>>>(
                raw, d.dim[0], d.dim[1], d.dim[2], d.block_size, d.padding, vol->grid[0],
                vol->grid[1], slot_brick_dev, vol->pool, (long long)vol->slot_stride, s0);
            HY_UP(cudaGetLastError());
        }
    }
    std::vector<int2> info(nb);
    for (int i = 0; i < nb; ++i) info[i] = make_int2(vol->cheb[i], vol->reg_of_brick[i]);
    std::vector<hy::RegEntry> reg(nslots);
    for (int s = 0; s < nslots; ++s) {
        reg[s] = hy::RegEntry{vol->k, vol->b, vol->b, vol->b, (long long)s * (long long)vol->slot_stride,
                              {0, 0}};
    }
    HY_UP(cudaMalloc(&vol->info_dev, nb * sizeof(int2)));
    HY_UP(cudaMalloc(&vol->reg_dev, nslots * sizeof(hy::RegEntry)));
    HY_UP(cudaMalloc(&vol->mean_dev, nb * sizeof(float)));
    HY_UP(cudaMemcpyAsync(vol->info_dev, info.data(), nb * sizeof(int2), cudaMemcpyHostToDevice,
                          ctx->stream));
    HY_UP(cudaMemcpyAsync(vol->reg_dev, reg.data(), nslots * sizeof(hy::RegEntry),
                          cudaMemcpyHostToDevice, ctx->stream));
    HY_UP(cudaMemcpyAsync(vol->mean_dev, vol->mean.data(), nb * sizeof(float),
                          cudaMemcpyHostToDevice, ctx->stream));
    HY_UP(cudaStreamSynchronize(ctx->stream));
#undef HY_UP
    cleanup();
    vol->uploaded = true;
    return build_gather(vol);
}

}  // namespace

int hy_volume_init(hy_ctx *ctx, const hy_volume_desc *desc, hy_volume *v) {
    if (desc->dtype != HY_DTYPE_U8 && desc->dtype != HY_DTYPE_F32)
        return hy_fail(ctx, HY_ERR_INVALID, "volume: dtype must be u8 or f32");
    if (desc->block_size <= 0 || desc->padding < 0 || desc->padding > desc->block_size)
        return hy_fail(ctx, HY_ERR_INVALID, "volume: bad block_size/padding");
    for (int i = 0; i < 3; ++i)
        if (desc->dim[i] <= 0) return hy_fail(ctx, HY_ERR_INVALID, "volume: bad dims");
    v->ctx = ctx;
    v->desc = *desc;
    for (int i = 0; i < 3; ++i) v->grid[i] = (desc->dim[i] + desc->block_size - 1) / desc->block_size;
    long long nb = (long long)v->grid[0] * v->grid[1] * v->grid[2];
    if (nb > (1 << 24)) return hy_fail(ctx, HY_ERR_INVALID, "volume: more than 2^24 bricks");
    v->nbricks = int(nb);
    v->P = desc->block_size + 2 * desc->padding;
    v->elem = desc->dtype == HY_DTYPE_U8 ? 1 : 4;
    size_t bytes = size_t(v->P) * v->P * v->P * v->elem;
    v->slot_stride = (bytes + 255) / 256 * 256;
    // lossless_block_paging.cc:20-22 / rt_block_paging.cc:219-221
    v->k = float(desc->block_size) / float(v->P);
    v->b = float(desc->padding) / float(desc->block_size) * v->k;
    // basic_renderer.hpp:104-118: bbox = [0, raw / block_size], du = 1 / block_size
    float blksz = float(desc->block_size);
    for (int i = 0; i < 3; ++i) v->bbox_max[i] = float(desc->dim[i]) / blksz;
    v->du = 1.f / blksz;
    return HY_OK;
}

extern "C" int hy_volume_create(hy_ctx *ctx, const hy_volume_desc *desc, hy_volume **out) {
    if (!ctx || !desc || !out) return HY_ERR_INVALID;
    *out = nullptr;
    hy_volume *v = new hy_volume();
    int rc = hy_volume_init(ctx, desc, v);
    if (rc) {
        delete v;
        return rc;
    }
    *out = v;
    return HY_OK;
}

extern "C" int hy_volume_destroy(hy_volume *vol) {
    if (!vol) return HY_OK;
    cudaSetDevice(vol->ctx->device);
    cudaStreamSynchronize(vol->ctx->stream);
    free_volume_device(vol);
    delete vol;
    return HY_OK;
}

extern "C" int hy_volume_upload(hy_volume *vol, const void *host_voxels) {
    if (!vol || !host_voxels) return HY_ERR_INVALID;
    if (vol->uploaded || vol->paged)
        return hy_fail(vol->ctx, HY_ERR_STATE,
                       "volume: already has its bricks (create a new volume for new data)");
    HY_CUDA(vol->ctx, cudaSetDevice(vol->ctx->device));
    if (vol->desc.dtype == HY_DTYPE_U8) return upload_impl<unsigned char>(vol, host_voxels);
    return upload_impl<float>(vol, host_voxels);
}

const hy::TexEntry *hy_volume_gather_table(const hy_volume *v) {
    return (v->tex_sampling && v->tex_dev) ? v->tex_dev : nullptr;
}

void hy_volume_gather_view(const hy_volume *v, hy::DevVolume *dv) {
    dv->tex = v->paged_gather ? nullptr : hy_volume_gather_table(v);
    dv->info4 = dv->tex ? v->info4_dev : nullptr;
    dv->paged_gather = v->paged_gather ? 1 : 0;
    // every entry a valid handle (the last texture repeated)
    const int n = int(v->atlas_tex.size());
    const bool any = (dv->tex || v->paged_gather) && n > 0;
    for (int i = 0; i < hy::kMaxGatherTextures; ++i)
        dv->gtex[i] = any ? v->atlas_tex[std::min(i, n - 1)] : 0ull;
}

int hy_gather_layout(hy_ctx *ctx, int P, bool *ok, int *cols, int *rowblocks) {
    *ok = false;
    *cols = *rowblocks = 0;
    int gw = 0, gh = 0;
    HY_CUDA(ctx, cudaDeviceGetAttribute(&gw, cudaDevAttrMaxTexture2DGatherWidth, ctx->device));
    HY_CUDA(ctx, cudaDeviceGetAttribute(&gh, cudaDevAttrMaxTexture2DGatherHeight, ctx->device));
    const long long brick_rows = (long long)P * P;
    if (P <= 0 || P > gw || brick_rows > gh) return HY_OK;
    int rc = gather_check(ctx, ok);
    if (rc) return rc;
    *cols = gw / P;
    *rowblocks = int(gh / brick_rows);
    return HY_OK;
}

int hy_gather_texture_create(hy_ctx *ctx, size_t width, size_t height, cudaArray_t *arr,
                             unsigned long long *tex, unsigned long long *surf) {
    *arr = nullptr;
    *tex = 0;
    if (surf) *surf = 0;
    cudaChannelFormatDesc cd = cudaCreateChannelDesc(8, 0, 0, 0, cudaChannelFormatKindUnsigned);
    const unsigned int flags = cudaArrayTextureGather | (surf ? cudaArraySurfaceLoadStore : 0u);
    cudaError_t e = cudaMallocArray(arr, &cd, width, height, flags);
    if (e != cudaSuccess) {
        *arr = nullptr;
        return hy_cuda_fail(ctx, e, "gather texture allocation");
    }
    cudaTextureObject_t t = make_gather_texture(*arr, &e);
    if (e != cudaSuccess) {
        cudaFreeArray(*arr);
        *arr = nullptr;
        return hy_cuda_fail(ctx, e, "gather texture object");
    }
    if (surf) {
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = *arr;
        cudaSurfaceObject_t so = 0;
        e = cudaCreateSurfaceObject(&so, &rd);
        if (e != cudaSuccess) {
            cudaDestroyTextureObject(t);
            cudaFreeArray(*arr);
            *arr = nullptr;
            return hy_cuda_fail(ctx, e, "gather texture surface");
        }
        *surf = (unsigned long long)so;
    }
    *tex = (unsigned long long)t;
    return HY_OK;
}

void hy_volume_free_gather(hy_volume *v) { free_gather(v); }

extern "C" int hy_volume_set_gather_sampling(hy_volume *vol, int32_t enable) {
    if (!vol) return HY_ERR_INVALID;
    vol->tex_sampling = enable != 0;
    return HY_OK;
}

extern "C" int hy_volume_gather_sampling(const hy_volume *vol, int32_t *active) {
    if (!vol || !active) return HY_ERR_INVALID;
    *active = hy_volume_gather_table(vol) ? 1 : 0;
    return HY_OK;
}

extern "C" int hy_volume_get_info(const hy_volume *vol, hy_volume_info *out) {
    if (!vol || !out) return HY_ERR_INVALID;
    for (int i = 0; i < 3; ++i) {
        out->grid[i] = vol->grid[i];
        out->bbox_max[i] = vol->bbox_max[i];
    }
    out->nbricks = vol->nbricks;
    out->nonempty = vol->nonempty;
    out->resident = vol->resident;
    out->padded = vol->P;
    out->slot_bytes = (int64_t)vol->slot_stride;
    out->pool_bytes = (int64_t)vol->pool_bytes;
    return HY_OK;
}

extern "C" int hy_volume_thumbnails(const hy_volume *vol, int32_t *chebyshev, float *mean) {
    if (!vol) return HY_ERR_INVALID;
    if (!vol->uploaded) return hy_fail(vol->ctx, HY_ERR_STATE, "volume: not uploaded");
    for (int i = 0; i < vol->nbricks; ++i) {
        if (chebyshev) chebyshev[i] = vol->cheb[i];
        if (mean) mean[i] = vol->mean[i];
    }
    return HY_OK;
}
