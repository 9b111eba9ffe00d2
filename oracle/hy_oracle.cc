// hy_oracle.cc -- TEST INFRASTRUCTURE ONLY (see hy_oracle.h).
//
// A CPU restatement of Hydrant's CPU shading backend for the ray-marching
// path.  Every function names the reference lines it follows.  It is built
// with -ffp-contract=off so that every multiply and add rounds separately,
// which is how the reference's host code evaluates on x86-64; the result is
// then the same on x86-64 and aarch64.
//
// PARITY UNPINNED: no reference build and no reference golden vectors exist
// for this path (see hy_oracle.h).
//
// Vector/matrix helpers are written from their definitions (component-wise
// IEEE float operations, left-to-right sums).  min/max follow the
// "(b < a) ? b : a" / "(a < b) ? b : a" forms, so a NaN in the first
// argument propagates and one in the second does not.

#include "hy_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct F3 {
    float x, y, z;
};
struct F4 {
    float x, y, z, w;
};

inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
inline F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline F3 mul(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline F3 muls(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
inline F3 adds(F3 a, float s) { return f3(a.x + s, a.y + s, a.z + s); }
inline F3 floor3(F3 a) { return f3(std::floor(a.x), std::floor(a.y), std::floor(a.z)); }
inline float gmin(float a, float b) { return (b < a) ? b : a; }
inline float gmax(float a, float b) { return (a < b) ? b : a; }
inline int imin(int a, int b) { return (b < a) ? b : a; }
inline int imax(int a, int b) { return (a < b) ? b : a; }
inline int iclamp(int x, int lo, int hi) { return imin(imax(x, lo), hi); }
inline float fclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(F3 a) { return std::sqrt(dot(a, a)); }
inline F3 normalize(F3 a) { return muls(a, 1.f / std::sqrt(dot(a, a))); }
inline F3 cross(F3 a, F3 b) {
    return f3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
inline float comp_max(F3 a) { return gmax(gmax(a.x, a.y), a.z); }
inline float comp_min(F3 a) { return gmin(gmin(a.x, a.y), a.z); }
inline float fsign(float x) { return float((0.f < x) - (x < 0.f)); }
// float -> int conversion, defined for every input: truncation toward zero,
// saturating at the int range, NaN -> 0.  C++ leaves NaN / out-of-range
// undefined; this is what the GPU conversion instruction does.
inline int f2i(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.f) return 2147483647;
    if (x <= -2147483648.f) return (-2147483647 - 1);
    return int(x);
}
// Steps skipped over empty bricks: the reference's value is a small
// non-negative integer; degenerate (NaN / negative / huge) values are pinned
// to [0, 2^30] so nsteps cannot overflow.
inline int skip_count(float di) {
    return (di >= 0.f) ? (di < 1073741824.f ? int(di) : 1073741824) : 0;
}

// Column-major 4x4: m[c*4 + r].
struct M4 {
    float m[16];
};
inline M4 ident() {
    M4 r{};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.f;
    return r;
}
inline F4 mulv(const M4 &a, F4 v) {
    F4 r;
    r.x = a.m[0] * v.x + a.m[4] * v.y + a.m[8] * v.z + a.m[12] * v.w;
    r.y = a.m[1] * v.x + a.m[5] * v.y + a.m[9] * v.z + a.m[13] * v.w;
    r.z = a.m[2] * v.x + a.m[6] * v.y + a.m[10] * v.z + a.m[14] * v.w;
    r.w = a.m[3] * v.x + a.m[7] * v.y + a.m[11] * v.z + a.m[15] * v.w;
    return r;
}
inline M4 mulm(const M4 &a, const M4 &b) {
    M4 r;
    for (int c = 0; c < 4; ++c) {
        F4 col = mulv(a, F4{b.m[c * 4 + 0], b.m[c * 4 + 1], b.m[c * 4 + 2], b.m[c * 4 + 3]});
        r.m[c * 4 + 0] = col.x;
        r.m[c * 4 + 1] = col.y;
        r.m[c * 4 + 2] = col.z;
        r.m[c * 4 + 3] = col.w;
    }
    return r;
}
// General inverse by cofactor expansion (adjugate / determinant).
M4 inverse(const M4 &in) {
    const float *a = in.m;
    float inv[16];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] +
             a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] -
             a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] +
             a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] -
              a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] -
             a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] +
             a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] -
             a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] +
              a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] +
             a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] -
             a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] +
              a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] -
              a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] -
             a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] +
             a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] -
              a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] +
              a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    float rdet = 1.f / det;
    M4 r;
    for (int i = 0; i < 16; ++i) r.m[i] = inv[i] * rdet;
    return r;
}
// Axis-angle rotation matrix R = cI + (1-c) k k^T + s [k]x, column-major.
M4 rotation(float angle, F3 axis_in) {
    float c = std::cos(angle), s = std::sin(angle);
    F3 k = normalize(axis_in);
    F3 t = muls(k, 1.f - c);
    M4 r = ident();
    r.m[0] = c + t.x * k.x;
    r.m[1] = t.x * k.y + s * k.z;
    r.m[2] = t.x * k.z - s * k.y;
    r.m[4] = t.y * k.x - s * k.z;
    r.m[5] = c + t.y * k.y;
    r.m[6] = t.y * k.z + s * k.x;
    r.m[8] = t.z * k.x + s * k.y;
    r.m[9] = t.z * k.y - s * k.x;
    r.m[10] = c + t.z * k.z;
    return r;
}
// Right-handed view matrix (world -> eye), eye looking down -z.
M4 look_at(F3 eye, F3 center, F3 up) {
    F3 f = normalize(sub(center, eye));
    F3 s = normalize(cross(f, up));
    F3 u = cross(s, f);
    M4 r = ident();
    r.m[0] = s.x;
    r.m[4] = s.y;
    r.m[8] = s.z;
    r.m[1] = u.x;
    r.m[5] = u.y;
    r.m[9] = u.z;
    r.m[2] = -f.x;
    r.m[6] = -f.y;
    r.m[10] = -f.z;
    r.m[12] = -dot(s, eye);
    r.m[13] = -dot(u, eye);
    r.m[14] = dot(f, eye);
    return r;
}
inline float radians(float deg) { return deg * 0.01745329251994329576923690768489f; }

}  // namespace

// ---------------------------------------------------------------------------
// Volume: bricks, page table, thumbnails.
// The brick layout (padded bricks, apron replicated at the volume border)
// and the thumbnails (chebyshev distance in bricks to the nearest non-empty
// brick, 0 = non-empty; mean of the normalised core voxels) are this
// project's definition of the dataset the renderers read through
// lossless_block_paging.cc:17-22 and basic_renderer.hpp:104-118 (the varch
// archive and thumbnail builders that define them in the reference are not
// vendored).
// ---------------------------------------------------------------------------
struct orc_volume {
    int dim[3];
    int bs, pad, P, dtype;
    int grid[3];
    int nbricks;
    int nonempty;
    std::vector<float> bricks;  // nbricks * P^3, normalised like texture_3d.hpp:78-86
    std::vector<int> cheb;
    std::vector<int> vaddr;     // brick -> registry id or -1
    // BlockSampler registry (block_paging.hpp:24-36): brick data + mapping
    struct Entry {
        const float *data;
        float k, bx, by, bz;
    };
    std::vector<Entry> reg;
    int lowest_blkcnt = 0;      // registry ids below this sample the coarse level
    int coarse_level = 0;
    int coarse_grid[3] = {0, 0, 0};
    std::vector<float> coarse_bricks;
    std::vector<uint8_t> nonempty_mask;
    std::vector<float> mean;
    float k;                    // BlockSamplerMapping (lossless_block_paging.cc:21-22)
    float b;
    F3 bbox_max;                // raw / block_size (basic_renderer.hpp:109-117)
    float du;
    F3 center, size;            // Exhibit (basic_renderer.hpp:112-115)
};

namespace {

template <typename T>
void brick_volume(orc_volume *v, const T *raw) {
    const int P = v->P;
    const size_t P3 = size_t(P) * P * P;
    v->bricks.assign(size_t(v->nbricks) * P3, 0.f);
    v->nonempty_mask.assign(v->nbricks, 0);
    v->mean.assign(v->nbricks, 0.f);
    const int *d = v->dim;
    for (int bz = 0; bz < v->grid[2]; ++bz)
        for (int by = 0; by < v->grid[1]; ++by)
            for (int bx = 0; bx < v->grid[0]; ++bx) {
                int bid = (bz * v->grid[1] + by) * v->grid[0] + bx;
                float *dst = &v->bricks[size_t(bid) * P3];
                bool any = false;
                double sum = 0.0;
                for (int k = 0; k < P; ++k)
                    for (int j = 0; j < P; ++j)
                        for (int i = 0; i < P; ++i) {
                            int gx = iclamp(bx * v->bs + i - v->pad, 0, d[0] - 1);
                            int gy = iclamp(by * v->bs + j - v->pad, 0, d[1] - 1);
                            int gz = iclamp(bz * v->bs + k - v->pad, 0, d[2] - 1);
                            T val = raw[(size_t(gz) * d[1] + gy) * d[0] + gx];
                            float f;
                            if (sizeof(T) == 1) {
                                f = fclamp(float(val) / 255.f, 0.f, 1.f);
                            } else {
                                f = float(val);
                            }
                            dst[(size_t(k) * P + j) * P + i] = f;
                            if (val != T(0)) any = true;
                            bool core = i >= v->pad && i < v->pad + v->bs && j >= v->pad &&
                                        j < v->pad + v->bs && k >= v->pad && k < v->pad + v->bs;
                            if (core) sum += double(val);
                        }
                v->nonempty_mask[bid] = any ? 1 : 0;
                double n = double(v->bs) * v->bs * v->bs;
                if (sizeof(T) == 1)
                    v->mean[bid] = float(sum / 255.0 / n);
                else
                    v->mean[bid] = float(sum / n);
            }
}

// Chebyshev (L-infinity) distance in bricks by repeated 26-neighbour
// dilation; bricks with no non-empty brick anywhere get max(grid).
void chebyshev_transform(orc_volume *v) {
    const int gx = v->grid[0], gy = v->grid[1], gz = v->grid[2];
    const int cap = std::max(gx, std::max(gy, gz));
    std::vector<int> d(v->nbricks, -1);
    int nonempty = 0;
    for (int i = 0; i < v->nbricks; ++i)
        if (v->nonempty_mask[i]) {
            d[i] = 0;
            ++nonempty;
        }
    v->nonempty = nonempty;
    for (int r = 1; r <= cap; ++r) {
        bool changed = false;
        std::vector<int> nd = d;
        for (int z = 0; z < gz; ++z)
            for (int y = 0; y < gy; ++y)
                for (int x = 0; x < gx; ++x) {
                    int id = (z * gy + y) * gx + x;
                    if (d[id] >= 0) continue;
                    bool hit = false;
                    for (int dz = -1; dz <= 1 && !hit; ++dz)
                        for (int dy = -1; dy <= 1 && !hit; ++dy)
                            for (int dx = -1; dx <= 1 && !hit; ++dx) {
                                int X = x + dx, Y = y + dy, Z = z + dz;
                                if (X < 0 || Y < 0 || Z < 0 || X >= gx || Y >= gy || Z >= gz)
                                    continue;
                                if (d[(Z * gy + Y) * gx + X] == r - 1) hit = true;
                            }
                    if (hit) {
                        nd[id] = r;
                        changed = true;
                    }
                }
        d.swap(nd);
        if (!changed) break;
    }
    for (int i = 0; i < v->nbricks; ++i)
        if (d[i] < 0) d[i] = cap;
    v->cheb = d;
}

}  // namespace

extern "C" orc_volume *orc_volume_create(const int32_t dim[3], int32_t block_size,
                                         int32_t padding, int32_t dtype, const void *voxels) {
    if (!dim || block_size <= 0 || padding < 0 || !voxels) return nullptr;
    auto *v = new orc_volume();
    for (int i = 0; i < 3; ++i) {
        v->dim[i] = dim[i];
        v->grid[i] = (dim[i] + block_size - 1) / block_size;
    }
    v->bs = block_size;
    v->pad = padding;
    v->P = block_size + 2 * padding;
    v->dtype = dtype;
    v->nbricks = v->grid[0] * v->grid[1] * v->grid[2];
    if (dtype == 0)
        brick_volume(v, static_cast<const uint8_t *>(voxels));
    else
        brick_volume(v, static_cast<const float *>(voxels));
    chebyshev_transform(v);
    v->vaddr.assign(v->nbricks, -1);
    for (int i = 0; i < v->nbricks; ++i)
        if (v->nonempty_mask[i]) v->vaddr[i] = i;
    // lossless_block_paging.cc:20-22: k = float(bs)/pad_bs; b = float(pad)/bs*k
    v->k = float(block_size) / float(v->P);
    v->b = float(padding) / float(block_size) * v->k;
    const size_t P3 = size_t(v->P) * v->P * v->P;
    v->reg.resize(v->nbricks);
    for (int i = 0; i < v->nbricks; ++i) v->reg[i] = {&v->bricks[i * P3], v->k, v->b, v->b, v->b};
    // basic_renderer.hpp:104-118
    float blksz = float(block_size);
    v->bbox_max = f3(float(dim[0]) / blksz, float(dim[1]) / blksz, float(dim[2]) / blksz);
    v->center = f3(v->bbox_max.x / 2.f, v->bbox_max.y / 2.f, v->bbox_max.z / 2.f);
    v->size = v->bbox_max;
    v->du = 1.f / blksz;
    return v;
}

extern "C" void orc_volume_free(orc_volume *v) { delete v; }

extern "C" void orc_volume_grid(const orc_volume *v, int32_t grid[3], int32_t *nonempty) {
    for (int i = 0; i < 3; ++i) grid[i] = v->grid[i];
    if (nonempty) *nonempty = v->nonempty;
}

extern "C" void orc_volume_thumbnails(const orc_volume *v, int32_t *chebyshev, float *mean) {
    for (int i = 0; i < v->nbricks; ++i) {
        if (chebyshev) chebyshev[i] = v->cheb[i];
        if (mean) mean[i] = v->mean[i];
    }
}

// Absent bricks read the coarse level when there is one (the basic vaddr of
// rt_block_paging.cc:212-218, restored on eviction at 262-264), else -1.
extern "C" void orc_volume_set_present(orc_volume *v, const uint8_t *present) {
    for (int i = 0; i < v->nbricks; ++i) {
        if (!v->nonempty_mask[i])
            v->vaddr[i] = -1;
        else if (present[i])
            v->vaddr[i] = v->lowest_blkcnt + i;
        else
            v->vaddr[i] = v->coarse_level ? i : -1;
    }
}

// The lowest sample level: the volume box-filtered by s = 2^level (mean of
// the fine voxels of each s^3 cube inside the volume, u8 rounded half up),
// bricked like the fine level; registry [0, nbricks) = one coarse sampler per
// fine brick (k = bs/P/s, b = pad/P + d*k, rt_block_paging.cc:141-188),
// [nbricks, 2*nbricks) = the fine bricks.
extern "C" int orc_volume_build_coarse(orc_volume *v, int32_t level) {
    if (level < 1 || level > 12 || v->bs % (1 << level) != 0) return -1;
    const int sc = 1 << level, bs = v->bs, pad = v->pad, P = v->P;
    const size_t P3 = size_t(P) * P * P;
    int cdim[3];
    for (int i = 0; i < 3; ++i) {
        cdim[i] = (v->dim[i] + sc - 1) / sc;
        v->coarse_grid[i] = (cdim[i] + bs - 1) / bs;
    }
    // fine voxel (x, y, z) is the core voxel of brick (x, y, z) / bs
    auto fine = [&](int x, int y, int z) {
        const int b = ((z / bs) * v->grid[1] + y / bs) * v->grid[0] + x / bs;
        const int lx = x % bs + pad, ly = y % bs + pad, lz = z % bs + pad;
        return v->bricks[b * P3 + (size_t(lz) * P + ly) * P + lx];
    };
    std::vector<float> cvol(size_t(cdim[0]) * cdim[1] * cdim[2]);
    for (int Z = 0; Z < cdim[2]; ++Z)
        for (int Y = 0; Y < cdim[1]; ++Y)
            for (int X = 0; X < cdim[0]; ++X) {
                long long isum = 0, cnt = 0;
                double fsum = 0.0;
                for (int z = Z * sc; z < std::min((Z + 1) * sc, v->dim[2]); ++z)
                    for (int y = Y * sc; y < std::min((Y + 1) * sc, v->dim[1]); ++y)
                        for (int x = X * sc; x < std::min((X + 1) * sc, v->dim[0]); ++x) {
                            const float f = fine(x, y, z);
                            if (v->dtype == 0)
                                isum += (long long)(f * 255.f + 0.5f);  // u / 255.f -> u
                            else
                                fsum += double(f);
                            ++cnt;
                        }
                float c;
                if (v->dtype == 0)
                    c = float(int((isum + cnt / 2) / cnt)) / 255.f;
                else
                    c = float(fsum / double(cnt));
                cvol[(size_t(Z) * cdim[1] + Y) * cdim[0] + X] = c;
            }
    const int *g = v->coarse_grid;
    const int ncoarse = g[0] * g[1] * g[2];
    v->coarse_bricks.assign(size_t(ncoarse) * P3, 0.f);
    for (int cb = 0; cb < ncoarse; ++cb) {
        const int bx = cb % g[0], by = (cb / g[0]) % g[1], bz = cb / (g[0] * g[1]);
        for (int k = 0; k < P; ++k)
            for (int j = 0; j < P; ++j)
                for (int i = 0; i < P; ++i) {
                    const int x = iclamp(bx * bs + i - pad, 0, cdim[0] - 1);
                    const int y = iclamp(by * bs + j - pad, 0, cdim[1] - 1);
                    const int z = iclamp(bz * bs + k - pad, 0, cdim[2] - 1);
                    v->coarse_bricks[cb * P3 + (size_t(k) * P + j) * P + i] =
                        cvol[(size_t(z) * cdim[1] + y) * cdim[0] + x];
                }
    }
    const float kc = float(bs) / float(P) / float(sc);
    const float b0 = float(pad) / float(P);
    v->reg.resize(2 * size_t(v->nbricks));
    for (int b = 0; b < v->nbricks; ++b) {
        const int x = b % v->grid[0], y = (b / v->grid[0]) % v->grid[1],
                  z = b / (v->grid[0] * v->grid[1]);
        const int cid = ((z / sc) * g[1] + y / sc) * g[0] + x / sc;
        v->reg[b] = {&v->coarse_bricks[cid * P3], kc, b0 + float(x % sc) * kc,
                     b0 + float(y % sc) * kc, b0 + float(z % sc) * kc};
        v->reg[v->nbricks + b] = {&v->bricks[b * P3], v->k, v->b, v->b, v->b};
    }
    v->coarse_level = level;
    v->lowest_blkcnt = v->nbricks;
    for (int i = 0; i < v->nbricks; ++i) v->vaddr[i] = v->nonempty_mask[i] ? v->nbricks + i : -1;
    return 0;
}

extern "C" int32_t orc_volume_lowest_blkcnt(const orc_volume *v) { return v->lowest_blkcnt; }

extern "C" void orc_volume_coarse_brick(const orc_volume *v, int32_t brick, float *out) {
    const size_t P3 = size_t(v->P) * v->P * v->P;
    std::memcpy(out, &v->coarse_bricks[size_t(brick) * P3], P3 * sizeof(float));
}

extern "C" void orc_volume_brick(const orc_volume *v, int32_t brick, float *out) {
    size_t P3 = size_t(v->P) * v->P * v->P;
    std::memcpy(out, &v->bricks[size_t(brick) * P3], P3 * sizeof(float));
}

// ---------------------------------------------------------------------------
// Camera (scene.hpp:20-81, raycaster.hpp:249-258, isosurface.cc:108-113).
// ---------------------------------------------------------------------------
namespace {
M4 exhibit_iet(const orc_volume *v) {
    // scene.hpp:20-29: d = max(|center - size|, |center|), scale = compMax(d)
    F3 c = v->center, s = v->size;
    F3 a = f3(std::fabs(c.x - s.x), std::fabs(c.y - s.y), std::fabs(c.z - s.z));
    F3 b = f3(std::fabs(c.x), std::fabs(c.y), std::fabs(c.z));
    F3 d = f3(gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z));
    float scale = comp_max(d);
    M4 et{};
    et.m[0] = scale;
    et.m[5] = scale;
    et.m[10] = scale;
    et.m[12] = c.x;
    et.m[13] = c.y;
    et.m[14] = c.z;
    et.m[15] = 1.f;
    return et;
}
}  // namespace

extern "C" void orc_camera_orbit(const float arm[3], const float center[3], float fovy_deg,
                                 float out[10]) {
    // scene.hpp:68-81: rotate (arm.z,0,0) by arm.y deg about z, then arm.x deg about y
    M4 rz = rotation(radians(arm[1]), f3(0, 0, 1));
    F4 p = mulv(rz, F4{arm[2], 0.f, 0.f, 1.f});
    M4 ry = rotation(radians(arm[0]), f3(0, 1, 0));
    F4 q = mulv(ry, F4{p.x, p.y, p.z, 1.f});
    out[0] = q.x;
    out[1] = q.y;
    out[2] = q.z;
    out[3] = center[0];
    out[4] = center[1];
    out[5] = center[2];
    out[6] = 0.f;
    out[7] = 1.f;
    out[8] = 0.f;
    out[9] = 1.f / std::tan(radians(fovy_deg / 2.f));  // scene.hpp:52-54
}

extern "C" void orc_camera_ptu(const float pos[3], const float target[3], const float up[3],
                               float fovy_deg, float out[10]) {
    for (int i = 0; i < 3; ++i) {
        out[i] = pos[i];
        out[3 + i] = target[i];
        out[6 + i] = up[i];
    }
    out[9] = 1.f / std::tan(radians(fovy_deg / 2.f));
}

extern "C" void orc_camera_view(const orc_volume *v, const float cam[10], float view[20]) {
    // raycaster.hpp:249-258: trans = iet * inverse(lookAt), ray_o = iet * eye
    F3 eye = f3(cam[0], cam[1], cam[2]);
    M4 iet = exhibit_iet(v);
    M4 ivt = inverse(look_at(eye, f3(cam[3], cam[4], cam[5]), f3(cam[6], cam[7], cam[8])));
    M4 trans = mulm(iet, ivt);
    for (int i = 0; i < 16; ++i) view[i] = trans.m[i];
    view[16] = cam[9];
    F4 o = mulv(iet, F4{eye.x, eye.y, eye.z, 1.f});
    view[17] = o.x;
    view[18] = o.y;
    view[19] = o.z;
}

extern "C" void orc_iso_lighting(const orc_volume *v, const float cam[10], orc_params *p) {
    // isosurface.cc:108-113
    M4 tw = inverse(exhibit_iet(v));
    for (int i = 0; i < 16; ++i) p->to_world[i] = tw.m[i];
    F3 pos = f3(cam[0], cam[1], cam[2]), tgt = f3(cam[3], cam[4], cam[5]),
       up = f3(cam[6], cam[7], cam[8]);
    F3 l = add(add(add(pos, tgt), up), cross(tgt, up));
    p->light_pos[0] = l.x;
    p->light_pos[1] = l.y;
    p->light_pos[2] = l.z;
    p->eye_pos[0] = pos.x;
    p->eye_pos[1] = pos.y;
    p->eye_pos[2] = pos.z;
}

// ---------------------------------------------------------------------------
// Shading.
// ---------------------------------------------------------------------------
namespace {

struct Ray {
    F3 o, d;
};

// glm_math.hpp:58-72 (slab test)
bool intersect(const Ray &r, F3 bmin, F3 bmax, float &tnear, float &tfar) {
    F3 invr = f3(1.f / r.d.x, 1.f / r.d.y, 1.f / r.d.z);
    F3 tbot = mul(invr, sub(bmin, r.o));
    F3 ttop = mul(invr, sub(bmax, r.o));
    F3 tmin = f3(gmin(ttop.x, tbot.x), gmin(ttop.y, tbot.y), gmin(ttop.z, tbot.z));
    F3 tmax = f3(gmax(ttop.x, tbot.x), gmax(ttop.y, tbot.y), gmax(ttop.z, tbot.z));
    tnear = comp_max(tmin);
    tfar = comp_min(tmax);
    return tfar > tnear;
}

// Pixel state: IPixel + StdVec4Pixel + the per-shader extras
// (shader.hpp:26-34, pixel_template.hpp:11-20, volume_shader.hpp:11-15,
// isosurface_shader.hpp:11-15).
struct Px {
    Ray ray;
    int nsteps, step_size;
    F4 v;
    F3 theta;   // Volume
    float phi;  // Volume
    F3 origin;  // Isosurface
    float depth;
};

struct Ctx {
    const orc_volume *vol;
    const F4 *tf;
    int ntf;
    orc_params p;
    F3 bbox_min, bbox_max;
    float step, du;
    int max_steps;
};

// Thumbnail / page-table textures: non-normalised, nearest, Clamp
// (basic_renderer.hpp:195-206, lossless_block_paging.cc:47-52;
// cpu_sampler.hpp:142-166 with filter_none 72-76).
inline int thumb_index(const orc_volume *v, F3 x) {
    float fx = fclamp(x.x, 0.f, float(v->grid[0]));
    float fy = fclamp(x.y, 0.f, float(v->grid[1]));
    float fz = fclamp(x.z, 0.f, float(v->grid[2]));
    int ix = iclamp(f2i(std::floor(fx)), 0, v->grid[0] - 1);
    int iy = iclamp(f2i(std::floor(fy)), 0, v->grid[1] - 1);
    int iz = iclamp(f2i(std::floor(fz)), 0, v->grid[2] - 1);
    return (iz * v->grid[1] + iy) * v->grid[0] + ix;
}

inline float lerp(float x, float y, float a) { return x * (1.f - a) + y * a; }  // cpu_sampler.hpp:126-129

// Brick sample: BlockSampler::sample_3d (block_paging.hpp:24-36) ->
// CpuSampler::sample_impl with normalised coords, Wrap, Linear
// (cpu_sampler.hpp:142-166, filter_linear 88-104).
float sample_brick(const orc_volume *v, int pgid, F3 x) {
    const int P = v->P;
    const orc_volume::Entry &e = v->reg[pgid];
    const float *data = e.data;
    F3 m = f3(e.k * x.x + e.bx, e.k * x.y + e.by, e.k * x.z + e.bz);
    float fd = float(P);
    F3 fx = f3(fd * m.x, fd * m.y, fd * m.z);
    // glm mod(x, y) = x - y * floor(x / y)
    fx = f3(fx.x - fd * std::floor(fx.x / fd), fx.y - fd * std::floor(fx.y / fd),
            fx.z - fd * std::floor(fx.z / fd));
    F3 u = f3(fx.x - .5f, fx.y - .5f, fx.z - .5f);
    F3 flr = floor3(u);
    F3 a = sub(u, flr);
    int ix = iclamp(f2i(flr.x), 0, P - 1), iy = iclamp(f2i(flr.y), 0, P - 1),
        iz = iclamp(f2i(flr.z), 0, P - 1);
    int jx = iclamp(f2i(std::ceil(u.x)), 0, P - 1), jy = iclamp(f2i(std::ceil(u.y)), 0, P - 1),
        jz = iclamp(f2i(std::ceil(u.z)), 0, P - 1);
    auto at = [&](int X, int Y, int Z) { return data[(size_t(Z) * P + Y) * P + X]; };
    float x0_0 = lerp(at(ix, iy, iz), at(jx, iy, iz), a.x);
    float x1_0 = lerp(at(ix, jy, iz), at(jx, jy, iz), a.x);
    float x0_1 = lerp(at(ix, iy, jz), at(jx, iy, jz), a.x);
    float x1_1 = lerp(at(ix, jy, jz), at(jx, jy, jz), a.x);
    float y0 = lerp(x0_0, x1_0, a.y);
    float y1 = lerp(x0_1, x1_1, a.y);
    return lerp(y0, y1, a.z);
}

// TransferFn: 1-D, normalised coords, Border, Linear (transfer_fn.hpp:16-23;
// cpu_sampler.hpp:117-124, 137-140, 142-166).
F4 sample_tf(const Ctx &c, float s) {
    float fd = float(c.ntf);
    float fx = fd * s;
    if (!(0.f <= fx && fx <= fd)) return F4{0, 0, 0, 0};
    float u = fx - .5f;
    float flr = std::floor(u);
    float a = u - flr;
    int ix = iclamp(f2i(flr), 0, c.ntf - 1);
    int jx = iclamp(f2i(std::ceil(u)), 0, c.ntf - 1);
    F4 x = c.tf[ix], y = c.tf[jx];
    return F4{lerp(x.x, y.x, a), lerp(x.y, y.y, a), lerp(x.z, y.z, a), lerp(x.w, y.w, a)};
}

// volume_shader.cu:5-14 (identical in blocks_shader.cu and isosurface_shader.cu)
int skip_nblock_steps(Ray &ray, F3 ip, int nblocks, float cdu, float step) {
    float tnear, tfar;
    intersect(ray, ip, adds(ip, 1.f), tnear, tfar);
    float di = std::ceil((tfar + float(nblocks - 1) * cdu) / step);
    ray.o = add(ray.o, muls(muls(ray.d, di), step));
    return skip_count(di);
}

// VolumeShaderKernel::main (volume_shader.cu:32-81)
int64_t volume_main(const Ctx &c, Px &px) {
    const orc_volume *v = c.vol;
    int64_t samples = 0;
    const float cdu = 1.f / comp_max(f3(std::fabs(px.ray.d.x), std::fabs(px.ray.d.y),
                                        std::fabs(px.ray.d.z)));
    Ray &ray = px.ray;
    while (px.nsteps > 0) {
        F3 ip = floor3(ray.o);
        int bid = thumb_index(v, ip);
        if (int cd = v->cheb[bid]) {
            px.nsteps -= skip_nblock_steps(ray, ip, cd, cdu, c.step * float(px.step_size));
        } else {
            int pgid = v->vaddr[bid];
            if (pgid == -1) break;
            float s = sample_brick(v, pgid, sub(ray.o, ip));
            ++samples;
            F4 ub = sample_tf(c, s);
            if (c.p.mode == 1) {  // Partition
                // mix(lower, upper, rank) * length(rgb), mix(x,y,a) = x*(1-a) + y*a
                F3 lower = f3(1, 0, 0), upper = f3(0, 0, 1);
                float r = c.p.rank;
                F3 m = add(muls(lower, 1.f - r), muls(upper, r));
                float len = length(f3(ub.x, ub.y, ub.z));
                F3 t = muls(m, len);
                ub = F4{t.x, t.y, t.z, ub.w};
            } else if (c.p.mode == 2) {  // Paging
                if (pgid >= c.p.lowest_blkcnt)
                    ub = F4{0, 1, 0, ub.w};
                else
                    ub = F4{1, 0, 0, ub.w};
            }
            // opacity scale (1 reproduces the reference exactly)
            ub.w = ub.w * c.p.density;
            float w = ub.w;
            ub = F4{ub.x * w, ub.y * w, ub.z * w, ub.w * 1.f};
            px.theta = add(px.theta, muls(f3(ub.x, ub.y, ub.z), px.phi));
            px.phi = px.phi * (1.f - ub.w);
            float t = 1.f - px.v.w;
            px.v = F4{px.v.x + ub.x * t, px.v.y + ub.y * t, px.v.z + ub.z * t, px.v.w + ub.w * t};
            if (double(px.v.w) > 0.93) {
                px.step_size = 16;
            } else if (double(px.v.w) > 0.85) {
                px.step_size = 4;
            }
        }
        ray.o = add(ray.o, muls(muls(ray.d, c.step), float(px.step_size)));
        px.nsteps -= px.step_size;
    }
    return samples;
}

// VisBlocksShaderKernel::main (blocks_shader.cu:16-50)
int64_t blocks_main(const Ctx &c, Px &px) {
    const orc_volume *v = c.vol;
    int64_t samples = 0;
    const float cdu = 1.f / comp_max(f3(std::fabs(px.ray.d.x), std::fabs(px.ray.d.y),
                                        std::fabs(px.ray.d.z)));
    const float opacity_threshold = 0.95f;
    Ray &ray = px.ray;
    while (px.nsteps > 0) {
        F3 ip = floor3(ray.o);
        int bid = thumb_index(v, ip);
        if (int cd = v->cheb[bid]) {
            px.nsteps -= skip_nblock_steps(ray, ip, cd, cdu, c.step);
        } else {
            F3 hi = f3(c.bbox_max.x - 1.f, c.bbox_max.y - 1.f, c.bbox_max.z - 1.f);
            F3 cl = f3(fclamp(ip.x, c.bbox_min.x, hi.x), fclamp(ip.y, c.bbox_min.y, hi.y),
                       fclamp(ip.z, c.bbox_min.z, hi.z));
            F3 ext = sub(c.bbox_max, c.bbox_min);
            F3 rip = f3(cl.x / ext.x, cl.y / ext.y, cl.z / ext.z);
            ++samples;
            if (c.p.mode == 0) {  // Volume
                float mean = v->mean[bid];
                F4 col = F4{rip.x * c.p.density * mean, rip.y * c.p.density * mean,
                            rip.z * c.p.density * mean, 1.f * c.p.density * mean};
                float t = 1.f - px.v.w;
                px.v = F4{px.v.x + col.x * t, px.v.y + col.y * t, px.v.z + col.z * t,
                          px.v.w + col.w * t};
                if (px.v.w > opacity_threshold) {
                    px.nsteps = 0;
                    break;
                }
            } else {  // Solid
                px.v = F4{rip.x, rip.y, rip.z, 1.f};
                px.nsteps = 0;
                break;
            }
        }
        ray.o = add(ray.o, muls(ray.d, c.step));
        px.nsteps -= 1;
    }
    return samples;
}

// PagingShaderKernel::main (paging_shader.cu:26-61): a constant colour per
// non-empty brick entered (green 0.5 if its registry id >= lowest_blkcnt,
// red 0.2 otherwise), then a skip to the brick's exit; opacity > 0.95 or a
// page fault ends the ray without touching nsteps.
int64_t paging_main(const Ctx &c, Px &px) {
    const orc_volume *v = c.vol;
    int64_t samples = 0;
    const float cdu = 1.f / comp_max(f3(std::fabs(px.ray.d.x), std::fabs(px.ray.d.y),
                                        std::fabs(px.ray.d.z)));
    const float opacity_threshold = 0.95f;
    Ray &ray = px.ray;
    while (px.nsteps > 0) {
        F3 ip = floor3(ray.o);
        int bid = thumb_index(v, ip);
        if (int cd = v->cheb[bid]) {
            px.nsteps -= skip_nblock_steps(ray, ip, cd, cdu, c.step);
        } else {
            int pgid = v->vaddr[bid];
            if (pgid == -1) break;  // page fault
            F4 col = pgid >= c.p.lowest_blkcnt ? F4{0.f * .5f, 1.f * .5f, 0.f * .5f, 1.f * .5f}
                                               : F4{1.f * .2f, 0.f * .2f, 0.f * .2f, 1.f * .2f};
            px.nsteps -= skip_nblock_steps(ray, ip, 1, cdu, c.step);
            ++samples;
            float t = 1.f - px.v.w;
            px.v = F4{px.v.x + col.x * t, px.v.y + col.y * t, px.v.z + col.z * t,
                      px.v.w + col.w * t};
            if (px.v.w > opacity_threshold) break;
        }
        ray.o = add(ray.o, muls(ray.d, c.step));
        px.nsteps -= 1;
    }
    return samples;
}

float iso_linear_to_srgb(float linear) {
    // isosurface_shader.cu:25-32 (double-precision constants)
    if (double(linear) <= 0.0031308) return float(12.92 * double(linear));
    return float((1.0 + 0.055) * std::pow(double(linear), 1.0 / 2.4) - 0.055);
}

// IsosurfaceShaderKernel::main (isosurface_shader.cu:50-125)
int64_t iso_main(const Ctx &c, Px &px) {
    const orc_volume *v = c.vol;
    int64_t samples = 0;
    const float cdu = 1.f / comp_max(f3(std::fabs(px.ray.d.x), std::fabs(px.ray.d.y),
                                        std::fabs(px.ray.d.z)));
    const float prev_value = 0.0f;
    const float iso = c.p.isovalue;
    Ray &ray = px.ray;
    while (px.nsteps > 0) {
        F3 ip = floor3(ray.o);
        int bid = thumb_index(v, ip);
        if (int cd = v->cheb[bid]) {
            px.nsteps -= skip_nblock_steps(ray, ip, cd, cdu, c.step);
        } else {
            int pgid = v->vaddr[bid];
            if (pgid != -1) {
                float value = sample_brick(v, pgid, sub(ray.o, ip));
                ++samples;
                if (fsign(value - iso) != fsign(prev_value - iso)) {
                    F3 p = ray.o, d = ray.d;
                    float dt = c.step;
                    px.v = F4{c.p.surface_color[0], c.p.surface_color[1], c.p.surface_color[2],
                              1.f};
                    float a = (iso - prev_value) / (value - prev_value);
                    F3 q = sub(p, muls(d, dt));
                    F3 inter_p = add(muls(q, 1.f - a), muls(p, a));
                    // central difference (isosurface_shader.cu:17-23), dt = du * 2
                    F3 lp = sub(inter_p, ip);
                    float g = c.du * 2.f;
                    F3 nn = f3(sample_brick(v, pgid, f3(lp.x - g, lp.y - 0.f, lp.z - 0.f)) -
                                   sample_brick(v, pgid, f3(lp.x + g, lp.y + 0.f, lp.z + 0.f)),
                               sample_brick(v, pgid, f3(lp.x - 0.f, lp.y - g, lp.z - 0.f)) -
                                   sample_brick(v, pgid, f3(lp.x + 0.f, lp.y + g, lp.z + 0.f)),
                               sample_brick(v, pgid, f3(lp.x - 0.f, lp.y - 0.f, lp.z - g)) -
                                   sample_brick(v, pgid, f3(lp.x + 0.f, lp.y + 0.f, lp.z + g)));
                    samples += 6;
                    M4 tw;
                    std::memcpy(tw.m, c.p.to_world, sizeof(tw.m));
                    F4 wp4 = mulv(tw, F4{inter_p.x, inter_p.y, inter_p.z, 1.f});
                    F3 world_p = f3(wp4.x, wp4.y, wp4.z);
                    F4 n4 = mulv(tw, F4{nn.x, nn.y, nn.z, 0.f});
                    F3 n = normalize(f3(n4.x, n4.y, n4.z));
                    F3 light = f3(c.p.light_pos[0], c.p.light_pos[1], c.p.light_pos[2]);
                    F3 light_dir = normalize(sub(light, world_p));
                    F3 h = normalize(sub(light_dir, world_p));
                    const float ambient = 0.2f;
                    float diffuse = .6f * fclamp(dot(light_dir, n), 0.f, 1.f);
                    float specular = .2f * std::pow(fclamp(dot(h, n), 0.f, 1.f), 100.f);
                    F3 eye = f3(c.p.eye_pos[0], c.p.eye_pos[1], c.p.eye_pos[2]);
                    float distance = length(sub(world_p, eye)) / 2.f;
                    if (c.p.mode == 0) {  // Color
                        float f = ambient + (diffuse + specular) / distance;
                        px.v = F4{px.v.x * f, px.v.y * f, px.v.z * f, px.v.w * f};
                        px.v = F4{iso_linear_to_srgb(px.v.x), iso_linear_to_srgb(px.v.y),
                                  iso_linear_to_srgb(px.v.z), px.v.w};
                    } else if (c.p.mode == 2) {  // Position
                        px.v = F4{inter_p.x / c.bbox_max.x, inter_p.y / c.bbox_max.y,
                                  inter_p.z / c.bbox_max.z, 1.f};
                    } else {  // Normal
                        px.v = F4{n.x, n.y, n.z, 1.f};
                    }
                    px.depth = length(sub(px.origin, ray.o));
                    px.nsteps = 0;
                    break;
                }
            } else {
                break;
            }
        }
        ray.o = add(ray.o, muls(ray.d, c.step));
        px.nsteps -= 1;
    }
    return samples;
}

int64_t run_main(const Ctx &c, Px &px) {
    switch (c.p.shader) {
        case 0:
            return volume_main(c, px);
        case 1:
            return blocks_main(c, px);
        case 3:
            return paging_main(c, px);
        default:
            return iso_main(c, px);
    }
}

// ray_emit_shader_impl (shader.hpp:113-137) against box [bmin, bmax]
int64_t emit(const Ctx &c, const Ray &ray_in, F3 bmin, F3 bmax, Px &px) {
    px = Px{};
    // init (volume_shader.cu:16-21, isosurface_shader.cu:34-39)
    px.theta = f3(0, 0, 0);
    px.phi = 1.f;
    px.origin = ray_in.o;
    px.depth = INFINITY;
    px.ray = ray_in;
    float tnear, tfar;
    if (intersect(px.ray, bmin, bmax, tnear, tfar)) {
        if (tnear < 0) tnear = 0;
        if (tfar < 0) tfar = 0;
        px.ray.o = add(px.ray.o, muls(px.ray.d, tnear));
        px.nsteps = imin(c.max_steps, f2i((tfar - tnear) / c.step));
        px.step_size = 1;
        return run_main(c, px);
    }
    px.nsteps = 0;
    px.step_size = 1;
    return 0;
}

// cuda_shading.cu:24-29 == cpu_shading.cc:14-21
Ray gen_ray(const float view[20], int x, int y, int W, int H) {
    float ccx = float(W) / 2.f, ccy = float(H) / 2.f;
    float uvx = (float(x) - ccx) * 2.f / float(H);
    float uvy = (float(y) - ccy) * 2.f / float(H);
    M4 t;
    std::memcpy(t.m, view, sizeof(t.m));
    F4 p = mulv(t, F4{uvx, -uvy, -view[16], 1.f});
    F3 o = f3(view[17], view[18], view[19]);
    Ray r;
    r.o = o;
    r.d = normalize(sub(f3(p.x, p.y, p.z), o));
    return r;
}

inline uint8_t saturate_u8(float f) {
    // glm_math.hpp:75-81: (uchar)clamp(f * 255, 0, 255), truncating
    return (uint8_t)fclamp(f * 255.f, 0.f, 255.f);
}

float vol_linear_to_srgb(float x) {
    // volume.cc:175-181
    if (x <= 0.0031308f) return 12.92f * x;
    return 1.055f * std::pow(x, 1.f / 2.4f) - 0.055f;
}

struct Out {
    float *v;
    uint8_t *rgba;
    float *aux;
    void *film;
};

void write_film(const Ctx &c, const Px &px, void *film, size_t idx) {
    float buf[16];
    buf[0] = px.ray.o.x;
    buf[1] = px.ray.o.y;
    buf[2] = px.ray.o.z;
    buf[3] = px.ray.d.x;
    buf[4] = px.ray.d.y;
    buf[5] = px.ray.d.z;
    std::memcpy(&buf[6], &px.nsteps, 4);
    std::memcpy(&buf[7], &px.step_size, 4);
    buf[8] = px.v.x;
    buf[9] = px.v.y;
    buf[10] = px.v.z;
    buf[11] = px.v.w;
    size_t bytes = 48;
    if (c.p.shader == 0) {
        buf[12] = px.theta.x;
        buf[13] = px.theta.y;
        buf[14] = px.theta.z;
        buf[15] = px.phi;
        bytes = 64;
    } else if (c.p.shader == 2) {
        buf[12] = px.origin.x;
        buf[13] = px.origin.y;
        buf[14] = px.origin.z;
        buf[15] = px.depth;
        bytes = 64;
    }
    std::memcpy(static_cast<char *>(film) + idx * bytes, buf, bytes);
}

void read_film(const Ctx &c, Px &px, const void *film, size_t idx) {
    size_t bytes = (c.p.shader == 1 || c.p.shader == 3) ? 48 : 64;
    float buf[16] = {};
    std::memcpy(buf, static_cast<const char *>(film) + idx * bytes, bytes);
    px = Px{};
    px.ray.o = f3(buf[0], buf[1], buf[2]);
    px.ray.d = f3(buf[3], buf[4], buf[5]);
    std::memcpy(&px.nsteps, &buf[6], 4);
    std::memcpy(&px.step_size, &buf[7], 4);
    px.v = F4{buf[8], buf[9], buf[10], buf[11]};
    if (c.p.shader == 0) {
        px.theta = f3(buf[12], buf[13], buf[14]);
        px.phi = buf[15];
    } else if (c.p.shader == 2) {
        px.origin = f3(buf[12], buf[13], buf[14]);
        px.depth = buf[15];
    }
}

void write_pixel(const Ctx &c, const F4 &v, const float *aux4, const Out &o, size_t idx) {
    if (o.v) {
        o.v[idx * 4 + 0] = v.x;
        o.v[idx * 4 + 1] = v.y;
        o.v[idx * 4 + 2] = v.z;
        o.v[idx * 4 + 3] = v.w;
    }
    if (o.aux && aux4)
        for (int i = 0; i < 4; ++i) o.aux[idx * 4 + i] = aux4[i];
    if (o.rgba) {
        uint8_t *p = &o.rgba[idx * 4];
        // StdVec4Pixel::write_to (pixel_template.hpp:11-20); alpha = saturate(v.a)
        if (v.w != 0.f) {
            p[0] = saturate_u8(v.x);
            p[1] = saturate_u8(v.y);
            p[2] = saturate_u8(v.z);
            p[3] = saturate_u8(v.w);
        } else {
            p[0] = saturate_u8(c.p.clear_color[0]);
            p[1] = saturate_u8(c.p.clear_color[1]);
            p[2] = saturate_u8(c.p.clear_color[2]);
            p[3] = 0;
        }
    }
}

// Front-to-back enumeration of the bricks a ray crosses inside the volume
// box (3-D DDA over the brick grid).  Used by the per-brick sort-last mode.
template <typename F>
void for_each_brick(const Ctx &c, const Ray &r, F &&fn) {
    float tnear, tfar;
    if (!intersect(r, c.bbox_min, c.bbox_max, tnear, tfar)) return;
    float t0 = tnear < 0.f ? 0.f : tnear;
    float t1 = tfar;
    if (!(t1 > t0)) return;
    const orc_volume *v = c.vol;
    F3 p = add(r.o, muls(r.d, t0));
    int cell[3] = {iclamp(f2i(std::floor(p.x)), 0, v->grid[0] - 1),
                   iclamp(f2i(std::floor(p.y)), 0, v->grid[1] - 1),
                   iclamp(f2i(std::floor(p.z)), 0, v->grid[2] - 1)};
    float d[3] = {r.d.x, r.d.y, r.d.z}, o[3] = {r.o.x, r.o.y, r.o.z};
    int stp[3];
    float tmax[3], tdelta[3];
    for (int a = 0; a < 3; ++a) {
        stp[a] = d[a] > 0.f ? 1 : (d[a] < 0.f ? -1 : 0);
        if (stp[a] != 0) {
            float nb = float(stp[a] > 0 ? cell[a] + 1 : cell[a]);
            tmax[a] = (nb - o[a]) / d[a];
            tdelta[a] = 1.f / std::fabs(d[a]);
        } else {
            tmax[a] = INFINITY;
            tdelta[a] = INFINITY;
        }
    }
    int limit = v->grid[0] + v->grid[1] + v->grid[2] + 3;
    for (int it = 0; it < limit; ++it) {
        fn((cell[2] * v->grid[1] + cell[1]) * v->grid[0] + cell[0], cell);
        int a = 0;
        if (tmax[1] < tmax[a]) a = 1;
        if (tmax[2] < tmax[a]) a = 2;
        if (!(tmax[a] < t1)) break;
        cell[a] += stp[a];
        if (cell[a] < 0 || cell[a] >= v->grid[a]) break;
        tmax[a] = tmax[a] + tdelta[a];
    }
}

int64_t shade_pixel(const Ctx &c, const float view[20], int x, int y, int W, int H,
                    const Out &o) {
    size_t idx = size_t(y) * W + x;
    Ray r = gen_ray(view, x, y, W, H);
    if (!c.p.composite) {
        Px px;
        int64_t n = emit(c, r, c.bbox_min, c.bbox_max, px);
        float aux[4] = {0, 0, 0, 0};
        if (c.p.shader == 0) {
            aux[0] = px.theta.x;
            aux[1] = px.theta.y;
            aux[2] = px.theta.z;
            aux[3] = px.phi;
        } else if (c.p.shader == 2) {
            aux[0] = px.depth;
        }
        write_pixel(c, px.v, aux, o, idx);
        if (o.film) write_film(c, px, o.film, idx);
        return n;
    }
    // Per-brick sort-last: each non-empty brick is an emit against its own
    // box (the per-rank bbox of dbuf_renderer.hpp:38-40), composited front
    // to back with volume.cc:267-280 (Volume), isosurface.cc:272-290
    // (Isosurface, depth-min) or the over operator (Blocks).
    int64_t n = 0;
    bool first = true;
    F4 acc{0, 0, 0, 0};
    F3 acc_theta = f3(0, 0, 0);
    float acc_phi = 1.f;
    float acc_depth = INFINITY;
    for_each_brick(c, r, [&](int bid, const int *cell) {
        if (c.vol->cheb[bid] != 0) return;
        F3 bmin = f3(float(cell[0]), float(cell[1]), float(cell[2]));
        F3 bmax = adds(bmin, 1.f);
        Px px;
        n += emit(c, r, bmin, bmax, px);
        if (c.p.shader == 0) {
            if (first) {
                acc = px.v;
                acc_theta = px.theta;
                acc_phi = px.phi;
            } else {
                F3 vn = f3(acc.x + px.v.x - acc.w * px.theta.x, acc.y + px.v.y - acc.w * px.theta.y,
                           acc.z + px.v.z - acc.w * px.theta.z);
                float an = px.phi * acc.w + px.v.w;
                acc = F4{vn.x, vn.y, vn.z, an};
            }
        } else if (c.p.shader == 2) {
            if (first || px.depth < acc_depth) {
                acc = px.v;
                acc_depth = px.depth;
            }
        } else {
            float t = 1.f - acc.w;
            acc = F4{acc.x + px.v.x * t, acc.y + px.v.y * t, acc.z + px.v.z * t, acc.w + px.v.w * t};
        }
        first = false;
    });
    if (c.p.shader == 0 && c.p.srgb) {
        acc = F4{vol_linear_to_srgb(acc.x), vol_linear_to_srgb(acc.y), vol_linear_to_srgb(acc.z),
                 acc.w};
    }
    float aux[4] = {0, 0, 0, 0};
    if (c.p.shader == 0) {
        aux[0] = acc_theta.x;
        aux[1] = acc_theta.y;
        aux[2] = acc_theta.z;
        aux[3] = acc_phi;
    } else if (c.p.shader == 2) {
        aux[0] = acc_depth;
    }
    write_pixel(c, acc, aux, o, idx);
    return n;
}

Ctx make_ctx(const orc_volume *v, const float *tf, int ntf, const orc_params *p) {
    Ctx c;
    c.vol = v;
    c.tf = reinterpret_cast<const F4 *>(tf);
    c.ntf = ntf;
    c.p = *p;
    c.bbox_min = f3(0, 0, 0);
    c.bbox_max = v->bbox_max;
    c.du = v->du;
    c.step = v->du / 4.f / p->sample_rate;  // basic_renderer.hpp:129
    c.max_steps = p->max_steps;
    return c;
}

}  // namespace

extern "C" int64_t orc_render_rows(const orc_volume *v, const float *tf, int32_t ntf,
                                   const orc_params *p, const float view[20], int32_t W,
                                   int32_t H, int32_t y0, int32_t y1, int32_t nthreads,
                                   float *v_out, uint8_t *rgba_out, float *aux_out,
                                   void *film_out) {
    if (!v || !p || !view || W <= 0 || H <= 0) return -1;
    if ((p->shader == 0) && (!tf || ntf <= 0)) return -1;
    Ctx c = make_ctx(v, tf, ntf, p);
    Out o{v_out, rgba_out, aux_out, film_out};
    if (nthreads <= 0) nthreads = int(std::thread::hardware_concurrency());
    if (nthreads <= 0) nthreads = 1;
    std::vector<int64_t> counts(nthreads, 0);
    std::vector<std::thread> threads;
    // cpu_shading.cc:9-31: thread i takes rows y = i, i + N, ...
    for (int i = 0; i < nthreads; ++i) {
        threads.emplace_back([&, i] {
            int64_t n = 0;
            for (int y = y0 + i; y < y1; y += nthreads)
                for (int x = 0; x < W; ++x) n += shade_pixel(c, view, x, y, W, H, o);
            counts[i] = n;
        });
    }
    for (auto &t : threads) t.join();
    int64_t total = 0;
    for (auto n : counts) total += n;
    return total;
}

// A bounded sample for the CPU baseline: rows y0, y0 + ystep, ... below y1,
// the m-th of them on thread m mod N (cpu_shading.cc's interleave over the
// sampled rows).
extern "C" int64_t orc_render_row_step(const orc_volume *v, const float *tf, int32_t ntf,
                                       const orc_params *p, const float view[20], int32_t W,
                                       int32_t H, int32_t y0, int32_t y1, int32_t ystep,
                                       int32_t nthreads, float *v_out, uint8_t *rgba_out) {
    if (!v || !p || !view || W <= 0 || H <= 0 || ystep <= 0) return -1;
    if ((p->shader == 0) && (!tf || ntf <= 0)) return -1;
    Ctx c = make_ctx(v, tf, ntf, p);
    Out o{v_out, rgba_out, nullptr, nullptr};
    if (nthreads <= 0) nthreads = int(std::thread::hardware_concurrency());
    if (nthreads <= 0) nthreads = 1;
    std::vector<int64_t> counts(nthreads, 0);
    std::vector<std::thread> threads;
    for (int i = 0; i < nthreads; ++i) {
        threads.emplace_back([&, i] {
            int64_t n = 0;
            for (long long y = y0 + (long long)i * ystep; y < y1; y += (long long)nthreads * ystep)
                for (int x = 0; x < W; ++x) n += shade_pixel(c, view, x, int(y), W, H, o);
            counts[i] = n;
        });
    }
    for (auto &t : threads) t.join();
    int64_t total = 0;
    for (auto n : counts) total += n;
    return total;
}

extern "C" int64_t orc_render(const orc_volume *v, const float *tf, int32_t ntf,
                              const orc_params *p, const float view[20], int32_t W, int32_t H,
                              int32_t nthreads, float *v_out, uint8_t *rgba_out, float *aux_out,
                              void *film_out) {
    return orc_render_rows(v, tf, ntf, p, view, W, H, 0, H, nthreads, v_out, rgba_out, aux_out,
                           film_out);
}

extern "C" int64_t orc_march_film(const orc_volume *v, const float *tf, int32_t ntf,
                                  const orc_params *p, int32_t W, int32_t H, int32_t nthreads,
                                  void *film) {
    if (!v || !p || !film || W <= 0 || H <= 0) return -1;
    Ctx c = make_ctx(v, tf, ntf, p);
    if (nthreads <= 0) nthreads = 1;
    std::vector<int64_t> counts(nthreads, 0);
    std::vector<std::thread> threads;
    // ray_march_shader_impl (shader.hpp:146-157) over every pixel
    for (int i = 0; i < nthreads; ++i) {
        threads.emplace_back([&, i] {
            int64_t n = 0;
            for (int y = i; y < H; y += nthreads)
                for (int x = 0; x < W; ++x) {
                    size_t idx = size_t(y) * W + x;
                    Px px;
                    read_film(c, px, film, idx);
                    n += run_main(c, px);
                    write_film(c, px, film, idx);
                }
            counts[i] = n;
        });
    }
    for (auto &t : threads) t.join();
    int64_t total = 0;
    for (auto n : counts) total += n;
    return total;
}

// ---------------------------------------------------------------------------
// Visible-brick culling: OctreeCuller::cull (octree_culler.hpp:121-161) with
// get_frustrum (324-345) and Frustum::contains / contains_fast (18-74).
// Reproduced as written, including that the frustum's border directions stay
// in camera space while its plane normals and origin are transformed to
// object space (octree_culler.hpp:329-343).  The selection of the nearest
// `limit` bricks breaks distance ties by brick index (std::nth_element leaves
// them unspecified), and the result is ordered by brick index (x fastest).
// ---------------------------------------------------------------------------
namespace {

struct Frustum {
    F3 norm[4];
    F3 border[4];
    F3 orig;
    bool contains(F3 p) const {
        return dot(norm[0], sub(p, orig)) > 0.f && dot(norm[1], sub(p, orig)) > 0.f &&
               dot(norm[2], sub(p, orig)) > 0.f && dot(norm[3], sub(p, orig)) > 0.f;
    }
    bool contains_fast(F3 mn, F3 mx) const {
        const F3 vp[2] = {mn, mx};
        for (int i = 0; i != 2; ++i)
            for (int j = 0; j != 2; ++j)
                for (int k = 0; k != 2; ++k)
                    if (contains(f3(vp[i].x, vp[j].y, vp[k].z))) return true;
        for (int i = 0; i != 4; ++i) {
            Ray r;
            r.o = orig;
            r.d = normalize(border[i]);
            float tnear, tfar;
            if (intersect(r, mn, mx, tnear, tfar) && tfar > 0.f) return true;
        }
        return false;
    }
};

Frustum make_frustum(const float view[20], const float rect[4]) {
    // rect = {min.x, min.y, max.x, max.y}
    Frustum f;
    const float ctg = view[16];
    f.border[0] = f3(rect[2], rect[3], -ctg);
    f.border[1] = f3(rect[2], rect[1], -ctg);
    f.border[2] = f3(rect[0], rect[1], -ctg);
    f.border[3] = f3(rect[0], rect[3], -ctg);
    f.orig = f3(0, 0, 0);
    f.norm[0] = cross(f.border[0], f.border[1]);
    f.norm[1] = cross(f.border[1], f.border[2]);
    f.norm[2] = cross(f.border[2], f.border[3]);
    f.norm[3] = cross(f.border[3], f.border[0]);
    M4 t;
    std::memcpy(t.m, view, sizeof(t.m));
    F4 o = mulv(t, F4{f.orig.x, f.orig.y, f.orig.z, 1.f});
    f.orig = f3(o.x, o.y, o.z);
    for (auto &n : f.norm) {
        F4 m = mulv(t, F4{n.x, n.y, n.z, 0.f});
        n = f3(m.x, m.y, m.z);
    }
    return f;
}

}  // namespace

extern "C" int32_t orc_cull(const orc_volume *v, const float view[20], const float rect_in[4],
                            int32_t limit, int32_t *ids_out, float *dist2_out) {
    const float def_rect[4] = {-1.f, -1.f, 1.f, 1.f};
    const float *rect = rect_in ? rect_in : def_rect;
    Frustum f = make_frustum(view, rect);
    struct Item {
        float d2;
        int id;
    };
    std::vector<Item> buf;
    for (int z = 0; z < v->grid[2]; ++z)
        for (int y = 0; y < v->grid[1]; ++y)
            for (int x = 0; x < v->grid[0]; ++x) {
                int id = (z * v->grid[1] + y) * v->grid[0] + x;
                if (v->cheb[id] != 0) continue;
                F3 mn = f3(float(x), float(y), float(z));
                F3 mx = f3(float(x + 1), float(y + 1), float(z + 1));
                if (f.contains_fast(mn, mx)) {
                    F3 c = f3(float(x) + .5f, float(y) + .5f, float(z) + .5f);
                    F3 d = sub(c, f.orig);
                    buf.push_back(Item{dot(d, d), id});
                }
            }
    size_t n = buf.size();
    if (limit >= 0 && size_t(limit) < n) {
        std::nth_element(buf.begin(), buf.begin() + limit, buf.end(), [](const Item &a, const Item &b) {
            return a.d2 < b.d2 || (a.d2 == b.d2 && a.id < b.id);
        });
        n = size_t(limit);
        buf.resize(n);
    }
    std::sort(buf.begin(), buf.end(), [](const Item &a, const Item &b) { return a.id < b.id; });
    for (size_t i = 0; i < n; ++i) {
        if (ids_out) ids_out[i] = buf[i].id;
        if (dist2_out) dist2_out[i] = buf[i].d2;
    }
    return int32_t(n);
}

// LosslessBlockPagingServer::start (lossless_block_paging.cc:116-135): the
// visible bricks ordered by the distance of their centres to
// cp = inverse(iet) * camera position -- the inverse exhibit transform, as
// the reference writes it -- with ties broken by brick index.
extern "C" void orc_lossless_order(const orc_volume *v, const float cam[10], const int32_t *ids,
                                   int32_t n, int32_t *order_out) {
    M4 et = inverse(exhibit_iet(v));
    F4 c4 = mulv(et, F4{cam[0], cam[1], cam[2], 1.f});
    F3 cp = f3(c4.x, c4.y, c4.z);
    std::vector<std::pair<float, int>> d(n);
    for (int i = 0; i < n; ++i) {
        int id = ids[i];
        int x = id % v->grid[0], y = (id / v->grid[0]) % v->grid[1], z = id / (v->grid[0] * v->grid[1]);
        F3 c = f3(float(x) + 0.5f, float(y) + 0.5f, float(z) + 0.5f);
        d[i] = {length(sub(c, cp)), id};
    }
    std::sort(d.begin(), d.end());
    for (int i = 0; i < n; ++i) order_out[i] = d[i].second;
}

// ---------------------------------------------------------------------------
// Differentiable Volume march (one dense brick of n^3 voxels, 1-voxel
// replicate apron; step_size fixed at 1, no empty-space skipping).  The float
// version uses the reference's float operations and is the forward parity
// target; the double version, with its analytic gradient, is the FP64
// reference gradient.  Loss L = sum over pixels and RGBA of (v - target)^2.
// ---------------------------------------------------------------------------
namespace {

template <typename T>
struct DiffCtx {
    const T *vol;
    int n;
    T k, b, step, density;
    const T *tf;  // ntf * 4
    int ntf;
    int max_steps;
};

template <typename T>
T dfloor(T x) { return std::floor(x); }

// sample at brick-local l in [0,1]; fills raw indices and weights
template <typename T>
T diff_sample(const DiffCtx<T> &c, const T l[3], long long idx[8], T w[8]) {
    const int P = c.n + 2;
    const T fd = T(P);
    T a[3];
    int i0[3], i1[3];
    for (int ax = 0; ax < 3; ++ax) {
        T f = fd * (c.k * l[ax] + c.b);
        f = f - fd * dfloor(f / fd);  // Wrap (identity for l in [0,1])
        const T u = f - T(0.5);
        const T flr = dfloor(u);
        a[ax] = u - flr;
        const int ix = iclamp(f2i(float(flr)), 0, P - 1);
        const int jx = iclamp(f2i(float(std::ceil(u))), 0, P - 1);
        i0[ax] = iclamp(ix - 1, 0, c.n - 1);
        i1[ax] = iclamp(jx - 1, 0, c.n - 1);
    }
    auto at = [&](int X, int Y, int Z) {
        return (long long)(Z * (long long)c.n + Y) * c.n + X;
    };
    const long long id[8] = {at(i0[0], i0[1], i0[2]), at(i1[0], i0[1], i0[2]),
                             at(i0[0], i1[1], i0[2]), at(i1[0], i1[1], i0[2]),
                             at(i0[0], i0[1], i1[2]), at(i1[0], i0[1], i1[2]),
                             at(i0[0], i1[1], i1[2]), at(i1[0], i1[1], i1[2])};
    const T bx = T(1) - a[0], by = T(1) - a[1], bz = T(1) - a[2];
    const T x0_0 = c.vol[id[0]] * bx + c.vol[id[1]] * a[0];
    const T x1_0 = c.vol[id[2]] * bx + c.vol[id[3]] * a[0];
    const T x0_1 = c.vol[id[4]] * bx + c.vol[id[5]] * a[0];
    const T x1_1 = c.vol[id[6]] * bx + c.vol[id[7]] * a[0];
    const T y0 = x0_0 * by + x1_0 * a[1];
    const T y1 = x0_1 * by + x1_1 * a[1];
    if (idx) {
        const T ww[8] = {bx * by * bz,   a[0] * by * bz,   bx * a[1] * bz,   a[0] * a[1] * bz,
                         bx * by * a[2], a[0] * by * a[2], bx * a[1] * a[2], a[0] * a[1] * a[2]};
        for (int t = 0; t < 8; ++t) {
            idx[t] = id[t];
            w[t] = ww[t];
        }
    }
    return y0 * bz + y1 * a[2];
}

template <typename T>
void diff_tf(const DiffCtx<T> &c, T s, T q[4], int &i, int &j, T &al, bool &inb) {
    const T fn = T(c.ntf);
    const T fx = fn * s;
    inb = (T(0) <= fx && fx <= fn);
    if (!inb) {
        q[0] = q[1] = q[2] = q[3] = T(0);
        i = j = 0;
        al = T(0);
        return;
    }
    const T u = fx - T(0.5);
    const T flr = dfloor(u);
    al = u - flr;
    i = iclamp(f2i(float(flr)), 0, c.ntf - 1);
    j = iclamp(f2i(float(std::ceil(u))), 0, c.ntf - 1);
    for (int ch = 0; ch < 4; ++ch)
        q[ch] = c.tf[4 * i + ch] * (T(1) - al) + c.tf[4 * j + ch] * al;
}

// ray for pixel (x, y) of a view; returns nsteps, sets o, d
template <typename T>
int diff_ray(const DiffCtx<T> &c, const float view[20], int x, int y, int W, int H, T o[3],
             T d[3]) {
    const T ccx = T(W) / T(2), ccy = T(H) / T(2);
    const T ux = (T(x) - ccx) * T(2) / T(H);
    const T uy = (T(y) - ccy) * T(2) / T(H);
    const T v4[4] = {ux, -uy, -T(view[16]), T(1)};
    T p[3];
    for (int r = 0; r < 3; ++r)
        p[r] = T(view[r]) * v4[0] + T(view[4 + r]) * v4[1] + T(view[8 + r]) * v4[2] +
               T(view[12 + r]) * v4[3];
    for (int r = 0; r < 3; ++r) {
        o[r] = T(view[17 + r]);
        d[r] = p[r] - o[r];
    }
    const T inv = T(1) / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int r = 0; r < 3; ++r) d[r] = d[r] * inv;
    // slab test against [0,1]^3
    T tn = -INFINITY, tf = INFINITY;
    T tmin[3], tmax[3];
    for (int r = 0; r < 3; ++r) {
        const T ir = T(1) / d[r];
        const T tb = ir * (T(0) - o[r]), tt = ir * (T(1) - o[r]);
        tmin[r] = (tb < tt) ? tb : tt;
        tmax[r] = (tt < tb) ? tb : tt;
    }
    tn = tmin[0];
    tn = (tn < tmin[1]) ? tmin[1] : tn;
    tn = (tn < tmin[2]) ? tmin[2] : tn;
    tf = tmax[0];
    tf = (tmax[1] < tf) ? tmax[1] : tf;
    tf = (tmax[2] < tf) ? tmax[2] : tf;
    if (!(tf > tn)) return 0;
    if (tn < 0) tn = 0;
    if (tf < 0) tf = 0;
    for (int r = 0; r < 3; ++r) o[r] = o[r] + d[r] * tn;
    return imin(c.max_steps, f2i(float((tf - tn) / c.step)));
}

template <typename T>
void diff_pixel(const DiffCtx<T> &c, const float view[20], int x, int y, int W, int H, T v[4]) {
    T o[3], d[3];
    const int ns = diff_ray(c, view, x, y, W, H, o, d);
    v[0] = v[1] = v[2] = v[3] = T(0);
    const T s3[3] = {d[0] * c.step, d[1] * c.step, d[2] * c.step};
    for (int s = 0; s < ns; ++s) {
        const T l[3] = {o[0] - dfloor(o[0]), o[1] - dfloor(o[1]), o[2] - dfloor(o[2])};
        const T val = diff_sample<T>(c, l, nullptr, nullptr);
        T q[4];
        int i, j;
        T al;
        bool inb;
        diff_tf(c, val, q, i, j, al, inb);
        q[3] = q[3] * c.density;
        const T w = q[3];
        const T ub[4] = {q[0] * w, q[1] * w, q[2] * w, q[3]};
        const T t = T(1) - v[3];
        for (int ch = 0; ch < 4; ++ch) v[ch] = v[ch] + ub[ch] * t;
        for (int r = 0; r < 3; ++r) o[r] = o[r] + s3[r];
    }
}

// FP64 adjoint of one pixel: g = dL/dv; accumulates into dvol / dtf.
void diff_pixel_grad(const DiffCtx<double> &c, const float view[20], int x, int y, int W, int H,
                     const double g[4], double *dvol, double *dtf) {
    double o[3], d[3];
    const int ns = diff_ray(c, view, x, y, W, H, o, d);
    const double s3[3] = {d[0] * c.step, d[1] * c.step, d[2] * c.step};
    std::vector<double> pw(ns), P(3 * size_t(ns));
    double vw = 0;
    for (int s = 0; s < ns; ++s) {
        for (int r = 0; r < 3; ++r) P[3 * s + r] = o[r];
        pw[s] = vw;
        const double l[3] = {o[0] - std::floor(o[0]), o[1] - std::floor(o[1]), o[2] - std::floor(o[2])};
        double q[4];
        int i, j;
        double al;
        bool inb;
        diff_tf(c, diff_sample<double>(c, l, nullptr, nullptr), q, i, j, al, inb);
        const double a = q[3] * c.density;
        vw = vw + a * (1.0 - vw);
        for (int r = 0; r < 3; ++r) o[r] = o[r] + s3[r];
    }
    double R[4] = {0, 0, 0, 0};
    for (int s = ns - 1; s >= 0; --s) {
        const double l[3] = {P[3 * s] - std::floor(P[3 * s]), P[3 * s + 1] - std::floor(P[3 * s + 1]),
                             P[3 * s + 2] - std::floor(P[3 * s + 2])};
        long long idx[8];
        double w[8];
        const double val = diff_sample(c, l, idx, w);
        double q[4];
        int i, j;
        double al;
        bool inb;
        diff_tf(c, val, q, i, j, al, inb);
        const double a = q[3] * c.density;
        const double T = 1.0 - pw[s];
        const double gc[4] = {T * g[0], T * g[1], T * g[2], T * g[3]};
        const double gdot = g[0] * R[0] + g[1] * R[1] + g[2] * R[2] + g[3] * R[3];
        const double da = gc[0] * q[0] + gc[1] * q[1] + gc[2] * q[2] + gc[3] - T * gdot;
        const double om = 1.0 - a;
        R[0] = q[0] * a + om * R[0];
        R[1] = q[1] * a + om * R[1];
        R[2] = q[2] * a + om * R[2];
        R[3] = a + om * R[3];
        if (!inb) continue;
        const double gq[4] = {gc[0] * a, gc[1] * a, gc[2] * a, da * c.density};
        double ds = 0;
        for (int ch = 0; ch < 4; ++ch) {
            dtf[4 * i + ch] += gq[ch] * (1.0 - al);
            dtf[4 * j + ch] += gq[ch] * al;
            ds += gq[ch] * (c.tf[4 * j + ch] - c.tf[4 * i + ch]);
        }
        ds *= double(c.ntf);
        for (int t = 0; t < 8; ++t) dvol[idx[t]] += ds * w[t];
    }
}

template <typename T>
DiffCtx<T> diff_ctx(const T *vol, int n, const T *tf, int ntf, float sample_rate, int max_steps,
                    float density) {
    DiffCtx<T> c;
    c.vol = vol;
    c.n = n;
    c.k = T(n) / T(n + 2);
    c.b = T(1) / T(n) * c.k;
    const T du = T(1) / T(n);
    c.step = du / T(4) / T(sample_rate);
    c.density = T(density);
    c.tf = tf;
    c.ntf = ntf;
    c.max_steps = max_steps;
    return c;
}

}  // namespace

extern "C" void orc_diff_forward(const float *vol, int32_t n, const float *tf, int32_t ntf,
                                 float sample_rate, int32_t max_steps, float density,
                                 const float *views, int32_t nviews, int32_t W, int32_t H,
                                 int32_t nthreads, float *image) {
    DiffCtx<float> c = diff_ctx<float>(vol, n, tf, ntf, sample_rate, max_steps, density);
    if (nthreads <= 0) nthreads = 1;
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t] {
            for (int row = t; row < nviews * H; row += nthreads) {
                const int v = row / H, y = row % H;
                for (int x = 0; x < W; ++x)
                    diff_pixel(c, views + 20 * v, x, y, W, H,
                               image + ((size_t(v) * H + y) * W + x) * 4);
            }
        });
    for (auto &x : th) x.join();
}

extern "C" double orc_diff_loss_grad64(const double *vol, int32_t n, const double *tf, int32_t ntf,
                                       float sample_rate, int32_t max_steps, float density,
                                       const float *views, int32_t nviews, int32_t W, int32_t H,
                                       const double *target, double *image, double *dvol,
                                       double *dtf) {
    DiffCtx<double> c = diff_ctx<double>(vol, n, tf, ntf, sample_rate, max_steps, density);
    double loss = 0;
    for (int v = 0; v < nviews; ++v)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                const size_t px = (size_t(v) * H + y) * W + x;
                double pv[4];
                diff_pixel(c, views + 20 * v, x, y, W, H, pv);
                double g[4];
                for (int ch = 0; ch < 4; ++ch) {
                    const double r = pv[ch] - (target ? target[px * 4 + ch] : 0.0);
                    loss += r * r;
                    g[ch] = 2.0 * r;
                    if (image) image[px * 4 + ch] = pv[ch];
                }
                if (dvol && dtf) diff_pixel_grad(c, views + 20 * v, x, y, W, H, g, dvol, dtf);
            }
    return loss;
}
