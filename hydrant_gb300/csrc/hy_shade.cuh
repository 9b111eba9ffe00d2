// hy_shade.cuh -- per-ray device code of the ray-marching path.
//
// Translation units that include this file are compiled with -fmad=false,
// -prec-div=true, -prec-sqrt=true, -ftz=false: each multiply and add rounds
// separately and divisions and square roots are IEEE, so a ray marched here
// takes the same steps and produces the same floats as the reference's CPU
// backend (the __host__ __device__ shaders run through CpuSampler).  Where a
// shortcut is taken it is exact; each one says why.
//
// Conventions: min(a,b) = (b < a) ? b : a and max(a,b) = (a < b) ? b : a
// (the forms the reference's math library uses); sums run left to right.
#pragma once

#include "hy_internal.h"

namespace hy {
namespace dev {

__device__ __forceinline__ float gmin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float gmax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ int iclamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
__device__ __forceinline__ float fclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ float fsign(float x) { return float((0.f < x) - (x < 0.f)); }
// float -> int: truncation, saturating, NaN -> 0 (the hardware conversion;
// the oracle defines the same, C++ leaves these cases undefined).
__device__ __forceinline__ int f2i(float x) { return int(x); }

// Two-lane float arithmetic (sm_100 and later).  Each lane rounds exactly as
// the scalar __fmul_rn / __fadd_rn / __fmaf_rn does, so packing two
// independent operations of the march changes no result, only the number of
// instructions issued.  There is no packed subtract: a - b is fma(b, -1, a),
// whose product is exact, so its one rounding is that of a - b (signed zeros,
// infinities and NaN included).
// One rule keeps it exact: a packed product is never an operand of a packed
// add.  The assembler fuses a packed multiply whose only use is a packed add
// (or fma(p, 1, q)) into one fused multiply-add, even for .rn instructions
// and with contraction disabled -- measured on GB300: 161,347 of 2,097,152
// lanes of fl(fl(a*b) + fl(c*d)) came out fused, while packed products summed
// by scalar adds, and scalar products summed by a packed add, matched bit for
// bit.  So products here are summed by scalar __fadd_rn.  HY_F32X2=0 builds
// the scalar forms.
#ifndef HY_F32X2
#define HY_F32X2 1
#endif
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// x * w + y * v per lane, products rounded separately (the reference's lerp
// x*(1-a) + y*a with w = 1-a, v = a): packed products, scalar sums
__device__ __forceinline__ float2 lerp2(float2 x, float2 w, float2 y, float2 v) {
    const float2 p = mul2(x, w), q = mul2(y, v);
    return f2(__fadd_rn(p.x, q.x), __fadd_rn(p.y, q.y));
}
// Steps skipped over empty bricks.  The reference's value is a small
// non-negative integer; NaN / negative / huge (degenerate rays only) are
// pinned to [0, 2^30] so nsteps can never overflow and the loop always ends.
__device__ __forceinline__ int skip_count(float di) {
    return (di >= 0.f) ? (di < 1073741824.f ? int(di) : 1073741824) : 0;
}

// IPixel + StdVec4Pixel + shader extras (shader.hpp:26-34,
// pixel_template.hpp:11-20, volume_shader.hpp:11-15, isosurface_shader.hpp:11-15).
// e0..e2: theta (Volume) or origin (Isosurface); e3: phi (Volume) or depth.
struct Px {
    float ox, oy, oz, dx, dy, dz;
    int nsteps, step_size;
    float vx, vy, vz, vw;
    float e0, e1, e2, e3;
};

// Slab test (glm_math.hpp:58-72) with the reciprocal direction precomputed
// (1/d is the same value on every call, so caching it is exact).
__device__ __forceinline__ bool intersect(float ox, float oy, float oz, float rx, float ry,
                                          float rz, float x0, float y0, float z0, float x1,
                                          float y1, float z1, float &tnear, float &tfar) {
    float tbx = rx * (x0 - ox), tby = ry * (y0 - oy), tbz = rz * (z0 - oz);
    float ttx = rx * (x1 - ox), tty = ry * (y1 - oy), ttz = rz * (z1 - oz);
    float nx = gmin(ttx, tbx), ny = gmin(tty, tby), nz = gmin(ttz, tbz);
    float fx = gmax(ttx, tbx), fy = gmax(tty, tby), fz = gmax(ttz, tbz);
    tnear = gmax(gmax(nx, ny), nz);
    tfar = gmin(gmin(fx, fy), fz);
    return tfar > tnear;
}

// Thumbnail / page-table lookup: non-normalised nearest texel with Clamp
// (cpu_sampler.hpp:142-166, filter_none 72-76).  ip is integral and the
// clamp bounds are integers, so floor() after the clamp is the identity.
// In float arithmetic with one conversion at the end: fmaxf(ip, 0) maps NaN
// to 0 (as the integer conversion of NaN does), clamping to [0, g - 1]
// equals clamping to [0, g] and the index then to g - 1, and the index sum
// is of whole numbers below 2^24 -- every step is exact.
__device__ __forceinline__ int thumb_index(const DevVolume &V, float ipx, float ipy, float ipz) {
    const float x = fminf(fmaxf(ipx, 0.f), V.gmx), y = fminf(fmaxf(ipy, 0.f), V.gmy),
                z = fminf(fmaxf(ipz, 0.f), V.gmz);
    return int((z * V.fgy + y) * V.fgx + x);
}

// skip_nblock_steps (volume_shader.cu:5-14, same in blocks/isosurface).
__device__ __forceinline__ int skip_nblock_steps(Px &p, float rx, float ry, float rz, float ipx,
                                                 float ipy, float ipz, int nblocks, float cdu,
                                                 float step) {
    float tnear, tfar;
    intersect(p.ox, p.oy, p.oz, rx, ry, rz, ipx, ipy, ipz, ipx + 1.f, ipy + 1.f, ipz + 1.f, tnear,
              tfar);
    float di = ceilf((tfar + float(nblocks - 1) * cdu) / step);
    p.ox = p.ox + (p.dx * di) * step;
    p.oy = p.oy + (p.dy * di) * step;
    p.oz = p.oz + (p.dz * di) * step;
    return skip_count(di);
}

// A resident brick: BlockSampler {storage, mapping} (block_paging.hpp:24-36);
// with GATHER its gather texture (which) and texel origin (TexEntry) instead
// of the pool address.
struct BrickRef {
    const unsigned char *base;
    float k, bx, by, bz;
    float tx, ty;
    int which;
};

// Samplers of the march: the brick pool by loads, the resident bricks'
// gather textures (one mapping for every brick, at most two textures), or a
// paged cache held in gather textures (each registry entry's own mapping --
// the coarse fallback reads a sub-box of a coarse brick -- and up to
// kMaxGatherTextures textures).
constexpr int kGatherNone = 0, kGatherResident = 1, kGatherPaged = 2;

__device__ __forceinline__ BrickRef load_brick(const DevVolume &V, int reg) {
    const float4 *e = reinterpret_cast<const float4 *>(V.reg + reg);
    float4 m = __ldg(e);
    float4 o = __ldg(e + 1);
    long long off = (long long)__float_as_uint(o.x) | ((long long)__float_as_uint(o.y) << 32);
    return BrickRef{V.pool + off, m.x, m.y, m.z, m.w, 0.f, 0.f, 0};
}

// A paged registry entry in gather textures: the mapping, and in the
// entry's last two words its texel origin + 1: (texture << 16 | x0 + 1,
// y0 + 1).  The pool offset stays 0 (a one-slot pool of zeros).
__device__ __forceinline__ BrickRef load_brick_paged(const DevVolume &V, int reg) {
    const float4 *e = reinterpret_cast<const float4 *>(V.reg + reg);
    const float4 m = __ldg(e);
    const int4 o = __ldg(reinterpret_cast<const int4 *>(e + 1));
    return BrickRef{nullptr, m.x, m.y, m.z, m.w, float(o.z & 0xffff), float(o.w),
                    (o.z >> 16) & (kMaxGatherTextures - 1)};
}

// Brick sample: BlockSampler::sample_3d -> CpuSampler with normalised
// coordinates, Wrap and Linear (cpu_sampler.hpp:88-104, 126-129, 142-166).
//  * Wrap is mod(f, P) = f - P*floor(f/P), which is f itself for 0 <= f < P;
//    only the out-of-range case pays for the division.
//  * With the lower corner i = floor(u) in [0, P-2] every neighbour index is
//    unclamped and the upper one is i+1 -- or i when u is integral, where the
//    weight a is 0 and x*(1-0) + y*0 == x for any finite y, so reading i+1
//    gives the same float.  Offsets are then immediates when P is a
//    compile-time constant.
// U8 voxels are normalised with lut[u] = u / 255.f (texture_3d.hpp:78-86).
//
// INTERIOR: the caller guarantees brick-local coordinates in [0,1] (the main
// loops sample at o - floor(o)) and an apron of at least one voxel.  Then
// f = P*(k*x + b) lies in [pad, bs+pad] (up to rounding far below 0.5), so
// Wrap is the identity and floor(f - 0.5) is in [pad-1, bs+pad-1] within
// [0, P-2]: both range checks are known to pass and are left out.
// u / 255.f for a u8 voxel without the table: 1/255 as an unevaluated sum
// hi + lo of two floats (hi = fl(1/255), lo = fl(1/255 - hi)) and
// q = fma(u, hi, u * lo) (multiplication by a constant carried in two words,
// Brisebarre & Muller 2008).  The exact quotient u/255 repeats u's 8 bits,
// so it lies at least 1/510 ulp from a rounding boundary while hi + lo and
// the rounding of u * lo are off by ~2^-48: q is the correctly rounded
// quotient for every u in 0..255 (also checked exhaustively,
// tests/test_u8_normalisation.py).  The interior sampler normalises every
// tap this way (two taps per packed instruction); in the scalar build
// (HY_F32X2=0) taps below HY_U8_ARITH_TAPS do, the others read the
// shared-memory table (whose lookups conflict on banks when neighbouring
// lanes read distant values) -- all eight arithmetic measured fastest.
#ifndef HY_U8_ARITH_TAPS
#define HY_U8_ARITH_TAPS 8
#endif
__device__ __forceinline__ float u8_norm(unsigned int u) {
    constexpr float hi = 1.f / 255.f;
    constexpr float lo = float(1.0 / 255.0 - double(1.f / 255.f));
    const float x = __uint2float_rn(u);
    return __fmaf_rn(x, hi, __fmul_rn(x, lo));
}
// two voxels at once, same operations per lane
__device__ __forceinline__ float2 u8_norm2(unsigned int a, unsigned int b) {
    constexpr float hi = 1.f / 255.f;
    constexpr float lo = float(1.0 / 255.0 - double(1.f / 255.f));
    const float2 x = f2(__uint2float_rn(a), __uint2float_rn(b));
    return fma2(x, f2(hi, hi), mul2(x, f2(lo, lo)));
}
__device__ __forceinline__ float lut_at(const float *__restrict__ lut, unsigned int u) {
    return lut[u];
}
template <int TAP>
__device__ __forceinline__ float u8_value(unsigned char u, const float *__restrict__ lut) {
    return TAP < HY_U8_ARITH_TAPS ? u8_norm(u) : lut_at(lut, u);
}

// The lerps of a trilinear sample (cpu_sampler.hpp:88-104, do_lerp
// x*(1-a) + y*a): the taps in z pairs, c<y><x> = (tap at layer z, tap at
// layer z + 1), fractions axy = (ax, ay) and az.
__device__ __forceinline__ float trilerp(float2 c00, float2 c01, float2 c10, float2 c11,
                                         float2 axy, float az) {
#if HY_F32X2
    // lerp along x of both z layers at once, then along y, then z:
    // X0 = (x0_0, x0_1), X1 = (x1_0, x1_1), Y = (y0, y1)
    const float2 bxy = sub2(f2(1.f, 1.f), axy);
    const float bz = 1.f - az;
    const float2 bx2 = f2(bxy.x, bxy.x), ax2 = f2(axy.x, axy.x);
    const float2 X0 = lerp2(c00, bx2, c01, ax2);
    const float2 X1 = lerp2(c10, bx2, c11, ax2);
    const float2 Y = lerp2(X0, f2(bxy.y, bxy.y), X1, f2(axy.y, axy.y));
    const float2 Z = mul2(Y, f2(bz, az));
    return __fadd_rn(Z.x, Z.y);
#else
    const float ax = axy.x, ay = axy.y;
    const float bx = 1.f - ax, by = 1.f - ay, bz = 1.f - az;
    float x0_0 = c00.x * bx + c01.x * ax;
    float x1_0 = c10.x * bx + c11.x * ax;
    float x0_1 = c00.y * bx + c01.y * ax;
    float x1_1 = c10.y * bx + c11.y * ax;
    float y0 = x0_0 * by + x1_0 * ay;
    float y1 = x0_1 * by + x1_1 * ay;
    return y0 * bz + y1 * az;
#endif
}

template <int PC, int DT, bool INTERIOR = false>
__device__ __forceinline__ float sample_brick(const BrickRef &b, int Prt, float lx, float ly,
                                              float lz, const float *__restrict__ lut) {
    const int P = PC ? PC : Prt;
    const float fd = float(P);
#if HY_F32X2
    // x and y in packed pairs, z alone; per lane the scalar sequence below
    const float2 kl = mul2(f2(b.k, b.k), f2(lx, ly));
    const float2 fxy0 = mul2(f2(fd, fd), f2(__fadd_rn(kl.x, b.bx), __fadd_rn(kl.y, b.by)));
    float fx = fxy0.x, fy = fxy0.y, fz = fd * (b.k * lz + b.bz);
#else
    float mx = b.k * lx + b.bx, my = b.k * ly + b.by, mz = b.k * lz + b.bz;
    float fx = fd * mx, fy = fd * my, fz = fd * mz;
#endif
    if (!INTERIOR) {
        if (!(fx >= 0.f && fx < fd)) fx = fx - fd * floorf(fx / fd);
        if (!(fy >= 0.f && fy < fd)) fy = fy - fd * floorf(fy / fd);
        if (!(fz >= 0.f && fz < fd)) fz = fz - fd * floorf(fz / fd);
    }
#if HY_F32X2
    const float ux = fx - .5f, uy = fy - .5f, uz = fz - .5f;  // fx, fy are products
    const float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
    const float2 axy = sub2(f2(ux, uy), f2(flx, fly));
    const float az = uz - flz;
#else
    float ux = fx - .5f, uy = fy - .5f, uz = fz - .5f;
    float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
    float ax = ux - flx, ay = uy - fly, az = uz - flz;
#endif
    int ix = int(flx), iy = int(fly), iz = int(flz);
    // the eight taps in z pairs: c<y><x> holds the taps at (x, y) of layers z and z+1
    float2 c00, c01, c10, c11;
    if (INTERIOR ||
        (ix >= 0 && ix <= P - 2 && iy >= 0 && iy <= P - 2 && iz >= 0 && iz <= P - 2)) {
        // a compile-time brick edge (<= 130) keeps the offset in 32 bits
        const long long base = PC ? (long long)((iz * PC + iy) * PC + ix)
                                  : ((long long)iz * P + iy) * P + ix;
        if (DT == HY_DTYPE_U8) {
            const unsigned char *q = b.base + base;
#if HY_F32X2
            c00 = u8_norm2(__ldg(q), __ldg(q + P * P));
            c01 = u8_norm2(__ldg(q + 1), __ldg(q + P * P + 1));
            c10 = u8_norm2(__ldg(q + P), __ldg(q + P * P + P));
            c11 = u8_norm2(__ldg(q + P + 1), __ldg(q + P * P + P + 1));
#else
            c00.x = u8_value<0>(__ldg(q), lut);
            c01.x = u8_value<1>(__ldg(q + 1), lut);
            c10.x = u8_value<2>(__ldg(q + P), lut);
            c11.x = u8_value<3>(__ldg(q + P + 1), lut);
            c00.y = u8_value<4>(__ldg(q + P * P), lut);
            c01.y = u8_value<5>(__ldg(q + P * P + 1), lut);
            c10.y = u8_value<6>(__ldg(q + P * P + P), lut);
            c11.y = u8_value<7>(__ldg(q + P * P + P + 1), lut);
#endif
        } else {
            const float *q = reinterpret_cast<const float *>(b.base) + base;
            c00 = f2(__ldg(q), __ldg(q + P * P));
            c01 = f2(__ldg(q + 1), __ldg(q + P * P + 1));
            c10 = f2(__ldg(q + P), __ldg(q + P * P + P));
            c11 = f2(__ldg(q + P + 1), __ldg(q + P * P + P + 1));
        }
    } else {
        int jx = iclamp(int(ceilf(ux)), 0, P - 1), jy = iclamp(int(ceilf(uy)), 0, P - 1),
            jz = iclamp(int(ceilf(uz)), 0, P - 1);
        ix = iclamp(ix, 0, P - 1);
        iy = iclamp(iy, 0, P - 1);
        iz = iclamp(iz, 0, P - 1);
        const long long r00 = ((long long)iz * P + iy) * P, r10 = ((long long)iz * P + jy) * P,
                        r01 = ((long long)jz * P + iy) * P, r11 = ((long long)jz * P + jy) * P;
        if (DT == HY_DTYPE_U8) {
            const unsigned char *q = b.base;
            c00 = f2(lut_at(lut, __ldg(q + r00 + ix)), lut_at(lut, __ldg(q + r01 + ix)));
            c01 = f2(lut_at(lut, __ldg(q + r00 + jx)), lut_at(lut, __ldg(q + r01 + jx)));
            c10 = f2(lut_at(lut, __ldg(q + r10 + ix)), lut_at(lut, __ldg(q + r11 + ix)));
            c11 = f2(lut_at(lut, __ldg(q + r10 + jx)), lut_at(lut, __ldg(q + r11 + jx)));
        } else {
            const float *q = reinterpret_cast<const float *>(b.base);
            c00 = f2(__ldg(q + r00 + ix), __ldg(q + r01 + ix));
            c01 = f2(__ldg(q + r00 + jx), __ldg(q + r01 + jx));
            c10 = f2(__ldg(q + r10 + ix), __ldg(q + r11 + ix));
            c11 = f2(__ldg(q + r10 + jx), __ldg(q + r11 + jx));
        }
    }
#if HY_F32X2
    return trilerp(c00, c01, c10, c11, axy, az);
#else
    return trilerp(c00, c01, c10, c11, f2(ax, ay), az);
#endif
}

#ifndef HY_GATHER_ROWS
#define HY_GATHER_ROWS 1
#endif
// Brick sample through the brick's gather texture (interior case only, the
// same arithmetic as sample_brick<PC, HY_DTYPE_U8, true>): the texel
// coordinates of the footprint are whole numbers, so the two gathers fetch
// exactly the taps the loads would, already normalised (u / 255, checked
// per device when the textures are built).
// The two gathers of a footprint from the volume's texture `which`: each
// branch names a handle from the kernel parameters, so the texture is
// warp-uniform in each (lanes in bricks of different textures take both).
__device__ __forceinline__ void gather2(const DevVolume &V, int which, float X, float Y, float fd,
                                        float4 &g0, float4 &g1) {
    // Warp-uniform first: when every lane's brick is in the same texture
    // the warp issues one pair of gathers (otherwise the compiler predicates
    // both textures' gathers): 64-view step 140.0 vs 149.0 ms.
    const unsigned int m = __activemask();
    if (__all_sync(m, which == 0)) {
        g0 = gather_r(V.gtex[0], X, Y);
        g1 = gather_r(V.gtex[0], X, Y + fd);
        return;
    }
    if (__all_sync(m, which != 0)) {
        g0 = gather_r(V.gtex[1], X, Y);
        g1 = gather_r(V.gtex[1], X, Y + fd);
        return;
    }
    if (which == 0) {
        g0 = gather_r(V.gtex[0], X, Y);
        g1 = gather_r(V.gtex[0], X, Y + fd);
    } else {
        g0 = gather_r(V.gtex[1], X, Y);
        g1 = gather_r(V.gtex[1], X, Y + fd);
    }
}

// The two gathers of a footprint from texture `which` of a paged cache.
// When every lane of the warp reads the same texture, a switch names its
// handle as a constant; otherwise the handle is indexed from the kernel
// parameters (every entry holds a valid handle) and the compiler issues the
// gathers once per distinct texture among the lanes.  Out-of-core orbit:
// 47.0 frames/s, against 46.3 with the indexed handle alone and 42.6-43.5
// for the cache in a pool read by loads.
template <int K>
__device__ __forceinline__ void gather2_const(const DevVolume &V, float X, float Y, float fd,
                                              float4 &g0, float4 &g1) {
    g0 = gather_r(V.gtex[K], X, Y);
    g1 = gather_r(V.gtex[K], X, Y + fd);
}
__device__ __forceinline__ void gather2_indexed(const DevVolume &V, int which, float X, float Y,
                                                float fd, float4 &g0, float4 &g1) {
    const unsigned int m = __activemask();
    const int w0 = __shfl_sync(m, which, __ffs(m) - 1);
    if (__all_sync(m, which == w0)) {
        switch (w0) {
            case 0: gather2_const<0>(V, X, Y, fd, g0, g1); return;
            case 1: gather2_const<1>(V, X, Y, fd, g0, g1); return;
            case 2: gather2_const<2>(V, X, Y, fd, g0, g1); return;
            case 3: gather2_const<3>(V, X, Y, fd, g0, g1); return;
            case 4: gather2_const<4>(V, X, Y, fd, g0, g1); return;
            case 5: gather2_const<5>(V, X, Y, fd, g0, g1); return;
            case 6: gather2_const<6>(V, X, Y, fd, g0, g1); return;
            case 7: gather2_const<7>(V, X, Y, fd, g0, g1); return;
            case 8: gather2_const<8>(V, X, Y, fd, g0, g1); return;
            case 9: gather2_const<9>(V, X, Y, fd, g0, g1); return;
            case 10: gather2_const<10>(V, X, Y, fd, g0, g1); return;
            case 11: gather2_const<11>(V, X, Y, fd, g0, g1); return;
            case 12: gather2_const<12>(V, X, Y, fd, g0, g1); return;
            case 13: gather2_const<13>(V, X, Y, fd, g0, g1); return;
            case 14: gather2_const<14>(V, X, Y, fd, g0, g1); return;
            default: gather2_const<15>(V, X, Y, fd, g0, g1); return;
        }
    }
    const unsigned long long h = V.gtex[which];
    g0 = gather_r(h, X, Y);
    g1 = gather_r(h, X, Y + fd);
}

template <int PC, int GATHER = kGatherResident>
__device__ __forceinline__ float sample_brick_gather(const DevVolume &V, const BrickRef &b,
                                                     int Prt, float lx, float ly, float lz) {
    const int P = PC ? PC : Prt;
    const float fd = float(P);
    // every resident brick's mapping, or the paged registry entry's
    const float k = GATHER == kGatherPaged ? b.k : V.map_k;
    const float mbx = GATHER == kGatherPaged ? b.bx : V.map_b;
    const float mby = GATHER == kGatherPaged ? b.by : V.map_b;
    const float mbz = GATHER == kGatherPaged ? b.bz : V.map_b;
#if HY_F32X2
    const float2 kl = mul2(f2(k, k), f2(lx, ly));
    const float2 fxy0 = mul2(f2(fd, fd), f2(__fadd_rn(kl.x, mbx), __fadd_rn(kl.y, mby)));
    const float fx = fxy0.x, fy = fxy0.y, fz = fd * (k * lz + mbz);
    const float ux = fx - .5f, uy = fy - .5f, uz = fz - .5f;
    const float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
    const float2 axy = sub2(f2(ux, uy), f2(flx, fly));
    const float az = uz - flz;
#else
    const float mx = k * lx + mbx, my = k * ly + mby, mz = k * lz + mbz;
    const float fx = fd * mx, fy = fd * my, fz = fd * mz;
    const float ux = fx - .5f, uy = fy - .5f, uz = fz - .5f;
    const float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
    const float2 axy = f2(ux - flx, uy - fly);
    const float az = uz - flz;
#endif
    // column of tap x + 1 and row of tap (y + 1, z) -- b.tx, |b.ty| are the
    // brick's texel origin + 1 (a resident brick's b.ty is negative in
    // texture 1; a paged entry names its texture in b.which): whole numbers
    // below 2^24, so the sums are exact and the gather's footprint is (x, y)
    // .. (x + 1, y + 1) of slice z (and, P rows further down, of slice z + 1)
    const float X = b.tx + flx;
    const float Y = fabsf(b.ty) + (flz * fd + fly);
    float4 g0, g1;
    if constexpr (GATHER == kGatherPaged)
        gather2_indexed(V, b.which, X, Y, fd, g0, g1);
    else
        gather2(V, b.which, X, Y, fd, g0, g1);
    // gather order: w = (x, y), z = (x + 1, y), x = (x, y + 1), y = (x + 1, y + 1)
#if HY_F32X2 && HY_GATHER_ROWS
    // The x lerps row by row, each row's two taps as the gather returns them
    // (adjacent registers): (x, y+1), (x+1, y+1) times (1-ax, ax) and
    // (x+1, y), (x, y) times (ax, 1-ax), then one scalar add per row (IEEE
    // addition commutes, so each row is fl(fl(c_x (1-ax)) + fl(c_x1 ax)) as
    // in trilerp); then y per slice and z as there.
    const float bx = 1.f - axy.x;
    const float2 w10 = f2(bx, axy.x), w01 = f2(axy.x, bx);
    const float2 r1z0 = mul2(f2(g0.x, g0.y), w10), r0z0 = mul2(f2(g0.z, g0.w), w01);
    const float2 r1z1 = mul2(f2(g1.x, g1.y), w10), r0z1 = mul2(f2(g1.z, g1.w), w01);
    const float2 X0 = f2(__fadd_rn(r0z0.x, r0z0.y), __fadd_rn(r0z1.x, r0z1.y));  // row y
    const float2 X1 = f2(__fadd_rn(r1z0.x, r1z0.y), __fadd_rn(r1z1.x, r1z1.y));  // row y + 1
    const float by = 1.f - axy.y, bz = 1.f - az;
    const float2 Yv = lerp2(X0, f2(by, by), X1, f2(axy.y, axy.y));
    const float2 Z = mul2(Yv, f2(bz, az));
    return __fadd_rn(Z.x, Z.y);
#else
    return trilerp(f2(g0.w, g1.w), f2(g0.z, g1.z), f2(g0.x, g1.x), f2(g0.y, g1.y), axy, az);
#endif
}

// The transfer function's knots in shared memory with the end knots
// repeated and two zero knots after them: tfs[0] = knot 0, tfs[i + 1] =
// knot i, tfs[n + 1] = knot n - 1, tfs[n + 2] = tfs[n + 3] = 0
// (n + kTfPad entries).
// Nothing is staged without knots (the Isosurface and Blocks shaders run
// without a transfer function and never call sample_tf).
constexpr int kTfPad = 4;
__device__ __forceinline__ void stage_tf(const float4 *__restrict__ tf, int n, float4 *tfs) {
    if (n <= 0) return;
    for (int i = threadIdx.x; i < n + kTfPad; i += blockDim.x)
        tfs[i] = i <= n + 1 ? tf[min(max(i - 1, 0), n - 1)] : make_float4(0.f, 0.f, 0.f, 0.f);
}

// TransferFn lookup: 1-D, normalised, Border, Linear (transfer_fn.hpp:16-23,
// cpu_sampler.hpp:117-124, 137-140), knots staged by stage_tf.
// NONNEG: s is +0, positive or NaN (a trilinear sample of u8 voxels: values
// u/255 >= 0 and weights a, 1-a >= 0 give products and sums >= +0), so the
// Border test 0 <= fx <= n reduces to !(fx <= n), which NaN fails as well.
template <bool NONNEG = false>
__device__ __forceinline__ float4 sample_tf(const float4 *__restrict__ tfs, int n, float fn,
                                            float s) {
    float fx = fn * s;
    if (NONNEG) {
        // The Border test as two selects rather than a branch: out of range
        // (fx > n, or NaN) reads the two zero knots past the end at fx = 0,
        // and their lerp is +0 in every channel, the value returned below.
        const bool in = fx <= fn;
        fx = in ? fx : 0.f;
        float u = fx - .5f;
        float flr = floorf(u);
        float a = u - flr;
        const float4 *k = tfs + (in ? int(flr) + 1 : n + 2);
        float4 x = k[0], y = k[1];
        float b = 1.f - a;
        const float2 bb = f2(b, b), aa = f2(a, a);
        const float2 rg = lerp2(f2(x.x, x.y), bb, f2(y.x, y.y), aa);
        const float2 ba = lerp2(f2(x.z, x.w), bb, f2(y.z, y.w), aa);
        return make_float4(rg.x, rg.y, ba.x, ba.y);
    }
    if (!(0.f <= fx && fx <= fn)) return make_float4(0.f, 0.f, 0.f, 0.f);
    // fx in [0, n] so fi = floor(fx - 0.5) is in [-1, n-1] and the clamped
    // neighbours knot[max(fi, 0)], knot[min(fi + 1, n - 1)] are tfs[fi + 1],
    // tfs[fi + 2].  The upper one is ceil(u) = floor(u) + 1, or floor(u) when
    // u is integral -- where a == 0 and the knot it picks is weighted by 0,
    // so floor(u) + 1 gives the same floats.
    float u = fx - .5f;
    float flr = floorf(u);
    float a = u - flr;
    const float4 *k = tfs + (int(flr) + 1);
    float4 x = k[0], y = k[1];
    float b = 1.f - a;
#if HY_F32X2
    const float2 bb = f2(b, b), aa = f2(a, a);
    const float2 rg = lerp2(f2(x.x, x.y), bb, f2(y.x, y.y), aa);
    const float2 ba = lerp2(f2(x.z, x.w), bb, f2(y.z, y.w), aa);
    return make_float4(rg.x, rg.y, ba.x, ba.y);
#else
    return make_float4(x.x * b + y.x * a, x.y * b + y.y * a, x.z * b + y.z * a, x.w * b + y.w * a);
#endif
}

struct Shared {
    const float4 *tf;
    int ntf;
    float fntf;
    const float *lut;
};
__device__ __forceinline__ Shared make_shared(const float4 *tf, int ntf, const float *lut) {
    return Shared{tf, ntf, float(ntf), lut};
}

// v.w > 0.93 and v.w > 0.85 are double comparisons in the reference
// (volume_shader.cu:71-75).  Both constants round up to float, so for a
// float x: x > 0.93 (double)  <=>  x >= 0.93f, and likewise for 0.85.
#define HY_T93 0.93f
#define HY_T85 0.85f

// Tracks the brick of the current sample position.  floor(o) only changes
// when o leaves [ip, ip+1) on some axis, so the texel lookups are redone only
// then (same texel, same values).  The test reads the brick-local
// coordinate l = o - ip the sampler needs anyway: l in [+0, 1) as an unsigned
// compare of its bits.  fl(o - ip) >= +0 and < 1 imply ip <= o < ip + 1
// (rounding is monotone and a non-zero difference of floats never rounds to
// 0); the converse can fail only where o - ip rounds up to 1, which merely
// redoes the lookups of the same cell.  NaN and the initial ip = +inf fail
// the test, so those steps redo them every time, like the reference.
__device__ __forceinline__ bool unit_interval(float l) { return __float_as_uint(l) < 0x3f800000u; }

struct BrickCursor {
    float ipx, ipy, ipz;
    int cur, cd, pg;
    bool sample;  // cd == 0 && pg != -1: the cell is sampled (one test per step)
    BrickRef br;
    __device__ __forceinline__ void reset() {
        ipx = ipy = ipz = __int_as_float(0x7f800000);
        cur = -1;
        cd = 0;
        pg = -1;
        sample = false;
        br = BrickRef{};
    }
    // o's cell changed (or may have): redo floor(o) and the thumbnail lookups
    template <int GATHER = 0>
    __device__ __forceinline__ void locate(const DevVolume &V, float ox, float oy, float oz) {
        ipx = floorf(ox);
        ipy = floorf(oy);
        ipz = floorf(oz);
        const int bid = thumb_index(V, ipx, ipy, ipz);
        // with GATHER a cell change is a brick change (the cell is the
        // brick): the entry is loaded without comparing indices
        if (GATHER || bid != cur) {
            cur = bid;
            if constexpr (GATHER == kGatherPaged) {
                const int2 in = __ldg(&V.info[bid]);
                cd = in.x;
                pg = in.y;
                sample = cd == 0 && pg != -1;
                if (sample) br = load_brick_paged(V, pg);
            } else if constexpr (GATHER) {
                // page table and texel origin in one load (no dependent
                // second load of the brick's gather-table entry)
                const int4 in = __ldg(&V.info4[bid]);
                cd = in.x;
                pg = in.y;
                sample = cd == 0 && pg != -1;
                br.tx = __int_as_float(in.z);
                br.ty = __int_as_float(in.w);  // negative: texture 1
                br.which = in.w < 0;
            } else {
                const int2 in = __ldg(&V.info[bid]);
                cd = in.x;
                pg = in.y;
                sample = cd == 0 && pg != -1;
                if (cd == 0 && pg >= 0) br = load_brick(V, pg);
            }
        }
    }
    // brick-local coordinates of o, relocating first when o left the cell
    template <int GATHER = 0>
    __device__ __forceinline__ void update(const DevVolume &V, float ox, float oy, float oz,
                                           float &lx, float &ly, float &lz) {
#if HY_F32X2
        const float2 lxy = sub2(f2(ox, oy), f2(ipx, ipy));
        lx = lxy.x;
        ly = lxy.y;
#else
        lx = ox - ipx;
        ly = oy - ipy;
#endif
        lz = oz - ipz;
        if (unit_interval(lx) & unit_interval(ly) & unit_interval(lz)) return;
        locate<GATHER>(V, ox, oy, oz);
        lx = ox - ipx;
        ly = oy - ipy;
        lz = oz - ipz;
    }
};

// VolumeShaderKernel::main (volume_shader.cu:32-81) as the per-ray state and
// one loop iteration; volume_main is the loop.  PADDED: the volume has an
// apron of >= 1 voxel, so the interior sampler applies.
// The reciprocals the empty-brick skip needs (1/d and 1/compMax(|d|)) are
// computed where a skip happens rather than held for the whole ray: the
// same floats, four registers fewer in the march.
struct VolumeMarch {
    BrickCursor c;
    float sx, sy, sz;  // (d * step) * step_size, redone only when step_size changes

    __device__ __forceinline__ void set_step(const Px &p, float step) {
        const float fs = float(p.step_size);
        sx = (p.dx * step) * fs;
        sy = (p.dy * step) * fs;
        sz = (p.dz * step) * fs;
    }

    // p.step_size is 1 for a new ray, or what a film pass left
    __device__ __forceinline__ void init(const Px &p, float step) {
        c.reset();
        set_step(p, step);
    }

    // The sample at brick-local (lx, ly, lz) of the current cell, its
    // transfer-function lookup, compositing and the adaptive step size.
    template <int PC, int DT, bool PADDED, bool LEAN = false, int GATHER = 0>
    __device__ __forceinline__ void shade(Px &p, const ShadeArgs &A, const Shared &S, float lx,
                                          float ly, float lz, unsigned int &samples) {
        const DevVolume &V = A.vol;
        {
            float s;
            if constexpr (GATHER)
                s = sample_brick_gather<PC, GATHER>(V, c.br, V.P, lx, ly, lz);
            else
                s = sample_brick<PC, DT, PADDED>(c.br, V.P, lx, ly, lz, S.lut);
            ++samples;
            float4 ub = sample_tf<DT == HY_DTYPE_U8>(S.tf, S.ntf, S.fntf, s);
            if (LEAN) {
            } else if (A.mode == HY_VOLUME_PARTITION) {
                float r = A.rank;
                float mr = 1.f * (1.f - r) + 0.f * r, mg = 0.f * (1.f - r) + 0.f * r,
                      mb = 0.f * (1.f - r) + 1.f * r;
                float len = sqrtf(ub.x * ub.x + ub.y * ub.y + ub.z * ub.z);
                ub = make_float4(mr * len, mg * len, mb * len, ub.w);
            } else if (A.mode == HY_VOLUME_PAGING) {
                ub = c.pg >= A.lowest_blkcnt ? make_float4(0.f, 1.f, 0.f, ub.w)
                                             : make_float4(1.f, 0.f, 0.f, ub.w);
            }
            ub.w = ub.w * A.density;  // opacity scale; exact identity at 1
            const float w = ub.w;
#if HY_F32X2
            const float2 uxy = mul2(f2(ub.x, ub.y), f2(w, w));
            ub.x = uxy.x;
            ub.y = uxy.y;
#else
            ub.x = ub.x * w;
            ub.y = ub.y * w;
#endif
            ub.z = ub.z * w;
            if (!LEAN) {
                p.e0 = p.e0 + ub.x * p.e3;
                p.e1 = p.e1 + ub.y * p.e3;
                p.e2 = p.e2 + ub.z * p.e3;
                p.e3 = p.e3 * (1.f - ub.w);
            }
            const float t = 1.f - p.vw;
#if HY_F32X2
            const float2 txy = mul2(f2(ub.x, ub.y), f2(t, t));
            const float2 tzw = mul2(f2(ub.z, ub.w), f2(t, t));
            p.vx = __fadd_rn(p.vx, txy.x);
            p.vy = __fadd_rn(p.vy, txy.y);
            p.vz = __fadd_rn(p.vz, tzw.x);
            p.vw = __fadd_rn(p.vw, tzw.y);
#else
            p.vx = p.vx + ub.x * t;
            p.vy = p.vy + ub.y * t;
            p.vz = p.vz + ub.z * t;
            p.vw = p.vw + ub.w * t;
#endif
            // v.w > 0.93 -> 16, else v.w > 0.85 -> 4 (volume_shader.cu:71-75),
            // nested so that the common case (v.w below both) tests once
            if (p.vw >= HY_T85) {
                const int ss = p.vw >= HY_T93 ? 16 : 4;
                if (p.step_size != ss) {
                    p.step_size = ss;
                    set_step(p, A.step);
                }
            }
        }
    }

    __device__ __forceinline__ void advance(Px &p) {
        p.ox = p.ox + sx;  // sx..sz are products: scalar adds
        p.oy = p.oy + sy;
        p.oz = p.oz + sz;
        p.nsteps -= p.step_size;
    }

    // One iteration of `while (nsteps > 0)`; false when the ray breaks out
    // on an absent brick (volume_shader.cu:50).  LEAN: Default mode and
    // nobody reads theta / phi (no film, aux output or per-brick
    // compositing), so their updates are left out; v is unchanged.
    // GATHER: u8 bricks with an apron sampled through their gather textures.
    template <int PC, int DT, bool PADDED, bool LEAN = false, int GATHER = 0>
    __device__ __forceinline__ bool step(Px &p, const ShadeArgs &A, const Shared &S,
                                         unsigned int &samples) {
        const DevVolume &V = A.vol;
        float lx, ly, lz;
        c.update<GATHER>(V, p.ox, p.oy, p.oz, lx, ly, lz);
        if (!c.sample) {
            if (c.cd == 0) return false;  // absent brick (pg == -1)
            const float cdu = 1.f / gmax(gmax(fabsf(p.dx), fabsf(p.dy)), fabsf(p.dz));
            p.nsteps -= skip_nblock_steps(p, 1.f / p.dx, 1.f / p.dy, 1.f / p.dz, c.ipx, c.ipy,
                                          c.ipz, c.cd, cdu, A.step * float(p.step_size));
        } else {
            shade<PC, DT, PADDED, LEAN, GATHER>(p, A, S, lx, ly, lz, samples);
        }
        advance(p);
        return true;
    }
};

// LOOP: the shape of the march loop.
//  kLoopOne  one step per iteration;
//  kLoopErt  early ray termination by warp vote (hy_shader_params.
//            early_termination): after each step the lanes still marching
//            vote; when v.w >= A.ert on all of them they stop together (a lane
//            alone stopping would not free its warp).  A lane stops only when
//            its own ray is that opaque, whichever lanes vote with it, so what
//            it leaves out adds at most 1 - A.ert per channel;
//  kLoopTwo  two steps per iteration (the batch's steps_per_iter = 2): the
//            same steps in the same order, one loop test per step still.
constexpr int kLoopOne = 0, kLoopErt = 1, kLoopTwo = 2;
template <int PC, int DT, bool PADDED, bool LEAN = false, int GATHER = 0, int LOOP = kLoopOne>
__device__ __forceinline__ long long volume_main(Px &p, const ShadeArgs &A, const Shared &S) {
    unsigned int samples = 0;
    VolumeMarch m;
    m.init(p, A.step);
    while (p.nsteps > 0) {
        if (!m.step<PC, DT, PADDED, LEAN, GATHER>(p, A, S, samples)) break;
        if (LOOP == kLoopErt && __all_sync(__activemask(), p.vw >= A.ert)) break;
        if (LOOP == kLoopTwo) {
            if (p.nsteps <= 0) break;
            if (!m.step<PC, DT, PADDED, LEAN, GATHER>(p, A, S, samples)) break;
        }
    }
    return samples;
}

// VisBlocksShaderKernel::main (blocks_shader.cu:16-50).
__device__ __forceinline__ long long blocks_main(Px &p, const ShadeArgs &A) {
    const DevVolume &V = A.vol;
    long long samples = 0;
    const float cdu = 1.f / gmax(gmax(fabsf(p.dx), fabsf(p.dy)), fabsf(p.dz));
    const float rx = 1.f / p.dx, ry = 1.f / p.dy, rz = 1.f / p.dz;
    const float opacity_threshold = 0.95f;
    const float hx = A.bbox_max[0] - 1.f, hy = A.bbox_max[1] - 1.f, hz = A.bbox_max[2] - 1.f;
    const float ex = A.bbox_max[0] - 0.f, ey = A.bbox_max[1] - 0.f, ez = A.bbox_max[2] - 0.f;
    const float sx = p.dx * A.step, sy = p.dy * A.step, sz = p.dz * A.step;
    while (p.nsteps > 0) {
        float ipx = floorf(p.ox), ipy = floorf(p.oy), ipz = floorf(p.oz);
        int bid = thumb_index(V, ipx, ipy, ipz);
        int cd = __ldg(&V.info[bid].x);
        if (cd) {
            p.nsteps -= skip_nblock_steps(p, rx, ry, rz, ipx, ipy, ipz, cd, cdu, A.step);
        } else {
            float rpx = fclamp(ipx, 0.f, hx) / ex, rpy = fclamp(ipy, 0.f, hy) / ey,
                  rpz = fclamp(ipz, 0.f, hz) / ez;
            ++samples;
            if (A.mode == HY_BLOCKS_VOLUME) {
                const float mean = __ldg(&V.mean[bid]);
                const float cx = rpx * A.density * mean, cy = rpy * A.density * mean,
                            cz = rpz * A.density * mean, cw = 1.f * A.density * mean;
                const float t = 1.f - p.vw;
                p.vx = p.vx + cx * t;
                p.vy = p.vy + cy * t;
                p.vz = p.vz + cz * t;
                p.vw = p.vw + cw * t;
                if (p.vw > opacity_threshold) {
                    p.nsteps = 0;
                    break;
                }
            } else {
                p.vx = rpx;
                p.vy = rpy;
                p.vz = rpz;
                p.vw = 1.f;
                p.nsteps = 0;
                break;
            }
        }
        p.ox = p.ox + sx;
        p.oy = p.oy + sy;
        p.oz = p.oz + sz;
        p.nsteps -= 1;
    }
    return samples;
}

// PagingShaderKernel::main (paging_shader.cu:26-61): the paging debug view.
// Each non-empty brick a ray enters adds one constant colour -- green 0.5 for
// a resident fine brick (registry id >= lowest_blkcnt), red 0.2 for a coarse
// stand-in -- and the ray skips to that brick's exit; opacity > 0.95 or an
// absent brick (page fault) ends the ray (nsteps is left as it is there).
__device__ __forceinline__ long long paging_main(Px &p, const ShadeArgs &A) {
    const DevVolume &V = A.vol;
    long long samples = 0;
    const float cdu = 1.f / gmax(gmax(fabsf(p.dx), fabsf(p.dy)), fabsf(p.dz));
    const float rx = 1.f / p.dx, ry = 1.f / p.dy, rz = 1.f / p.dz;
    const float opacity_threshold = 0.95f;
    const float sx = p.dx * A.step, sy = p.dy * A.step, sz = p.dz * A.step;
    while (p.nsteps > 0) {
        float ipx = floorf(p.ox), ipy = floorf(p.oy), ipz = floorf(p.oz);
        int bid = thumb_index(V, ipx, ipy, ipz);
        const int2 in = __ldg(&V.info[bid]);
        if (in.x) {
            p.nsteps -= skip_nblock_steps(p, rx, ry, rz, ipx, ipy, ipz, in.x, cdu, A.step);
        } else {
            if (in.y == -1) break;  // page fault
            const bool fine = in.y >= A.lowest_blkcnt;
            const float cx = fine ? 0.f * .5f : 1.f * .2f, cy = fine ? 1.f * .5f : 0.f * .2f,
                        cz = fine ? 0.f * .5f : 0.f * .2f, cw = fine ? 1.f * .5f : 1.f * .2f;
            p.nsteps -= skip_nblock_steps(p, rx, ry, rz, ipx, ipy, ipz, 1, cdu, A.step);
            ++samples;
            const float t = 1.f - p.vw;
            p.vx = p.vx + cx * t;
            p.vy = p.vy + cy * t;
            p.vz = p.vz + cz * t;
            p.vw = p.vw + cw * t;
            if (p.vw > opacity_threshold) break;
        }
        p.ox = p.ox + sx;
        p.oy = p.oy + sy;
        p.oz = p.oz + sz;
        p.nsteps -= 1;
    }
    return samples;
}

// linear_to_srgb of the isosurface shader: double-precision constants
// (isosurface_shader.cu:25-32).
__device__ __forceinline__ float iso_linear_to_srgb(float linear) {
    double l = double(linear);
    if (l <= 0.0031308) return float(12.92 * l);
    return float((1.0 + 0.055) * pow(l, 1.0 / 2.4) - 0.055);
}

__device__ __forceinline__ void mat_vec4(const float *m, float x, float y, float z, float w,
                                         float &ox, float &oy, float &oz) {
    ox = m[0] * x + m[4] * y + m[8] * z + m[12] * w;
    oy = m[1] * x + m[5] * y + m[9] * z + m[13] * w;
    oz = m[2] * x + m[6] * y + m[10] * z + m[14] * w;
}

__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
    const float r = 1.f / sqrtf(x * x + y * y + z * z);
    x = x * r;
    y = y * r;
    z = z * r;
}

// IsosurfaceShaderKernel::main (isosurface_shader.cu:50-125).  prev_value
// stays 0, as in the reference (it is never updated there).
template <int PC, int DT, bool PADDED>
__device__ __forceinline__ long long iso_main(Px &p, const ShadeArgs &A, const ViewArgs &Vw,
                                             const Shared &S) {
    const DevVolume &V = A.vol;
    long long samples = 0;
    const float cdu = 1.f / gmax(gmax(fabsf(p.dx), fabsf(p.dy)), fabsf(p.dz));
    const float rx = 1.f / p.dx, ry = 1.f / p.dy, rz = 1.f / p.dz;
    const float prev_value = 0.0f;
    const float iso = A.isovalue;
    // sign(value - iso) != sign(prev_value - iso), prev_value = 0 (never
    // updated, isosurface_shader.cu:58-70).  The rounded difference of two
    // floats has the sign of the exact one (and is 0 only when they are
    // equal), so per sign of -iso the test is one comparison; NaN values
    // (sign 0) and a NaN isovalue behave as with fsign.
    const float prev_sign = fsign(prev_value - iso);
    const float sx = p.dx * A.step, sy = p.dy * A.step, sz = p.dz * A.step;
    BrickCursor c;
    c.reset();
    while (p.nsteps > 0) {
        float l0x, l0y, l0z;
        c.update(V, p.ox, p.oy, p.oz, l0x, l0y, l0z);
        const float ipx = c.ipx, ipy = c.ipy, ipz = c.ipz;
        const BrickRef &br = c.br;
        if (c.cd) {
            p.nsteps -= skip_nblock_steps(p, rx, ry, rz, ipx, ipy, ipz, c.cd, cdu, A.step);
        } else {
            if (c.pg == -1) break;  // page fault: resume in the next march pass
            float value = sample_brick<PC, DT, PADDED>(br, V.P, l0x, l0y, l0z, S.lut);
            ++samples;
            const bool crossed = prev_sign < 0.f   ? !(value < iso)
                                 : prev_sign > 0.f ? !(value > iso)
                                                   : (value < iso || value > iso);
            if (crossed) {
                const float dt = A.step;
                p.vx = A.surface[0];
                p.vy = A.surface[1];
                p.vz = A.surface[2];
                p.vw = 1.f;
                const float a = (iso - prev_value) / (value - prev_value);
                const float qx = p.ox - dt * p.dx, qy = p.oy - dt * p.dy, qz = p.oz - dt * p.dz;
                const float ia = 1.f - a;
                const float ipx2 = ia * qx + a * p.ox, ipy2 = ia * qy + a * p.oy,
                            ipz2 = ia * qz + a * p.oz;
                // central difference in brick-local coordinates, dt = du * 2
                const float lx = ipx2 - ipx, ly = ipy2 - ipy, lz = ipz2 - ipz;
                const float g = A.du * 2.f;
                float nnx = sample_brick<0, DT>(br, V.P, lx - g, ly - 0.f, lz - 0.f, S.lut) -
                            sample_brick<0, DT>(br, V.P, lx + g, ly + 0.f, lz + 0.f, S.lut);
                float nny = sample_brick<0, DT>(br, V.P, lx - 0.f, ly - g, lz - 0.f, S.lut) -
                            sample_brick<0, DT>(br, V.P, lx + 0.f, ly + g, lz + 0.f, S.lut);
                float nnz = sample_brick<0, DT>(br, V.P, lx - 0.f, ly - 0.f, lz - g, S.lut) -
                            sample_brick<0, DT>(br, V.P, lx + 0.f, ly + 0.f, lz + g, S.lut);
                samples += 6;
                float wx, wy, wz, nx, ny, nz;
                mat_vec4(A.to_world, ipx2, ipy2, ipz2, 1.f, wx, wy, wz);
                mat_vec4(A.to_world, nnx, nny, nnz, 0.f, nx, ny, nz);
                normalize3(nx, ny, nz);
                float lx2 = Vw.light[0] - wx, ly2 = Vw.light[1] - wy, lz2 = Vw.light[2] - wz;
                normalize3(lx2, ly2, lz2);
                float hx = lx2 - wx, hy = ly2 - wy, hz = lz2 - wz;
                normalize3(hx, hy, hz);
                const float ambient = 0.2f;
                const float diffuse = .6f * fclamp(lx2 * nx + ly2 * ny + lz2 * nz, 0.f, 1.f);
                const float specular =
                    .2f * powf(fclamp(hx * nx + hy * ny + hz * nz, 0.f, 1.f), 100.f);
                const float ex = wx - Vw.eye[0], ey = wy - Vw.eye[1], ez = wz - Vw.eye[2];
                const float distance = sqrtf(ex * ex + ey * ey + ez * ez) / 2.f;
                if (A.mode == HY_ISO_COLOR) {
                    const float f = ambient + (diffuse + specular) / distance;
                    p.vx = iso_linear_to_srgb(p.vx * f);
                    p.vy = iso_linear_to_srgb(p.vy * f);
                    p.vz = iso_linear_to_srgb(p.vz * f);
                    p.vw = p.vw * f;
                } else if (A.mode == HY_ISO_POSITION) {
                    p.vx = ipx2 / A.bbox_max[0];
                    p.vy = ipy2 / A.bbox_max[1];
                    p.vz = ipz2 / A.bbox_max[2];
                    p.vw = 1.f;
                } else {
                    p.vx = nx;
                    p.vy = ny;
                    p.vz = nz;
                    p.vw = 1.f;
                }
                const float ddx = p.e0 - p.ox, ddy = p.e1 - p.oy, ddz = p.e2 - p.oz;
                p.e3 = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
                p.nsteps = 0;
                break;
            }
        }
        p.ox = p.ox + sx;
        p.oy = p.oy + sy;
        p.oz = p.oz + sz;
        p.nsteps -= 1;
    }
    return samples;
}

template <int SHADER, int PC, int DT, bool PADDED, bool LEAN = false, int GATHER = 0,
          int LOOP = kLoopOne>
__device__ __forceinline__ long long run_main(Px &p, const ShadeArgs &A, const ViewArgs &Vw,
                                             const Shared &S) {
    if (SHADER == HY_SHADER_VOLUME)
        return volume_main<PC, DT, PADDED, LEAN, GATHER, LOOP>(p, A, S);
    if (SHADER == HY_SHADER_BLOCKS) return blocks_main(p, A);
    if (SHADER == HY_SHADER_PAGING) return paging_main(p, A);
    return iso_main<PC, DT, PADDED>(p, A, Vw, S);
}

// Ray generation (cuda_shading.cu:24-29 == cpu_shading.cc:14-21).
__device__ __forceinline__ void gen_ray(const ViewArgs &Vw, int x, int y, float &ox, float &oy,
                                        float &oz, float &dx, float &dy, float &dz) {
    const float ccx = float(Vw.W) / 2.f, ccy = float(Vw.H) / 2.f;
    const float fh = float(Vw.H);
    const float ux = (float(x) - ccx) * 2.f / fh;
    const float uy = (float(y) - ccy) * 2.f / fh;
    float px, py, pz;
    mat_vec4(Vw.trans, ux, -uy, -Vw.ctg, 1.f, px, py, pz);
    ox = Vw.ray_o[0];
    oy = Vw.ray_o[1];
    oz = Vw.ray_o[2];
    dx = px - ox;
    dy = py - oy;
    dz = pz - oz;
    normalize3(dx, dy, dz);
}

// ray_emit_shader_impl (shader.hpp:113-137) against box [b0, b1] up to the
// call of main: init() of the Volume (volume_shader.cu:16-21) and Isosurface
// (isosurface_shader.cu:34-39) shaders, slab test, advance to tnear, step
// count.  Returns false for a miss (nsteps = 0).
template <int SHADER>
__device__ __forceinline__ bool emit_setup(Px &p, const ShadeArgs &A, float ox, float oy,
                                           float oz, float dx, float dy, float dz, float x0,
                                           float y0, float z0, float x1, float y1, float z1) {
    p.ox = ox;
    p.oy = oy;
    p.oz = oz;
    p.dx = dx;
    p.dy = dy;
    p.dz = dz;
    p.vx = p.vy = p.vz = p.vw = 0.f;
    if (SHADER == HY_SHADER_VOLUME) {
        p.e0 = p.e1 = p.e2 = 0.f;
        p.e3 = 1.f;
    } else if (SHADER == HY_SHADER_ISOSURFACE) {
        p.e0 = ox;
        p.e1 = oy;
        p.e2 = oz;
        p.e3 = __int_as_float(0x7f800000);  // INFINITY
    } else {
        p.e0 = p.e1 = p.e2 = p.e3 = 0.f;
    }
    p.step_size = 1;
    float tnear, tfar;
    if (intersect(ox, oy, oz, 1.f / dx, 1.f / dy, 1.f / dz, x0, y0, z0, x1, y1, z1, tnear, tfar)) {
        if (tnear < 0) tnear = 0;
        if (tfar < 0) tfar = 0;
        p.ox = p.ox + p.dx * tnear;
        p.oy = p.oy + p.dy * tnear;
        p.oz = p.oz + p.dz * tnear;
        p.nsteps = min(A.max_steps, int((tfar - tnear) / A.step));
        return true;
    }
    p.nsteps = 0;
    return false;
}

// ray_emit_shader_impl: emit_setup, then main on a hit (shader.hpp:113-137).
template <int SHADER, int PC, int DT, bool PADDED, bool LEAN = false, int GATHER = 0,
          int LOOP = kLoopOne>
__device__ __forceinline__ long long emit(Px &p, const ShadeArgs &A, const ViewArgs &Vw,
                                          const Shared &S, float ox,
                                          float oy, float oz, float dx, float dy, float dz,
                                          float x0, float y0, float z0, float x1, float y1,
                                          float z1) {
    if (emit_setup<SHADER>(p, A, ox, oy, oz, dx, dy, dz, x0, y0, z0, x1, y1, z1))
        return run_main<SHADER, PC, DT, PADDED, LEAN, GATHER, LOOP>(p, A, Vw, S);
    return 0;
}

__device__ __forceinline__ unsigned char saturate_u8(float f) {
    return (unsigned char)fclamp(f * 255.f, 0.f, 255.f);  // glm_math.hpp:75-81 (truncating)
}

__device__ __forceinline__ float vol_linear_to_srgb(float x) {  // volume.cc:175-181
    if (x <= 0.0031308f) return 12.92f * x;
    return 1.055f * powf(x, 1.f / 2.4f) - 0.055f;
}

// Per-brick sort-last for one ray: 3-D DDA over the brick grid inside the
// volume box; each non-empty brick is an emit against its own box (the
// per-partition bbox of dbuf_renderer.hpp:38-40) and the partials are
// composited front to back with volume.cc:267-280 (Volume),
// isosurface.cc:272-290 (depth-min, Isosurface) or the over operator (Blocks).
template <int SHADER, int PC, int DT, bool PADDED, int GATHER = 0>
__device__ __forceinline__ long long composite_ray(const ShadeArgs &A, const ViewArgs &Vw,
                                                   const Shared &S, float ox,
                                                   float oy, float oz, float dx, float dy,
                                                   float dz, float4 &acc, float4 &aux) {
    long long samples = 0;
    acc = make_float4(0.f, 0.f, 0.f, 0.f);
    aux = make_float4(0.f, 0.f, 0.f, 1.f);
    float acc_depth = __int_as_float(0x7f800000);
    if (SHADER == HY_SHADER_ISOSURFACE) aux.w = 0.f;
    float tnear, tfar;
    if (SHADER == HY_SHADER_BLOCKS) aux.w = 0.f;
    if (!intersect(ox, oy, oz, 1.f / dx, 1.f / dy, 1.f / dz, 0.f, 0.f, 0.f, A.bbox_max[0],
                   A.bbox_max[1], A.bbox_max[2], tnear, tfar)) {
        if (SHADER == HY_SHADER_ISOSURFACE) aux.x = acc_depth;
        return 0;
    }
    const float t0 = tnear < 0.f ? 0.f : tnear;
    const float t1 = tfar;
    if (!(t1 > t0)) {
        if (SHADER == HY_SHADER_ISOSURFACE) aux.x = acc_depth;
        return 0;
    }
    const DevVolume &V = A.vol;
    const int g[3] = {V.gx, V.gy, V.gz};
    const float o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz};
    int cell[3];
    int stp[3];
    float tmax[3], tdelta[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float pa = o[a] + d[a] * t0;
        cell[a] = iclamp(int(floorf(pa)), 0, g[a] - 1);
        stp[a] = d[a] > 0.f ? 1 : (d[a] < 0.f ? -1 : 0);
        if (stp[a] != 0) {
            const float nb = float(stp[a] > 0 ? cell[a] + 1 : cell[a]);
            tmax[a] = (nb - o[a]) / d[a];
            tdelta[a] = 1.f / fabsf(d[a]);
        } else {
            tmax[a] = __int_as_float(0x7f800000);
            tdelta[a] = __int_as_float(0x7f800000);
        }
    }
    bool first = true;
    const int limit = g[0] + g[1] + g[2] + 3;
    for (int it = 0; it < limit; ++it) {
        const int bid = (cell[2] * g[1] + cell[1]) * g[0] + cell[0];
        if (__ldg(&V.info[bid].x) == 0) {
            const float bx = float(cell[0]), by = float(cell[1]), bz = float(cell[2]);
            Px p;
            samples += emit<SHADER, PC, DT, PADDED, false, GATHER>(p, A, Vw, S, ox, oy, oz, dx, dy, dz,
                                                                   bx, by, bz, bx + 1.f, by + 1.f,
                                                                   bz + 1.f);
            if (SHADER == HY_SHADER_VOLUME) {
                if (first) {
                    acc = make_float4(p.vx, p.vy, p.vz, p.vw);
                    aux = make_float4(p.e0, p.e1, p.e2, p.e3);
                } else {
                    const float nx = acc.x + p.vx - acc.w * p.e0;
                    const float ny = acc.y + p.vy - acc.w * p.e1;
                    const float nz = acc.z + p.vz - acc.w * p.e2;
                    const float na = p.e3 * acc.w + p.vw;
                    acc = make_float4(nx, ny, nz, na);
                }
            } else if (SHADER == HY_SHADER_ISOSURFACE) {
                if (first || p.e3 < acc_depth) {
                    acc = make_float4(p.vx, p.vy, p.vz, p.vw);
                    acc_depth = p.e3;
                }
            } else {
                const float t = 1.f - acc.w;
                acc = make_float4(acc.x + p.vx * t, acc.y + p.vy * t, acc.z + p.vz * t,
                                  acc.w + p.vw * t);
            }
            first = false;
        }
        int a = 0;
        if (tmax[1] < tmax[a]) a = 1;
        if (tmax[2] < tmax[a]) a = 2;
        if (!(tmax[a] < t1)) break;
        cell[a] += stp[a];
        if (cell[a] < 0 || cell[a] >= g[a]) break;
        tmax[a] = tmax[a] + tdelta[a];
    }
    if (SHADER == HY_SHADER_VOLUME && A.srgb) {
        acc.x = vol_linear_to_srgb(acc.x);
        acc.y = vol_linear_to_srgb(acc.y);
        acc.z = vol_linear_to_srgb(acc.z);
    }
    if (SHADER == HY_SHADER_ISOSURFACE) aux = make_float4(acc_depth, 0.f, 0.f, 0.f);
    if (SHADER == HY_SHADER_BLOCKS) aux = make_float4(0.f, 0.f, 0.f, 0.f);
    return samples;
}

}  // namespace dev
}  // namespace hy
