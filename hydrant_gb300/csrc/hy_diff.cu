// hy_diff.cu -- differentiable Volume rendering: forward with per-ray
// checkpoints and the adjoint ray march.
//
// The forward is the Volume shader's march (volume_shader.cu:32-81) over one
// dense f32 brick with a 1-voxel replicate apron, in the reference's float
// operations, with the discontinuous parts fixed: step_size stays 1 (no
// adaptive stepping) and there is no empty-space skipping.  Sampling the
// padded brick at index i is sampling the raw volume at clamp(i-1, 0, n-1),
// so the kernels read the caller's raw n^3 volume directly and the gradient
// of an apron voxel lands on the voxel it replicates.
//
// Every K steps the forward stores the ray state (position, v.w) in a
// checkpoint buffer.  The adjoint walks a ray's segments back to front: it
// restores a checkpoint, recomputes the K samples of that segment (positions,
// sample values, transmittance) into per-thread arrays, and back-propagates
// through front-to-back compositing, the transfer-function lookup and the
// trilinear weights without fetching the voxels a second time.  With c_n = (r a, g a, b a, a), T_n = 1 - v.w before sample n and
// R_n = c_n + (1 - a_n) R_{n+1} the colour composited behind sample n:
//   dL/dc_n = T_n g,   dL/da_n += -T_n (g . R_{n+1}),
// with g = dL/dv of the pixel.  A ray sums its knot and voxel gradients in
// registers while consecutive samples stay in one knot interval / voxel cell;
// knot sums then go through shared memory (one global atomic per knot channel
// and block), voxel sums straight to global atomics (eight per cell).

#include <algorithm>
#include <cstring>

#include "hy_shade.cuh"

using namespace hy;
using namespace hy::dev;

namespace {

constexpr int kMaxDiffViews = 64;
constexpr int kMaxK = 64;
constexpr int kMaxKnots = 256;

struct DiffView {
    float trans[16];
    float ctg;
    float ray_o[3];
};

struct DiffArgs {
    const float *vol;  // raw n^3, x fastest
    int n;             // edge (brick = whole volume)
    float k, b;        // BlockSamplerMapping of the padded brick
    float step;
    int max_steps;
    float density;
    const float4 *tf;
    int ntf;
    int K;             // checkpoint interval
    int max_ckpt;      // checkpoints per ray
    int W, H, nviews;
    DiffView views[kMaxDiffViews];
    float4 *image;     // nviews * H * W
    float4 *ckpt;      // nviews * H * W * max_ckpt (position.xyz, v.w)
    int *nsteps_out;   // steps taken per ray (for the adjoint)
    const float4 *dimage;
    float *dvol;
    float *dtf;        // ntf * 4
    // the padded volume as a gather texture (0: none): slice s of P = n + 2
    // in tile (s / gper, s % gper) of P x P texels, column tiles P apart,
    // with slice (c + 1) * gper repeated as row gper of column c, so slice
    // s + 1 of a footprint is always P rows below slice s
    unsigned long long gtex;
    int gper;
};

// Trilinear footprint of the padded brick at brick-local x in [0,1] (the
// interior case of sample_brick: apron >= 1, no wrap, no clamps): the raw
// volume rows and columns of the 2x2x2 taps and the lerp fractions.  Voxel
// indices fit in int (n^3 < 2^31 is checked on the host).
struct Cell {
    int r00, r10, r01, r11;  // row bases (z, y) -> (z * n + y) * n
    int x0, x1;
    float ax, ay, az;
};

__device__ __forceinline__ void diff_cell(const DiffArgs &a, float lx, float ly, float lz,
                                          Cell &c) {
    const int P = a.n + 2;
    const float fd = float(P);
    // x and y in packed pairs (products summed by scalar adds), z alone
    const float2 kl = mul2(f2(a.k, a.k), f2(lx, ly));
    const float2 fxy = mul2(f2(fd, fd), f2(__fadd_rn(kl.x, a.b), __fadd_rn(kl.y, a.b)));
    const float fz = fd * (a.k * lz + a.b);
    const float ux = fxy.x - .5f, uy = fxy.y - .5f, uz = fz - .5f;
    const float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
    const float2 axy = sub2(f2(ux, uy), f2(flx, fly));
    c.ax = axy.x;
    c.ay = axy.y;
    c.az = uz - flz;
    const int ix = int(flx), iy = int(fly), iz = int(flz);
    // padded index i -> raw clamp(i - 1, 0, n - 1)
    const int n = a.n;
    c.x0 = iclamp(ix - 1, 0, n - 1);
    c.x1 = iclamp(ix, 0, n - 1);
    const int y0 = iclamp(iy - 1, 0, n - 1), y1 = iclamp(iy, 0, n - 1);
    const int z0 = iclamp(iz - 1, 0, n - 1), z1 = iclamp(iz, 0, n - 1);
    c.r00 = (z0 * n + y0) * n;
    c.r10 = (z0 * n + y1) * n;
    c.r01 = (z1 * n + y0) * n;
    c.r11 = (z1 * n + y1) * n;
}

__device__ __forceinline__ float diff_fetch(const DiffArgs &a, const Cell &c) {
    // taps in z pairs: c<y><x> = (v_xy0, v_xy1); the lerps of sample_brick
    const float2 c00 = f2(__ldg(a.vol + c.r00 + c.x0), __ldg(a.vol + c.r01 + c.x0));
    const float2 c01 = f2(__ldg(a.vol + c.r00 + c.x1), __ldg(a.vol + c.r01 + c.x1));
    const float2 c10 = f2(__ldg(a.vol + c.r10 + c.x0), __ldg(a.vol + c.r11 + c.x0));
    const float2 c11 = f2(__ldg(a.vol + c.r10 + c.x1), __ldg(a.vol + c.r11 + c.x1));
    const float2 bxy = sub2(f2(1.f, 1.f), f2(c.ax, c.ay));
    const float bz = 1.f - c.az;
    const float2 bx2 = f2(bxy.x, bxy.x), ax2 = f2(c.ax, c.ax);
    const float2 X0 = lerp2(c00, bx2, c01, ax2);  // (x0_0, x0_1)
    const float2 X1 = lerp2(c10, bx2, c11, ax2);  // (x1_0, x1_1)
    const float2 Y = lerp2(X0, f2(bxy.y, bxy.y), X1, f2(c.ay, c.ay));
    const float2 Z = mul2(Y, f2(bz, c.az));
    return __fadd_rn(Z.x, Z.y);
}

__device__ __forceinline__ float diff_sample(const DiffArgs &a, float lx, float ly, float lz) {
    Cell c;
    diff_cell(a, lx, ly, lz, c);
    return diff_fetch(a, c);
}

// diff_sample through the gather texture: the same fractions and lerps, the
// eight taps by two gathers (slices iz and iz + 1 of the padded volume,
// whose texels repeat the clamped border exactly as diff_cell's indices do).
// In the interior a footprint's lower index lies in [0, P - 2], so the
// whole-number texel coordinates stay inside the slice's tile.
__device__ __forceinline__ float diff_sample_gather(const DiffArgs &a, float lx, float ly,
                                                    float lz) {
    const int P = a.n + 2;
    const float fd = float(P);
    const float2 kl = mul2(f2(a.k, a.k), f2(lx, ly));
    const float2 fxy = mul2(f2(fd, fd), f2(__fadd_rn(kl.x, a.b), __fadd_rn(kl.y, a.b)));
    const float fz = fd * (a.k * lz + a.b);
    const float ux = fxy.x - .5f, uy = fxy.y - .5f, uz = fz - .5f;
    const float flx = floorf(ux), fly = floorf(uy), flz = floorf(uz);
    const float2 axy = sub2(f2(ux, uy), f2(flx, fly));
    const float az = uz - flz;
    const int iz = int(flz);
    const int col = iz / a.gper, row = iz - col * a.gper;
    const float X = float(col * P + 1) + flx, Y = float(row * P + 1) + fly;
    const float4 g0 = gather_r(a.gtex, X, Y), g1 = gather_r(a.gtex, X, Y + fd);
    // gather order: w = (x, y), z = (x + 1, y), x = (x, y + 1), y = (x + 1, y + 1)
    const float2 c00 = f2(g0.w, g1.w), c01 = f2(g0.z, g1.z);
    const float2 c10 = f2(g0.x, g1.x), c11 = f2(g0.y, g1.y);
    const float2 bxy = sub2(f2(1.f, 1.f), axy);
    const float bz = 1.f - az;
    const float2 bx2 = f2(bxy.x, bxy.x), ax2 = f2(axy.x, axy.x);
    const float2 X0 = lerp2(c00, bx2, c01, ax2);
    const float2 X1 = lerp2(c10, bx2, c11, ax2);
    const float2 Yv = lerp2(X0, f2(bxy.y, bxy.y), X1, f2(axy.y, axy.y));
    const float2 Z = mul2(Yv, f2(bz, az));
    return __fadd_rn(Z.x, Z.y);
}

// The padded volume into the gather texture: one thread per texel of a
// slice row (x), rows (y) and slices (z) on the grid's other axes.
__global__ void diff_fill_kernel(const float *__restrict__ vol, int n, int gper,
                                 unsigned long long surf) {
    const int P = n + 2;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, s = blockIdx.z;
    if (x >= P) return;
    const int vx = min(max(x - 1, 0), n - 1), vy = min(max(y - 1, 0), n - 1),
              vz = min(max(s - 1, 0), n - 1);
    const float v = vol[(size_t(vz) * n + vy) * n + vx];
    const cudaSurfaceObject_t so = cudaSurfaceObject_t(surf);
    const int col = s / gper, row = s - col * gper;
    surf2Dwrite(v, so, (col * P + x) * int(sizeof(float)), row * P + y, cudaBoundaryModeZero);
    if (row == 0 && col > 0)
        surf2Dwrite(v, so, ((col - 1) * P + x) * int(sizeof(float)), gper * P + y,
                    cudaBoundaryModeZero);
}

// emit against the unit box; returns nsteps, sets o and d
__device__ __forceinline__ int diff_emit(const DiffArgs &a, int view, int x, int y, float &ox,
                                         float &oy, float &oz, float &dx, float &dy, float &dz) {
    const DiffView &vw = a.views[view];
    ViewArgs va;
    // gen_ray reads trans / ctg / ray_o / W / H only
    for (int i = 0; i < 16; ++i) va.trans[i] = vw.trans[i];
    va.ctg = vw.ctg;
    va.ray_o[0] = vw.ray_o[0];
    va.ray_o[1] = vw.ray_o[1];
    va.ray_o[2] = vw.ray_o[2];
    va.W = a.W;
    va.H = a.H;
    gen_ray(va, x, y, ox, oy, oz, dx, dy, dz);
    float tnear, tfar;
    if (!intersect(ox, oy, oz, 1.f / dx, 1.f / dy, 1.f / dz, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f, tnear,
                   tfar))
        return 0;
    if (tnear < 0) tnear = 0;
    if (tfar < 0) tfar = 0;
    ox = ox + dx * tnear;
    oy = oy + dy * tnear;
    oz = oz + dz * tnear;
    return min(a.max_steps, int((tfar - tnear) / a.step));
}

// transfer function value and its derivative in s
__device__ __forceinline__ float4 tf_eval(const float4 *tf, int n, float s, int &i, int &j,
                                          float &al, bool &inb) {
    const float fn = float(n);
    const float fx = fn * s;
    inb = (0.f <= fx && fx <= fn);
    if (!inb) {
        i = j = 0;
        al = 0.f;
        return make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const float u = fx - .5f;
    const float flr = floorf(u);
    al = u - flr;
    const int fi = int(flr);
    i = max(fi, 0);
    j = min(fi + 1, n - 1);
    const float4 p = tf[i], q = tf[j];
    const float bb = 1.f - al;
    const float2 b2 = f2(bb, bb), a2 = f2(al, al);
    const float2 rg = lerp2(f2(p.x, p.y), b2, f2(q.x, q.y), a2);
    const float2 ba = lerp2(f2(p.z, p.w), b2, f2(q.z, q.w), a2);
    return make_float4(rg.x, rg.y, ba.x, ba.y);
}

__device__ __forceinline__ void pixel_of(const DiffArgs &a, int &x, int &y, int &view) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
    y = blockIdx.y * 8 + (warp >> 1) * 4 + (lane >> 3);
    view = blockIdx.z;
}

template <bool GATHER>
__global__ void __launch_bounds__(128) diff_forward_kernel(const __grid_constant__ DiffArgs a) {
    __shared__ float4 tf[kMaxKnots];
    for (int i = threadIdx.x; i < a.ntf; i += blockDim.x) tf[i] = a.tf[i];
    __syncthreads();
    int x, y, view;
    pixel_of(a, x, y, view);
    if (x >= a.W || y >= a.H) return;
    const size_t ray = (size_t(view) * a.H + y) * a.W + x;
    float ox, oy, oz, dx, dy, dz;
    const int nsteps = diff_emit(a, view, x, y, ox, oy, oz, dx, dy, dz);
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    const float sx = dx * a.step, sy = dy * a.step, sz = dz * a.step;  // step_size 1
    float4 *cp = a.ckpt ? a.ckpt + ray * a.max_ckpt : nullptr;
    int until_ckpt = 0;  // a checkpoint before steps 0, K, 2K, ...
    for (int s = 0; s < nsteps; ++s) {
        if (until_ckpt == 0) {
            if (cp) *cp++ = make_float4(ox, oy, oz, v.w);
            until_ckpt = a.K;
        }
        --until_ckpt;
        const float ipx = floorf(ox), ipy = floorf(oy), ipz = floorf(oz);
        const float val = GATHER ? diff_sample_gather(a, ox - ipx, oy - ipy, oz - ipz)
                                 : diff_sample(a, ox - ipx, oy - ipy, oz - ipz);
        int i, j;
        float al;
        bool inb;
        float4 ub = tf_eval(tf, a.ntf, val, i, j, al, inb);
        ub.w = ub.w * a.density;
        const float w = ub.w;
        const float2 uxy = mul2(f2(ub.x, ub.y), f2(w, w));
        ub.z = ub.z * w;
        const float t = 1.f - v.w;
        // packed products, scalar sums (see mul2)
        const float2 txy = mul2(uxy, f2(t, t)), tzw = mul2(f2(ub.z, ub.w), f2(t, t));
        v.x = __fadd_rn(v.x, txy.x);
        v.y = __fadd_rn(v.y, txy.y);
        v.z = __fadd_rn(v.z, tzw.x);
        v.w = __fadd_rn(v.w, tzw.y);
        ox = ox + sx;
        oy = oy + sy;
        oz = oz + sz;
    }
    a.image[ray] = v;
    if (a.nsteps_out) a.nsteps_out[ray] = nsteps;
}

// Gradient accumulators of one ray.  Consecutive samples mostly share a knot
// interval and a voxel cell, so gradients are summed in registers and flushed
// (one atomic per knot channel / cell corner) only when those change.
struct GradAcc {
    int ki = -1, kj = -1;
    float4 acc_i = make_float4(0.f, 0.f, 0.f, 0.f), acc_j = make_float4(0.f, 0.f, 0.f, 0.f);
    Cell cell;
    bool has_cell = false;
    float cacc[8];

    __device__ __forceinline__ void flush_knots(float4 *gtf) {
        if (ki < 0) return;
        atomicAdd(&gtf[ki].x, acc_i.x);
        atomicAdd(&gtf[ki].y, acc_i.y);
        atomicAdd(&gtf[ki].z, acc_i.z);
        atomicAdd(&gtf[ki].w, acc_i.w);
        atomicAdd(&gtf[kj].x, acc_j.x);
        atomicAdd(&gtf[kj].y, acc_j.y);
        atomicAdd(&gtf[kj].z, acc_j.z);
        atomicAdd(&gtf[kj].w, acc_j.w);
        acc_i = make_float4(0.f, 0.f, 0.f, 0.f);
        acc_j = acc_i;
    }
    __device__ __forceinline__ void flush_cell(float *dvol) {
        if (!has_cell) return;
        const int idx[8] = {cell.r00 + cell.x0, cell.r00 + cell.x1, cell.r10 + cell.x0,
                            cell.r10 + cell.x1, cell.r01 + cell.x0, cell.r01 + cell.x1,
                            cell.r11 + cell.x0, cell.r11 + cell.x1};
#pragma unroll
        for (int t = 0; t < 8; ++t)
            if (cacc[t] != 0.f) atomicAdd(dvol + idx[t], cacc[t]);
    }
};

// Back-propagates one sample: its position's cell, its value `val`, the
// transmittance T before it and R (the colour composited behind it, updated
// to include this sample).
__device__ __forceinline__ void diff_adjoint_sample(const DiffArgs &a, const float4 *tf,
                                                    float4 *gtf, GradAcc &G, const float4 &g,
                                                    float4 &R, float px, float py, float pz,
                                                    float val, float T) {
    int i, j;
    float al;
    bool inb;
    const float4 q = tf_eval(tf, a.ntf, val, i, j, al, inb);
    const float aa = q.w * a.density;
    // The gradient arithmetic has no float-exact counterpart to follow, so it
    // uses fused multiply-adds (the file is compiled with contraction off).
    // dL/dc = T g ; transmittance term through later samples
    const float2 gcxy = mul2(f2(T, T), f2(g.x, g.y)), gczw = mul2(f2(T, T), f2(g.z, g.w));
    const float gcx = gcxy.x, gcy = gcxy.y, gcz = gczw.x, gcw = gczw.y;
    const float gdot = __fmaf_rn(g.w, R.w, __fmaf_rn(g.z, R.z, __fmaf_rn(g.y, R.y, g.x * R.x)));
    const float da =
        __fmaf_rn(-T, gdot, __fmaf_rn(gcz, q.z, __fmaf_rn(gcy, q.y, __fmaf_rn(gcx, q.x, gcw))));
    // R_n = c_n + (1 - a_n) R_{n+1}
    const float om = 1.f - aa;
    const float2 om2 = f2(om, om);
    const float2 Rxy = fma2(om2, f2(R.x, R.y), mul2(f2(q.x, q.y), f2(aa, aa)));
    const float2 Rzw = fma2(om2, f2(R.z, R.w), f2(q.z * aa, aa));
    R = make_float4(Rxy.x, Rxy.y, Rzw.x, Rzw.y);
    if (!inb) return;
    // gradient of the TF output (r, g, b, A)
    const float2 gqxy = mul2(gcxy, f2(aa, aa)), gqzw = mul2(f2(gcz, da), f2(aa, a.density));
    const float4 gq = make_float4(gqxy.x, gqxy.y, gqzw.x, gqzw.y);
    const float bb = 1.f - al;
    if (i != G.ki || j != G.kj) {
        G.flush_knots(gtf);
        G.ki = i;
        G.kj = j;
    }
    {
        const float2 b2 = f2(bb, bb), a2 = f2(al, al);
        const float2 ixy = fma2(gqxy, b2, f2(G.acc_i.x, G.acc_i.y));
        const float2 izw = fma2(gqzw, b2, f2(G.acc_i.z, G.acc_i.w));
        const float2 jxy = fma2(gqxy, a2, f2(G.acc_j.x, G.acc_j.y));
        const float2 jzw = fma2(gqzw, a2, f2(G.acc_j.z, G.acc_j.w));
        G.acc_i = make_float4(ixy.x, ixy.y, izw.x, izw.y);
        G.acc_j = make_float4(jxy.x, jxy.y, jzw.x, jzw.y);
    }
    // d TF / d s = (knot_j - knot_i) * n
    const float4 kj = tf[j], ki = tf[i];
    const float fn = float(a.ntf);
    const float ds = fn * __fmaf_rn(gq.w, kj.w - ki.w,
                                    __fmaf_rn(gq.z, kj.z - ki.z,
                                              __fmaf_rn(gq.y, kj.y - ki.y, gq.x * (kj.x - ki.x))));
    if (ds == 0.f) return;
    Cell c;
    diff_cell(a, px - floorf(px), py - floorf(py), pz - floorf(pz), c);
    if (!G.has_cell || c.r00 + c.x0 != G.cell.r00 + G.cell.x0 ||
        c.r11 + c.x1 != G.cell.r11 + G.cell.x1) {
        G.flush_cell(a.dvol);
        G.cell = c;
        G.has_cell = true;
#pragma unroll
        for (int t = 0; t < 8; ++t) G.cacc[t] = 0.f;
    }
    // trilinear weights w = (x-weight) * (y-weight) * (z-weight), times ds
    const float ax = c.ax, ay = c.ay, az = c.az;
    const float bx = 1.f - ax, by = 1.f - ay, bz = 1.f - az;
    const float2 ds2 = f2(ds, ds), yw = f2(by, ay);
    const float2 dz0 = mul2(ds2, mul2(yw, f2(bz, bz)));  // (d00, d10)
    const float2 dz1 = mul2(ds2, mul2(yw, f2(az, az)));  // (d01, d11)
    const float2 xw = f2(bx, ax);
    const float2 c01 = fma2(xw, f2(dz0.x, dz0.x), f2(G.cacc[0], G.cacc[1]));
    const float2 c23 = fma2(xw, f2(dz0.y, dz0.y), f2(G.cacc[2], G.cacc[3]));
    const float2 c45 = fma2(xw, f2(dz1.x, dz1.x), f2(G.cacc[4], G.cacc[5]));
    const float2 c67 = fma2(xw, f2(dz1.y, dz1.y), f2(G.cacc[6], G.cacc[7]));
    G.cacc[0] = c01.x;
    G.cacc[1] = c01.y;
    G.cacc[2] = c23.x;
    G.cacc[3] = c23.y;
    G.cacc[4] = c45.x;
    G.cacc[5] = c45.y;
    G.cacc[6] = c67.x;
    G.cacc[7] = c67.y;
}

// The adjoint walks a ray's segments back to front; a segment's recomputed
// sample values and transmittances sit in a per-thread array (8 bytes per
// step), and the reverse walk recomputes each sample position from the
// checkpoint as c + s * step (one rounding per axis instead of the forward's
// s additions: the positions agree to a few ulps, and the trilinear weights'
// derivative is continuous across cell faces, so a sample that lands in the
// neighbouring cell gets the same gradient to first order).
// HY_DIFF_MIN_BLOCKS: resident 128-thread blocks per SM the register budget
// is fitted to.  6 (80 registers, 36 bytes spilled, 24 warps) against the
// compiler's 96 registers and 20 warps, 256^3 f32, 16 views of 512^2, K = 32:
// adjoint 2.35 vs 2.55 ms/view; 8 (64 registers, 100 bytes spilled): 2.45.
#ifndef HY_DIFF_MIN_BLOCKS
#define HY_DIFF_MIN_BLOCKS 6
#endif
template <bool GATHER>
__global__ void __launch_bounds__(128, HY_DIFF_MIN_BLOCKS)
    diff_backward_kernel(const __grid_constant__ DiffArgs a) {
    __shared__ float4 tf[kMaxKnots];
    __shared__ float4 gtf[kMaxKnots];
    for (int i = threadIdx.x; i < a.ntf; i += blockDim.x) {
        tf[i] = a.tf[i];
        gtf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    int x, y, view;
    pixel_of(a, x, y, view);
    if (x < a.W && y < a.H) {
        const size_t ray = (size_t(view) * a.H + y) * a.W + x;
        const int nsteps = a.nsteps_out[ray];
        const float4 g = a.dimage[ray];
        float ox0, oy0, oz0, dx, dy, dz;
        diff_emit(a, view, x, y, ox0, oy0, oz0, dx, dy, dz);
        const float sx = dx * a.step, sy = dy * a.step, sz = dz * a.step;
        float4 R = make_float4(0.f, 0.f, 0.f, 0.f);
        const int K = a.K;
        float2 seg_vw[kMaxK];  // (sample value, v.w before the sample)
        const int nseg = (nsteps + K - 1) / K;
        GradAcc G;
        const float4 *cps = a.ckpt + ray * a.max_ckpt;
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const float4 c = cps[seg];
            float ox = c.x, oy = c.y, oz = c.z, vw = c.w;
            const int cnt = min(K, nsteps - seg * K);
            // recompute the segment: values and v.w before each sample
            for (int s = 0; s < cnt; ++s) {
                const float ipx = floorf(ox), ipy = floorf(oy), ipz = floorf(oz);
                const float val = GATHER ? diff_sample_gather(a, ox - ipx, oy - ipy, oz - ipz)
                                         : diff_sample(a, ox - ipx, oy - ipy, oz - ipz);
                seg_vw[s] = make_float2(val, vw);
                int i, j;
                float al;
                bool inb;
                const float4 ub = tf_eval(tf, a.ntf, val, i, j, al, inb);
                const float aa = ub.w * a.density;
                vw = vw + aa * (1.f - vw);
                ox = ox + sx;
                oy = oy + sy;
                oz = oz + sz;
            }
            for (int s = cnt - 1; s >= 0; --s) {
                const float fs = float(s);
                const float2 e = seg_vw[s];
                diff_adjoint_sample(a, tf, gtf, G, g, R, __fmaf_rn(fs, sx, c.x),
                                    __fmaf_rn(fs, sy, c.y), __fmaf_rn(fs, sz, c.z), e.x,
                                    1.f - e.y);
            }
        }
        G.flush_knots(gtf);
        G.flush_cell(a.dvol);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < a.ntf; i += blockDim.x) {
        const float4 v = gtf[i];
        if (v.x != 0.f) atomicAdd(a.dtf + 4 * i + 0, v.x);
        if (v.y != 0.f) atomicAdd(a.dtf + 4 * i + 1, v.y);
        if (v.z != 0.f) atomicAdd(a.dtf + 4 * i + 2, v.z);
        if (v.w != 0.f) atomicAdd(a.dtf + 4 * i + 3, v.w);
    }
}

int fill_diff(hy_ctx *ctx, const hy_diff_params *p, const float *vol, const float *tf,
              const hy_view *views, int nviews, int W, int H, DiffArgs &a) {
    if (!p || !vol || !tf || !views) return hy_fail(ctx, HY_ERR_INVALID, "diff: null argument");
    if (p->n <= 1) return hy_fail(ctx, HY_ERR_INVALID, "diff: volume edge must be > 1");
    if ((long long)p->n * p->n * p->n >= (1LL << 31))
        return hy_fail(ctx, HY_ERR_INVALID, "diff: volume edge must be <= 1290 (n^3 < 2^31)");
    if (nviews <= 0 || nviews > kMaxDiffViews)
        return hy_fail(ctx, HY_ERR_INVALID, "diff: 1..64 views");
    // the launch grid is W/16 x H/8 tiles (at most 65535 tile rows) per view
    if (W <= 0 || H <= 0 || (long long)W * H > (1ll << 31) || (H + 7) / 8 > 65535)
        return hy_fail(ctx, HY_ERR_INVALID, "diff: bad resolution");
    if (p->ntf <= 0 || p->ntf > kMaxKnots) return hy_fail(ctx, HY_ERR_INVALID, "diff: 1..256 knots");
    if (p->ckpt_k <= 0 || p->ckpt_k > kMaxK)
        return hy_fail(ctx, HY_ERR_INVALID, "diff: checkpoint interval 1..64");
    if (!(p->sample_rate > 0.f)) return hy_fail(ctx, HY_ERR_INVALID, "diff: sample_rate <= 0");
    std::memset(&a, 0, sizeof(a));
    a.vol = vol;
    a.n = p->n;
    // one brick of edge n with a 1-voxel apron (lossless_block_paging.cc:20-22)
    a.k = float(p->n) / float(p->n + 2);
    a.b = float(1) / float(p->n) * a.k;
    const float du = 1.f / float(p->n);
    a.step = du / 4.f / p->sample_rate;
    a.max_steps = p->max_steps;
    a.density = p->density;
    a.tf = reinterpret_cast<const float4 *>(tf);
    a.ntf = p->ntf;
    a.K = p->ckpt_k;
    // the unit box's diagonal bounds every ray's step count
    const long long maxn = std::min<long long>(p->max_steps, (long long)(1.7320509f / a.step) + 2);
    a.max_ckpt = int((maxn + a.K - 1) / a.K) + 1;
    a.W = W;
    a.H = H;
    a.nviews = nviews;
    for (int v = 0; v < nviews; ++v) {
        std::memcpy(a.views[v].trans, views[v].trans, sizeof(a.views[v].trans));
        a.views[v].ctg = views[v].ctg_fovy_2;
        for (int i = 0; i < 3; ++i) a.views[v].ray_o[i] = views[v].ray_o[i];
    }
    return HY_OK;
}

dim3 diff_grid(const DiffArgs &a) { return dim3((a.W + 15) / 16, (a.H + 7) / 8, a.nviews); }

// HY_DIFF_GATHER: the adjoint's segment recompute (1) -- and the forward
// too (2) -- sample the volume through a gather texture refreshed from the
// caller's volume at each call (the refresh inside the timed launch); 0:
// loads only.  256^3 f32, 16 views of 512^2, 32 knots, K = 32, per view:
//   0: forward 1.34 ms, forward + adjoint 3.70 ms (2.79x), fit iteration 59.9 ms
//   1: forward 1.34 ms, forward + adjoint 3.45 ms (2.58x), fit iteration 55.1 ms
//   2: forward 0.88 ms, forward + adjoint 2.97 ms (3.38x), fit iteration 47.5 ms
// 1 is the default: 2 gives the fastest fit, but its forward + adjoint is
// more than three times its (faster) forward.
#ifndef HY_DIFF_GATHER
#define HY_DIFF_GATHER 1
#endif
struct DiffGather {
    cudaArray_t arr = nullptr;
    unsigned long long tex = 0, surf = 0;
    int n = 0, gper = 0;
};

void free_diff_gather(DiffGather *g) {
    if (!g) return;
    if (g->surf) cudaDestroySurfaceObject(cudaSurfaceObject_t(g->surf));
    if (g->tex) cudaDestroyTextureObject(cudaTextureObject_t(g->tex));
    if (g->arr) cudaFreeArray(g->arr);
    delete g;
}

// The context's texture of an n^3 volume, (re)made for n, filled from vol on
// the stream.  *ok = false (no error) when this device cannot make it (an
// edge too large for a gather texture, or no memory left): the caller then
// samples by loads.
int diff_gather_refresh(hy_ctx *ctx, const float *vol, int n, DiffArgs &a, bool *ok) {
    *ok = false;
    DiffGather *g = static_cast<DiffGather *>(ctx->diff_gather);
    if (!g || g->n != n) {
        free_diff_gather(g);
        ctx->diff_gather = nullptr;
        int gw = 0, gh = 0;
        HY_CUDA(ctx, cudaDeviceGetAttribute(&gw, cudaDevAttrMaxTexture2DGatherWidth, ctx->device));
        HY_CUDA(ctx, cudaDeviceGetAttribute(&gh, cudaDevAttrMaxTexture2DGatherHeight, ctx->device));
        const int P = n + 2;
        const int gper = gh / P - 1;  // slices per column, plus the repeated one
        if (gper < 1) return HY_OK;
        const int cols = (P - 2) / gper + 1;  // columns of the footprints' lower slices
        if ((long long)cols * P > gw) return HY_OK;
        g = new DiffGather();
        g->n = n;
        g->gper = gper;
        cudaChannelFormatDesc cd = cudaCreateChannelDesc(32, 0, 0, 0, cudaChannelFormatKindFloat);
        cudaError_t e = cudaMallocArray(&g->arr, &cd, size_t(cols) * P, size_t(gper + 1) * P,
                                        cudaArrayTextureGather | cudaArraySurfaceLoadStore);
        cudaResourceDesc rd;
        std::memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = g->arr;
        cudaTextureDesc td;
        std::memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        cudaTextureObject_t t = 0;
        cudaSurfaceObject_t so = 0;
        if (e == cudaSuccess) e = cudaCreateTextureObject(&t, &rd, &td, nullptr);
        if (e == cudaSuccess) g->tex = (unsigned long long)t;
        if (e == cudaSuccess) e = cudaCreateSurfaceObject(&so, &rd);
        if (e == cudaSuccess) g->surf = (unsigned long long)so;
        if (e != cudaSuccess) {  // e.g. no room: the loads serve this call
            free_diff_gather(g);
            cudaGetLastError();
            return HY_OK;
        }
        ctx->diff_gather = g;
    }
    const int P = n + 2;
    diff_fill_kernel<<<dim3((P + 127) / 128, P, P), 128, 0, ctx->stream>>>(vol, n, g->gper,
                                                                          g->surf);
    HY_CUDA(ctx, cudaGetLastError());
    a.gtex = g->tex;
    a.gper = g->gper;
    *ok = true;
    return HY_OK;
}

}  // namespace

extern "C" int hy_diff_ckpt_bytes(const hy_diff_params *p, int32_t W, int32_t H, int32_t nviews,
                                  int64_t *bytes) {
    if (!p || !bytes || p->ckpt_k <= 0 || p->n <= 1 || !(p->sample_rate > 0.f))
        return HY_ERR_INVALID;
    const float step = 1.f / float(p->n) / 4.f / p->sample_rate;
    const long long maxn = std::min<long long>(p->max_steps, (long long)(1.7320509f / step) + 2);
    const long long per_ray = (maxn + p->ckpt_k - 1) / p->ckpt_k + 1;
    *bytes = (int64_t)per_ray * 16 * W * H * nviews;
    return HY_OK;
}

extern "C" int hy_diff_forward(hy_ctx *ctx, const hy_diff_params *p, const float *vol_dev,
                               const float *tf_dev, const hy_view *views, int32_t nviews,
                               int32_t W, int32_t H, float *image_dev, float *ckpt_dev,
                               int32_t *nsteps_dev) {
    if (!ctx) return HY_ERR_INVALID;
    // float4 records: knots, image, checkpoints; scalars: volume, step counts
    if (!hy_aligned(tf_dev, 16) || !hy_aligned(image_dev, 16) || !hy_aligned(ckpt_dev, 16) ||
        !hy_aligned(vol_dev, 4) || !hy_aligned(nsteps_dev, 4))
        return hy_fail(ctx, HY_ERR_INVALID,
                       "diff: misaligned buffer (knots, image, checkpoints 16-byte; others 4)");
    if (!image_dev) return hy_fail(ctx, HY_ERR_INVALID, "diff: null image");
    DiffArgs a;
    int rc = fill_diff(ctx, p, vol_dev, tf_dev, views, nviews, W, H, a);
    if (rc) return rc;
    if ((ckpt_dev == nullptr) != (nsteps_dev == nullptr))
        return hy_fail(ctx, HY_ERR_INVALID, "diff: checkpoints and step counts go together");
    a.image = reinterpret_cast<float4 *>(image_dev);
    a.ckpt = reinterpret_cast<float4 *>(ckpt_dev);
    a.nsteps_out = nsteps_dev;
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    // the texture's refresh is part of the timed launch
    HY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    bool gathers = false;
    if (HY_DIFF_GATHER >= 2) {
        rc = diff_gather_refresh(ctx, vol_dev, p->n, a, &gathers);
        if (rc) return rc;
    }
    if (gathers)
        diff_forward_kernel<true><<<diff_grid(a), 128, 0, ctx->stream>>>(a);
    else
        diff_forward_kernel<false><<<diff_grid(a), 128, 0, ctx->stream>>>(a);
    HY_CUDA(ctx, cudaGetLastError());
    HY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->stats_pending = true;
    ctx->pend_count = 0;
    ctx->pend_pixels = (int64_t)W * H * nviews;
    return HY_OK;
}

extern "C" int hy_diff_backward(hy_ctx *ctx, const hy_diff_params *p, const float *vol_dev,
                                const float *tf_dev, const hy_view *views, int32_t nviews,
                                int32_t W, int32_t H, const float *dimage_dev,
                                const float *ckpt_dev, const int32_t *nsteps_dev,
                                float *dvol_dev, float *dtf_dev) {
    if (!ctx) return HY_ERR_INVALID;
    if (!hy_aligned(tf_dev, 16) || !hy_aligned(dimage_dev, 16) || !hy_aligned(ckpt_dev, 16) ||
        !hy_aligned(vol_dev, 4) || !hy_aligned(nsteps_dev, 4) || !hy_aligned(dvol_dev, 4) ||
        !hy_aligned(dtf_dev, 4))
        return hy_fail(ctx, HY_ERR_INVALID,
                       "diff: misaligned buffer (knots, image, checkpoints 16-byte; others 4)");
    if (!dimage_dev || !ckpt_dev || !nsteps_dev || !dvol_dev || !dtf_dev)
        return hy_fail(ctx, HY_ERR_INVALID, "diff: null argument");
    DiffArgs a;
    int rc = fill_diff(ctx, p, vol_dev, tf_dev, views, nviews, W, H, a);
    if (rc) return rc;
    a.dimage = reinterpret_cast<const float4 *>(dimage_dev);
    a.ckpt = const_cast<float4 *>(reinterpret_cast<const float4 *>(ckpt_dev));
    a.nsteps_out = const_cast<int *>(nsteps_dev);
    a.dvol = dvol_dev;
    a.dtf = dtf_dev;
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    // the texture's refresh is part of the timed launch
    HY_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    bool gathers = false;
    if (HY_DIFF_GATHER >= 1) {
        rc = diff_gather_refresh(ctx, vol_dev, p->n, a, &gathers);
        if (rc) return rc;
    }
    if (gathers)
        diff_backward_kernel<true><<<diff_grid(a), 128, 0, ctx->stream>>>(a);
    else
        diff_backward_kernel<false><<<diff_grid(a), 128, 0, ctx->stream>>>(a);
    HY_CUDA(ctx, cudaGetLastError());
    HY_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->stats_pending = true;
    ctx->pend_count = 0;
    ctx->pend_pixels = (int64_t)W * H * nviews;
    return HY_OK;
}

void hy_diff_release(hy_ctx *ctx) {
    if (!ctx) return;
    free_diff_gather(static_cast<DiffGather *>(ctx->diff_gather));
    ctx->diff_gather = nullptr;
}
