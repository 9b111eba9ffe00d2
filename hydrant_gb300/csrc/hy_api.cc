// hy_api.cc -- context, errors, transfer function, camera helpers.
//
// Compiled with -ffp-contract=off: the camera helpers must round every
// multiply and add separately, like the reference's host code.

#include <cmath>
#include <cstring>

#include "hy_internal.h"

int hy_fail(hy_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int hy_cuda_fail(hy_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return hy_fail(ctx, e == cudaErrorMemoryAllocation ? HY_ERR_OOM : HY_ERR_CUDA, m);
}

int hy_stage(hy_ctx *ctx, size_t bytes, void **out) {
    if (bytes > ctx->stage_bytes) {
        if (ctx->stage) {
            HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFree(ctx->stage);
            ctx->stage = nullptr;
            ctx->stage_bytes = 0;
        }
        HY_CUDA(ctx, cudaMalloc(&ctx->stage, bytes));
        ctx->stage_bytes = bytes;
    }
    *out = ctx->stage;
    return HY_OK;
}

extern "C" int hy_ctx_create(int device, hy_ctx **out) {
    if (!out) return HY_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return HY_ERR_CUDA;
    if (device < 0 || device >= n) return HY_ERR_INVALID;
    hy_ctx *ctx = new hy_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->counter_dev, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e != cudaSuccess) {
        hy_ctx_destroy(ctx);
        return HY_ERR_CUDA;
    }
    *out = ctx;
    return HY_OK;
}

extern "C" int hy_ctx_destroy(hy_ctx *ctx) {
    if (!ctx) return HY_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->tf_dev) cudaFree(ctx->tf_dev);
    if (ctx->counter_dev) cudaFree(ctx->counter_dev);
    if (ctx->stage) cudaFree(ctx->stage);
    hy_diff_release(ctx);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HY_OK;
}

extern "C" const char *hy_last_error(const hy_ctx *ctx) { return ctx ? ctx->err.c_str() : ""; }

extern "C" int hy_ctx_synchronize(hy_ctx *ctx) {
    if (!ctx) return HY_ERR_INVALID;
    HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HY_OK;
}

extern "C" void *hy_ctx_stream(hy_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int hy_render_stats_get(hy_ctx *ctx, hy_render_stats *out) {
    if (!ctx || !out) return HY_ERR_INVALID;
    int rc = hy_finish_stats(ctx);
    if (rc) return rc;
    *out = ctx->stats;
    return HY_OK;
}

// TransferFn (transfer_fn.hpp:16-23): knots live in device memory and each
// launch stages them in shared memory.
extern "C" int hy_tf_set(hy_ctx *ctx, const float *rgba, int32_t n) {
    if (!ctx) return HY_ERR_INVALID;
    if (!rgba || n <= 0 || n > 2048) return hy_fail(ctx, HY_ERR_INVALID, "tf: need 1..2048 knots");
    HY_CUDA(ctx, cudaSetDevice(ctx->device));
    if (n > ctx->tf_cap) {
        if (ctx->tf_dev) {
            HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFree(ctx->tf_dev);
            ctx->tf_dev = nullptr;
        }
        HY_CUDA(ctx, cudaMalloc(&ctx->tf_dev, size_t(n) * sizeof(float4)));
        ctx->tf_cap = n;
    }
    HY_CUDA(ctx, cudaMemcpyAsync(ctx->tf_dev, rgba, size_t(n) * sizeof(float4),
                                 cudaMemcpyHostToDevice, ctx->stream));
    HY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->ntf = n;
    return HY_OK;
}

// ---------------------------------------------------------------------------
// Camera helpers: Camera (scene.hpp:32-82), Exhibit::get_iet (scene.hpp:20-29),
// Raycaster::fill_ray_emit_args (raycaster.hpp:249-258), light/eye of
// IsosurfaceRenderer (isosurface.cc:108-113).  Matrices are column-major
// (element (row r, column c) at m[4c + r]); sums run left to right.
// ---------------------------------------------------------------------------
namespace {

struct V3 {
    float v[3];
};
V3 v3(float a, float b, float c) { return V3{{a, b, c}}; }
float vdot(const V3 &a, const V3 &b) { return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2]; }
V3 vsub(const V3 &a, const V3 &b) { return v3(a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]); }
V3 vadd(const V3 &a, const V3 &b) { return v3(a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]); }
V3 vscale(const V3 &a, float s) { return v3(a.v[0] * s, a.v[1] * s, a.v[2] * s); }
V3 vnormalize(const V3 &a) { return vscale(a, 1.f / std::sqrt(vdot(a, a))); }
V3 vcross(const V3 &a, const V3 &b) {
    return v3(a.v[1] * b.v[2] - b.v[1] * a.v[2], a.v[2] * b.v[0] - b.v[2] * a.v[0],
              a.v[0] * b.v[1] - b.v[0] * a.v[1]);
}
float fmax_(float a, float b) { return (a < b) ? b : a; }

void mat_vec(const float m[16], const float x[4], float out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = m[r] * x[0] + m[4 + r] * x[1] + m[8 + r] * x[2] + m[12 + r] * x[3];
}
void mat_mul(const float a[16], const float b[16], float out[16]) {
    for (int c = 0; c < 4; ++c) mat_vec(a, &b[4 * c], &out[4 * c]);
}
// 4x4 inverse: adjugate (cofactors) divided by the determinant.
void mat_inverse(const float m[16], float out[16]) {
    // minors of the 2x2 blocks, then cofactors
    float c[16];
    c[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] +
           m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    c[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] -
           m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    c[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] +
           m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    c[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] -
           m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    c[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] -
           m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    c[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] +
           m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    c[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] -
           m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    c[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] +
           m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    c[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] +
           m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    c[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] -
           m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    c[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] +
            m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    c[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] -
            m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    c[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] -
            m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    c[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] +
            m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    c[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] -
            m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    c[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] +
            m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    float det = m[0] * c[0] + m[1] * c[4] + m[2] * c[8] + m[3] * c[12];
    float r = 1.f / det;
    for (int i = 0; i < 16; ++i) out[i] = c[i] * r;
}
void mat_identity(float m[16]) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.f : 0.f;
}
// rotation by `angle` radians about `axis`: cI + (1-c) k k^T + s [k]x
void mat_rotation(float angle, V3 axis, float m[16]) {
    float c = std::cos(angle), s = std::sin(angle);
    V3 k = vnormalize(axis);
    V3 t = vscale(k, 1.f - c);
    mat_identity(m);
    m[0] = c + t.v[0] * k.v[0];
    m[1] = t.v[0] * k.v[1] + s * k.v[2];
    m[2] = t.v[0] * k.v[2] - s * k.v[1];
    m[4] = t.v[1] * k.v[0] - s * k.v[2];
    m[5] = c + t.v[1] * k.v[1];
    m[6] = t.v[1] * k.v[2] + s * k.v[0];
    m[8] = t.v[2] * k.v[0] + s * k.v[1];
    m[9] = t.v[2] * k.v[1] - s * k.v[0];
    m[10] = c + t.v[2] * k.v[2];
}
// right-handed world -> eye matrix
void mat_look_at(V3 eye, V3 center, V3 up, float m[16]) {
    V3 f = vnormalize(vsub(center, eye));
    V3 s = vnormalize(vcross(f, up));
    V3 u = vcross(s, f);
    mat_identity(m);
    for (int i = 0; i < 3; ++i) {
        m[4 * i + 0] = s.v[i];
        m[4 * i + 1] = u.v[i];
        m[4 * i + 2] = -f.v[i];
    }
    m[12] = -vdot(s, eye);
    m[13] = -vdot(u, eye);
    m[14] = vdot(f, eye);
}
float deg2rad(float d) { return d * 0.01745329251994329576923690768489f; }

// Exhibit{center = f_dim/2, size = f_dim}.get_iet(): object = scale*world + center
void exhibit_iet(const hy_volume *vol, float m[16]) {
    float c[3], d[3];
    for (int i = 0; i < 3; ++i) {
        c[i] = vol->bbox_max[i] / 2.f;
        d[i] = fmax_(std::fabs(c[i] - vol->bbox_max[i]), std::fabs(c[i]));
    }
    float scale = fmax_(fmax_(d[0], d[1]), d[2]);
    for (int i = 0; i < 16; ++i) m[i] = 0.f;
    m[0] = m[5] = m[10] = scale;
    m[12] = c[0];
    m[13] = c[1];
    m[14] = c[2];
    m[15] = 1.f;
}

}  // namespace

extern "C" int hy_camera_orbit(const float arm[3], const float center[3], float fovy_deg,
                               hy_camera *out) {
    if (!arm || !out) return HY_ERR_INVALID;
    float rz[16], ry[16], p[4], q[4];
    mat_rotation(deg2rad(arm[1]), v3(0, 0, 1), rz);
    const float x0[4] = {arm[2], 0.f, 0.f, 1.f};
    mat_vec(rz, x0, p);
    mat_rotation(deg2rad(arm[0]), v3(0, 1, 0), ry);
    const float x1[4] = {p[0], p[1], p[2], 1.f};
    mat_vec(ry, x1, q);
    for (int i = 0; i < 3; ++i) {
        out->position[i] = q[i];
        out->target[i] = center ? center[i] : 0.f;
        out->up[i] = i == 1 ? 1.f : 0.f;
    }
    out->ctg_fovy_2 = 1.f / std::tan(deg2rad(fovy_deg / 2.f));
    return HY_OK;
}

extern "C" int hy_camera_ptu(const float position[3], const float target[3], const float up[3],
                             float fovy_deg, hy_camera *out) {
    if (!position || !target || !up || !out) return HY_ERR_INVALID;
    for (int i = 0; i < 3; ++i) {
        out->position[i] = position[i];
        out->target[i] = target[i];
        out->up[i] = up[i];
    }
    out->ctg_fovy_2 = 1.f / std::tan(deg2rad(fovy_deg / 2.f));
    return HY_OK;
}

extern "C" int hy_camera_view(const hy_volume *vol, const hy_camera *cam, hy_view *out) {
    if (!vol || !cam || !out) return HY_ERR_INVALID;
    float iet[16], vt[16], ivt[16];
    exhibit_iet(vol, iet);
    V3 eye = v3(cam->position[0], cam->position[1], cam->position[2]);
    mat_look_at(eye, v3(cam->target[0], cam->target[1], cam->target[2]),
                v3(cam->up[0], cam->up[1], cam->up[2]), vt);
    mat_inverse(vt, ivt);
    mat_mul(iet, ivt, out->trans);
    out->ctg_fovy_2 = cam->ctg_fovy_2;
    const float e4[4] = {eye.v[0], eye.v[1], eye.v[2], 1.f};
    float o[4];
    mat_vec(iet, e4, o);
    for (int i = 0; i < 3; ++i) out->ray_o[i] = o[i];
    return HY_OK;
}

extern "C" int hy_iso_lighting(const hy_volume *vol, const hy_camera *cam, hy_shader_params *p) {
    if (!vol || !cam || !p) return HY_ERR_INVALID;
    float iet[16];
    exhibit_iet(vol, iet);
    mat_inverse(iet, p->to_world);
    V3 pos = v3(cam->position[0], cam->position[1], cam->position[2]);
    V3 tgt = v3(cam->target[0], cam->target[1], cam->target[2]);
    V3 up = v3(cam->up[0], cam->up[1], cam->up[2]);
    V3 l = vadd(vadd(vadd(pos, tgt), up), vcross(tgt, up));
    for (int i = 0; i < 3; ++i) {
        p->light_pos[i] = l.v[i];
        p->eye_pos[i] = pos.v[i];
    }
    return HY_OK;
}
