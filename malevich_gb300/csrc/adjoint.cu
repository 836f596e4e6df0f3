// Differentiable shading and its hand-written adjoint (mlv_diff_forward / mlv_diff_backward).
//
// The reference's barycentrics are quantised (source/main.c:1092-1102): piecewise constant in the
// vertex positions, with zero gradient almost everywhere. The differentiable path keeps the
// visibility the exact rasteriser produced (one input triangle per pixel, fixed) and shades with
// continuous barycentrics at the reference's sample point, the pixel corner (main.c:1014):
//   lambda_k = cross(v_{k+1} - p, v_{k+2} - p) / cross(v1 - v0, v2 - v0)
// with passthrough screen coordinates (passthrough_vs.c:20-23, w = 1): X = W x, Y = H (1 - y).
// The pixel shader is vertex colour times the bilinear texel of an RGBA32F texture, addressed and
// weighted like the reference's bilinear_f (common_shader_core.h:143-161).
//
// Checkpointing: the forward writes only the per-pixel barycentrics (next to the primitive ids the
// rasteriser wrote); the backward recomputes the interpolation from them.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/malevich.h"
#include "internal.h"

namespace mlv {
void set_last_error(const std::string &msg);
}

using namespace mlv;

namespace {

constexpr int kDiffBlock = 256;

struct Texel4 {
    float v[3];
};

__device__ __forceinline__ int32_t clampi(int32_t x, int32_t hi) { return x < 0 ? 0 : (x > hi ? hi : x); }

__device__ __forceinline__ float3 texel(const float *tex, uint32_t tw, uint32_t th, int32_t i, int32_t j) {
    const float4 t = __ldg(reinterpret_cast<const float4 *>(tex) +
                           (size_t)clampi(j, (int32_t)th - 1) * tw + clampi(i, (int32_t)tw - 1));
    return make_float3(t.x, t.y, t.z);
}

struct PixelEval {
    float l0, l1, l2;
    float3 col, tex;
    float fs, ft;
    int32_t s0, t0;
    uint32_t vi[3];
};

// Interpolation and texture filtering for one covered pixel from its barycentrics.
__device__ __forceinline__ void shade(const mlv_diff_desc &d, float l1, float l2, uint32_t tri, PixelEval &e) {
    e.l1 = l1;
    e.l2 = l2;
    e.l0 = 1.0f - l1 - l2;
    const float l[3] = {e.l0, e.l1, e.l2};
    float u = 0.f, v = 0.f;
    e.col = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t q = __ldg(d.index_buffer + 3 * (size_t)tri + k);
        e.vi[k] = q;
        e.col.x += l[k] * __ldg(d.colors + 3 * (size_t)q);
        e.col.y += l[k] * __ldg(d.colors + 3 * (size_t)q + 1);
        e.col.z += l[k] * __ldg(d.colors + 3 * (size_t)q + 2);
        u += l[k] * __ldg(d.uvs + 2 * (size_t)q);
        v += l[k] * __ldg(d.uvs + 2 * (size_t)q + 1);
    }
    const float sf = (float)d.tex_width * u - 0.5f, tf = (float)d.tex_height * (1.0f - v) - 0.5f;
    e.s0 = (int32_t)floorf(sf);
    e.t0 = (int32_t)floorf(tf);
    e.fs = sf - (float)e.s0;
    e.ft = tf - (float)e.t0;
    const float3 t00 = texel(d.texture, d.tex_width, d.tex_height, e.s0, e.t0);
    const float3 t10 = texel(d.texture, d.tex_width, d.tex_height, e.s0 + 1, e.t0);
    const float3 t01 = texel(d.texture, d.tex_width, d.tex_height, e.s0, e.t0 + 1);
    const float3 t11 = texel(d.texture, d.tex_width, d.tex_height, e.s0 + 1, e.t0 + 1);
    const float a = 1.f - e.fs, b = 1.f - e.ft;
    e.tex.x = b * (a * t00.x + e.fs * t10.x) + e.ft * (a * t01.x + e.fs * t11.x);
    e.tex.y = b * (a * t00.y + e.fs * t10.y) + e.ft * (a * t01.y + e.fs * t11.y);
    e.tex.z = b * (a * t00.z + e.fs * t10.z) + e.ft * (a * t01.z + e.fs * t11.z);
}

__global__ void __launch_bounds__(kDiffBlock) k_diff_forward(mlv_diff_desc d) {
    const size_t npix = (size_t)d.width * d.height;
    const size_t i = (size_t)blockIdx.x * kDiffBlock + threadIdx.x;
    if (i >= npix * d.num_views) return;
    const uint32_t view = (uint32_t)(i / npix);
    const uint32_t p = (uint32_t)(i - (size_t)view * npix);
    const uint32_t tri = d.primitive_ids[i];
    float3 out = make_float3(0.f, 0.f, 0.f);
    float2 bary = make_float2(0.f, 0.f);
    if (tri != 0xFFFFFFFFu && tri < d.n_tris) {
        const float W = (float)d.width, H = (float)d.height;
        const float x = (float)(p % d.width), y = (float)(p / d.width);
        const float *pos = d.positions + (size_t)view * d.n_verts * 2;
        float X[3], Y[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t q = __ldg(d.index_buffer + 3 * (size_t)tri + k);
            X[k] = W * __ldg(pos + 2 * (size_t)q);
            Y[k] = H * (1.0f - __ldg(pos + 2 * (size_t)q + 1));
        }
        const float A = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0]);
        if (A != 0.0f) {
            const float l1 = ((X[2] - x) * (Y[0] - y) - (Y[2] - y) * (X[0] - x)) / A;
            const float l2 = ((X[0] - x) * (Y[1] - y) - (Y[0] - y) * (X[1] - x)) / A;
            PixelEval e;
            shade(d, l1, l2, tri, e);
            out = make_float3(e.col.x * e.tex.x, e.col.y * e.tex.y, e.col.z * e.tex.z);
            bary = make_float2(l1, l2);
        }
    }
    d.image[3 * i] = out.x;
    d.image[3 * i + 1] = out.y;
    d.image[3 * i + 2] = out.z;
    reinterpret_cast<float2 *>(d.barycentrics)[i] = bary;
}

__global__ void __launch_bounds__(kDiffBlock) k_diff_backward(mlv_diff_desc d) {
    const size_t npix = (size_t)d.width * d.height;
    const size_t i = (size_t)blockIdx.x * kDiffBlock + threadIdx.x;
    if (i >= npix * d.num_views) return;
    const uint32_t tri = d.primitive_ids[i];
    if (tri == 0xFFFFFFFFu || tri >= d.n_tris) return;
    const uint32_t view = (uint32_t)(i / npix);
    const uint32_t p = (uint32_t)(i - (size_t)view * npix);
    const float2 bary = reinterpret_cast<const float2 *>(d.barycentrics)[i];
    PixelEval e;
    shade(d, bary.x, bary.y, tri, e);
    const float3 dout = make_float3(d.grad_image[3 * i], d.grad_image[3 * i + 1], d.grad_image[3 * i + 2]);
    const float3 dcol = make_float3(dout.x * e.tex.x, dout.y * e.tex.y, dout.z * e.tex.z);
    const float3 dtex = make_float3(dout.x * e.col.x, dout.y * e.col.y, dout.z * e.col.z);
    const float l[3] = {e.l0, e.l1, e.l2};
    if (d.grad_colors) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float *g = d.grad_colors + 3 * (size_t)e.vi[k];
            atomicAdd(g, l[k] * dcol.x);
            atomicAdd(g + 1, l[k] * dcol.y);
            atomicAdd(g + 2, l[k] * dcol.z);
        }
    }
    const int32_t tw1 = (int32_t)d.tex_width - 1, th1 = (int32_t)d.tex_height - 1;
    if (d.grad_texture) {
        // scatter through the bilinear weights (common_shader_core.h:143-161)
        const float a = 1.f - e.fs, b = 1.f - e.ft;
        const float w[4] = {a * b, e.fs * b, a * e.ft, e.fs * e.ft};
        const int32_t si[4] = {e.s0, e.s0 + 1, e.s0, e.s0 + 1}, ti[4] = {e.t0, e.t0, e.t0 + 1, e.t0 + 1};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float *g = d.grad_texture + ((size_t)clampi(ti[q], th1) * d.tex_width + clampi(si[q], tw1)) * 4;
            atomicAdd(g, w[q] * dtex.x);
            atomicAdd(g + 1, w[q] * dtex.y);
            atomicAdd(g + 2, w[q] * dtex.z);
        }
    }
    if (d.grad_positions) {
        const float3 t00 = texel(d.texture, d.tex_width, d.tex_height, e.s0, e.t0);
        const float3 t10 = texel(d.texture, d.tex_width, d.tex_height, e.s0 + 1, e.t0);
        const float3 t01 = texel(d.texture, d.tex_width, d.tex_height, e.s0, e.t0 + 1);
        const float3 t11 = texel(d.texture, d.tex_width, d.tex_height, e.s0 + 1, e.t0 + 1);
        const float dfs = dtex.x * ((1.f - e.ft) * (t10.x - t00.x) + e.ft * (t11.x - t01.x)) +
                          dtex.y * ((1.f - e.ft) * (t10.y - t00.y) + e.ft * (t11.y - t01.y)) +
                          dtex.z * ((1.f - e.ft) * (t10.z - t00.z) + e.ft * (t11.z - t01.z));
        const float dft = dtex.x * (((1.f - e.fs) * t01.x + e.fs * t11.x) - ((1.f - e.fs) * t00.x + e.fs * t10.x)) +
                          dtex.y * (((1.f - e.fs) * t01.y + e.fs * t11.y) - ((1.f - e.fs) * t00.y + e.fs * t10.y)) +
                          dtex.z * (((1.f - e.fs) * t01.z + e.fs * t11.z) - ((1.f - e.fs) * t00.z + e.fs * t10.z));
        const float du = dfs * (float)d.tex_width, dv = -dft * (float)d.tex_height;
        float G[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const uint32_t q = e.vi[k];
            G[k] = du * __ldg(d.uvs + 2 * (size_t)q) + dv * __ldg(d.uvs + 2 * (size_t)q + 1) +
                   dcol.x * __ldg(d.colors + 3 * (size_t)q) + dcol.y * __ldg(d.colors + 3 * (size_t)q + 1) +
                   dcol.z * __ldg(d.colors + 3 * (size_t)q + 2);
        }
        const float W = (float)d.width, H = (float)d.height;
        const float x = (float)(p % d.width), y = (float)(p / d.width);
        const float *pos = d.positions + (size_t)view * d.n_verts * 2;
        float X[3], Y[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            X[k] = W * __ldg(pos + 2 * (size_t)e.vi[k]);
            Y[k] = H * (1.0f - __ldg(pos + 2 * (size_t)e.vi[k] + 1));
        }
        const float A = (X[1] - X[0]) * (Y[2] - Y[0]) - (X[2] - X[0]) * (Y[1] - Y[0]);
        if (A == 0.0f) return;
        const float rA = 1.0f / A;
        const float S = G[0] * l[0] + G[1] * l[1] + G[2] * l[2];
        // d lambda_k / d v_j from the numerators cross(v_{k+1} - p, v_{k+2} - p), minus S dA/dv_j
        float gX[3], gY[3];
        gX[0] = (G[1] * (-(Y[2] - y)) + G[2] * (Y[1] - y) - S * (-(Y[2] - Y[0]) + (Y[1] - Y[0]))) * rA;
        gY[0] = (G[1] * (X[2] - x) + G[2] * (-(X[1] - x)) - S * ((X[2] - X[0]) - (X[1] - X[0]))) * rA;
        gX[1] = (G[0] * (Y[2] - y) + G[2] * (-(Y[0] - y)) - S * (Y[2] - Y[0])) * rA;
        gY[1] = (G[0] * (-(X[2] - x)) + G[2] * (X[0] - x) - S * (-(X[2] - X[0]))) * rA;
        gX[2] = (G[0] * (-(Y[1] - y)) + G[1] * (Y[0] - y) - S * (-(Y[1] - Y[0]))) * rA;
        gY[2] = (G[0] * (X[1] - x) + G[1] * (-(X[0] - x)) - S * (X[1] - X[0])) * rA;
        float *gp = d.grad_positions + (size_t)view * d.n_verts * 2;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            atomicAdd(gp + 2 * (size_t)e.vi[k], W * gX[k]);
            atomicAdd(gp + 2 * (size_t)e.vi[k] + 1, -H * gY[k]);
        }
    }
}

mlv_status check_desc(const mlv_diff_desc *d, bool backward) {
    if (!d) {
        set_last_error("desc is NULL");
        return MLV_ERROR_INVALID_ARG;
    }
    if (!d->index_buffer || !d->colors || !d->uvs || !d->texture || !d->positions || !d->primitive_ids ||
        !d->barycentrics || !d->tex_width || !d->tex_height || !d->width || !d->height || !d->num_views) {
        set_last_error("index_buffer, colors, uvs, texture, positions, primitive_ids, barycentrics and sizes are required");
        return MLV_ERROR_INVALID_ARG;
    }
    if (!backward && !d->image) {
        set_last_error("the forward needs image");
        return MLV_ERROR_INVALID_ARG;
    }
    if (backward && !d->grad_image) {
        set_last_error("the backward needs grad_image");
        return MLV_ERROR_INVALID_ARG;
    }
    if ((uint64_t)d->width * d->height * d->num_views > 0xFFFFFFFFull * kDiffBlock) {
        set_last_error("too many pixels");
        return MLV_ERROR_INVALID_ARG;
    }
    return MLV_OK;
}

}  // namespace

extern "C" MLV_API mlv_status mlv_diff_forward(const mlv_diff_desc *d, void *stream) {
    mlv_status st = check_desc(d, false);
    if (st != MLV_OK) return st;
    const size_t n = (size_t)d->width * d->height * d->num_views;
    k_diff_forward<<<(unsigned)((n + kDiffBlock - 1) / kDiffBlock), kDiffBlock, 0, (cudaStream_t)stream>>>(*d);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("k_diff_forward: ") + cudaGetErrorString(e));
        return MLV_ERROR_DEVICE;
    }
    return MLV_OK;
}

extern "C" MLV_API mlv_status mlv_diff_backward(const mlv_diff_desc *d, void *stream) {
    mlv_status st = check_desc(d, true);
    if (st != MLV_OK) return st;
    const size_t n = (size_t)d->width * d->height * d->num_views;
    k_diff_backward<<<(unsigned)((n + kDiffBlock - 1) / kDiffBlock), kDiffBlock, 0, (cudaStream_t)stream>>>(*d);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("k_diff_backward: ") + cudaGetErrorString(e));
        return MLV_ERROR_DEVICE;
    }
    return MLV_OK;
}
