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

// a d - b c with Kahan's FMA algorithm (error within 2 ulp; Jeannerod, Louvet and Muller, "Further
// analysis of Kahan's algorithm for the accurate computation of 2x2 determinants", Math. Comp. 2013).
__device__ __forceinline__ float det2(float a, float b, float c, float d) {
    const float w = b * c;
    const float e = fmaf(-b, c, w);
    const float f = fmaf(a, d, -w);
    return f + e;
}

// The differentiable coverage: a pixel the rasteriser gave to a triangle counts when its corner's
// continuous barycentrics are all >= -1/8. The 28.4 snap moves a vertex by at most 1/32 pixel, so
// every covered corner of a triangle whose heights exceed 1/4 pixel passes; the corners it drops
// are those the snap pulled into slivers, where the continuous barycentrics extrapolate without
// bound. A dropped pixel shades to 0 and its checkpoint holds kDropped.
constexpr float kMinBarycentric = -0.125f;
constexpr float kDropped = -1.0f;

// The triangle relative to the pixel corner p = (x, y), in screen space X = W px, Y = H (1 - py):
// a, b, c = v0 - p, v1 - p, v2 - p (one rounding each: fmaf of the exact product and the exact
// integer offset), the edges e1 = v1 - v0, e2 = v2 - v0 from coordinate differences, and twice the
// signed area A = cross(e1, e2).
struct CornerGeom {
    float ax, ay, bx, by, cx, cy;
    float e1x, e1y, e2x, e2y, A;
};

__device__ __forceinline__ void corner_geometry(const float *pos, const uint32_t vi[3], float W, float H, float x,
                                                float y, CornerGeom &g) {
    const float2 p0 = __ldg(reinterpret_cast<const float2 *>(pos) + vi[0]);
    const float2 p1 = __ldg(reinterpret_cast<const float2 *>(pos) + vi[1]);
    const float2 p2 = __ldg(reinterpret_cast<const float2 *>(pos) + vi[2]);
    const float hy = H - y;
    g.ax = fmaf(W, p0.x, -x);
    g.ay = fmaf(-H, p0.y, hy);
    g.bx = fmaf(W, p1.x, -x);
    g.by = fmaf(-H, p1.y, hy);
    g.cx = fmaf(W, p2.x, -x);
    g.cy = fmaf(-H, p2.y, hy);
    g.e1x = W * (p1.x - p0.x);
    g.e1y = H * (p0.y - p1.y);
    g.e2x = W * (p2.x - p0.x);
    g.e2y = H * (p0.y - p2.y);
    g.A = det2(g.e1x, g.e2x, g.e1y, g.e2y);
}

__device__ __forceinline__ void load_triangle(const mlv_diff_desc &d, uint32_t tri, uint32_t vi[3]) {
    vi[0] = __ldg(d.index_buffer + 3 * (size_t)tri);
    vi[1] = __ldg(d.index_buffer + 3 * (size_t)tri + 1);
    vi[2] = __ldg(d.index_buffer + 3 * (size_t)tri + 2);
}

// Interpolation and texture filtering for one covered pixel from its barycentrics. The texel
// coordinates s = tw u - 1/2, t = th (1 - v) - 1/2 are formed as (vertex 0's coordinate, split
// exactly into an integer and a fraction) + (the barycentric deltas), so the bilinear fractions
// keep full single precision whatever the texture size.
__device__ __forceinline__ void shade(const mlv_diff_desc &d, float l1, float l2, const uint32_t vi[3], PixelEval &e) {
    e.l1 = l1;
    e.l2 = l2;
    e.l0 = 1.0f - l1 - l2;
    e.vi[0] = vi[0];
    e.vi[1] = vi[1];
    e.vi[2] = vi[2];
    const float2 uv0 = __ldg(reinterpret_cast<const float2 *>(d.uvs) + vi[0]);
    const float2 uv1 = __ldg(reinterpret_cast<const float2 *>(d.uvs) + vi[1]);
    const float2 uv2 = __ldg(reinterpret_cast<const float2 *>(d.uvs) + vi[2]);
    const float l[3] = {e.l0, l1, l2};
    e.col = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float *c = d.colors + 3 * (size_t)vi[k];
        e.col.x += l[k] * __ldg(c);
        e.col.y += l[k] * __ldg(c + 1);
        e.col.z += l[k] * __ldg(c + 2);
    }
    const float tw = (float)d.tex_width, th = (float)d.tex_height;
    // s at vertex 0: tw u0 = ps + pse exactly; ps - 1/2 is exact below 2^22
    const float ps = tw * uv0.x, pse = fmaf(tw, uv0.x, -ps);
    const float bs = ps - 0.5f, fbs = floorf(bs);
    // t at vertex 0: (th - 1/2) - th v0, with th v0 = q + qe exactly and the difference by two-sum
    const float q = th * uv0.y, qe = fmaf(th, uv0.y, -q);
    const float a = th - 0.5f, r = a - q, rb = r - a;
    const float re = (a - (r - rb)) + (-q - rb);
    const float fbt = floorf(r);
    const float rs = ((bs - fbs) + pse) + (l1 * (tw * (uv1.x - uv0.x)) + l2 * (tw * (uv2.x - uv0.x)));
    const float rt = ((r - fbt) + (re - qe)) - (l1 * (th * (uv1.y - uv0.y)) + l2 * (th * (uv2.y - uv0.y)));
    const float frs = floorf(rs), frt = floorf(rt);
    e.s0 = (int32_t)fbs + (int32_t)frs;
    e.t0 = (int32_t)fbt + (int32_t)frt;
    e.fs = rs - frs;
    e.ft = rt - frt;
    const float3 t00 = texel(d.texture, d.tex_width, d.tex_height, e.s0, e.t0);
    const float3 t10 = texel(d.texture, d.tex_width, d.tex_height, e.s0 + 1, e.t0);
    const float3 t01 = texel(d.texture, d.tex_width, d.tex_height, e.s0, e.t0 + 1);
    const float3 t11 = texel(d.texture, d.tex_width, d.tex_height, e.s0 + 1, e.t0 + 1);
    const float oa = 1.f - e.fs, ob = 1.f - e.ft;
    e.tex.x = ob * (oa * t00.x + e.fs * t10.x) + e.ft * (oa * t01.x + e.fs * t11.x);
    e.tex.y = ob * (oa * t00.y + e.fs * t10.y) + e.ft * (oa * t01.y + e.fs * t11.y);
    e.tex.z = ob * (oa * t00.z + e.fs * t10.z) + e.ft * (oa * t01.z + e.fs * t11.z);
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
        uint32_t vi[3];
        load_triangle(d, tri, vi);
        CornerGeom g;
        corner_geometry(d.positions + (size_t)view * d.n_verts * 2, vi, (float)d.width, (float)d.height,
                        (float)(p % d.width), (float)(p / d.width), g);
        bary = make_float2(kDropped, kDropped);
        if (g.A != 0.0f) {
            // lambda_k = cross(v_{k+1} - p, v_{k+2} - p) / A
            const float l1 = det2(g.cx, g.cy, g.ax, g.ay) / g.A;
            const float l2 = det2(g.ax, g.ay, g.bx, g.by) / g.A;
            const float l0 = 1.0f - l1 - l2;
            if (l0 >= kMinBarycentric && l1 >= kMinBarycentric && l2 >= kMinBarycentric) {
                PixelEval e;
                shade(d, l1, l2, vi, e);
                out = make_float3(e.col.x * e.tex.x, e.col.y * e.tex.y, e.col.z * e.tex.z);
                bary = make_float2(l1, l2);
            }
        }
    }
    d.image[3 * i] = out.x;
    d.image[3 * i + 1] = out.y;
    d.image[3 * i + 2] = out.z;
    reinterpret_cast<float2 *>(d.barycentrics)[i] = bary;
}

// Sums v over the lanes of the caller's run (lane .. end, end the run's last lane) into its first
// lane: a segmented suffix sum by shuffles; every lane of the warp calls it.
template <int N>
__device__ __forceinline__ void run_sum(float (&v)[N], uint32_t lane, int end) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            const float o = __shfl_down_sync(0xFFFFFFFFu, v[k], off);
            if ((int)lane + off <= end) v[k] += o;
        }
    }
}

// One thread per pixel. Texel gradients go out as float4 atomics; the vertex-colour and position
// gradients of a run of neighbouring pixels on the same triangle (the common case along a row)
// are summed in registers first and leave as one set of atomics per run.
__global__ void __launch_bounds__(kDiffBlock, 4) k_diff_backward(mlv_diff_desc d) {
    const size_t npix = (size_t)d.width * d.height;
    const size_t i = (size_t)blockIdx.x * kDiffBlock + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t tri = 0xFFFFFFFFu, view = 0, p = 0;
    float2 bary = make_float2(kDropped, kDropped);
    if (i < npix * d.num_views) {
        view = (uint32_t)(i / npix);
        p = (uint32_t)(i - (size_t)view * npix);
        tri = d.primitive_ids[i];
        if (tri < d.n_tris) bary = reinterpret_cast<const float2 *>(d.barycentrics)[i];
        if (tri >= d.n_tris || bary.x < kMinBarycentric) tri = 0xFFFFFFFFu;   // background or dropped
    }
    const bool live = tri != 0xFFFFFFFFu;
    float gc[9], gp[6];
#pragma unroll
    for (int k = 0; k < 9; ++k) gc[k] = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) gp[k] = 0.f;
    PixelEval e;
    if (live) {
        uint32_t vi[3];
        load_triangle(d, tri, vi);
        shade(d, bary.x, bary.y, vi, e);
        const float3 dout = make_float3(d.grad_image[3 * i], d.grad_image[3 * i + 1], d.grad_image[3 * i + 2]);
        const float3 dcol = make_float3(dout.x * e.tex.x, dout.y * e.tex.y, dout.z * e.tex.z);
        const float3 dtex = make_float3(dout.x * e.col.x, dout.y * e.col.y, dout.z * e.col.z);
        const float l[3] = {e.l0, e.l1, e.l2};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            gc[3 * k] = l[k] * dcol.x;
            gc[3 * k + 1] = l[k] * dcol.y;
            gc[3 * k + 2] = l[k] * dcol.z;
        }
        if (d.grad_texture) {
            // scatter through the bilinear weights (common_shader_core.h:143-161)
            const int32_t tw1 = (int32_t)d.tex_width - 1, th1 = (int32_t)d.tex_height - 1;
            const float a = 1.f - e.fs, b = 1.f - e.ft;
            const float w[4] = {a * b, e.fs * b, a * e.ft, e.fs * e.ft};
            const int32_t si[4] = {e.s0, e.s0 + 1, e.s0, e.s0 + 1}, ti[4] = {e.t0, e.t0, e.t0 + 1, e.t0 + 1};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float4 *g = reinterpret_cast<float4 *>(d.grad_texture) + (size_t)clampi(ti[q], th1) * d.tex_width +
                            clampi(si[q], tw1);
                atomicAdd(g, make_float4(w[q] * dtex.x, w[q] * dtex.y, w[q] * dtex.z, 0.f));
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
            const float dft =
                dtex.x * (((1.f - e.fs) * t01.x + e.fs * t11.x) - ((1.f - e.fs) * t00.x + e.fs * t10.x)) +
                dtex.y * (((1.f - e.fs) * t01.y + e.fs * t11.y) - ((1.f - e.fs) * t00.y + e.fs * t10.y)) +
                dtex.z * (((1.f - e.fs) * t01.z + e.fs * t11.z) - ((1.f - e.fs) * t00.z + e.fs * t10.z));
            const float du = dfs * (float)d.tex_width, dv = -dft * (float)d.tex_height;
            // G_k = dL/dlambda_k, taken relative to G_0 (the barycentric derivatives sum to zero)
            const float2 uv0 = __ldg(reinterpret_cast<const float2 *>(d.uvs) + e.vi[0]);
            const float *c0 = d.colors + 3 * (size_t)e.vi[0];
            float G[3];
            G[0] = 0.f;
#pragma unroll
            for (int k = 1; k < 3; ++k) {
                const float2 uvk = __ldg(reinterpret_cast<const float2 *>(d.uvs) + e.vi[k]);
                const float *ck = d.colors + 3 * (size_t)e.vi[k];
                G[k] = du * (uvk.x - uv0.x) + dv * (uvk.y - uv0.y) + dcol.x * (__ldg(ck) - __ldg(c0)) +
                       dcol.y * (__ldg(ck + 1) - __ldg(c0 + 1)) + dcol.z * (__ldg(ck + 2) - __ldg(c0 + 2));
            }
            const float W = (float)d.width, H = (float)d.height;
            CornerGeom g;
            corner_geometry(d.positions + (size_t)view * d.n_verts * 2, e.vi, W, H, (float)(p % d.width),
                            (float)(p / d.width), g);
            const float rA = 1.0f / g.A;
            const float S = G[1] * e.l1 + G[2] * e.l2;
            // sum_k G_k d lambda_k / d v_j = (sum_k G_k d n_k / d v_j - S dA / d v_j) / A, n_k the numerators
            const float gX0 = (G[2] * g.by - G[1] * g.cy - S * (g.e1y - g.e2y)) * rA;
            const float gY0 = (G[1] * g.cx - G[2] * g.bx - S * (g.e2x - g.e1x)) * rA;
            const float gX1 = (-G[2] * g.ay - S * g.e2y) * rA;
            const float gY1 = (G[2] * g.ax + S * g.e2x) * rA;
            const float gX2 = (G[1] * g.ay + S * g.e1y) * rA;
            const float gY2 = (-G[1] * g.ax - S * g.e1x) * rA;
            gp[0] = W * gX0; gp[1] = -H * gY0;
            gp[2] = W * gX1; gp[3] = -H * gY1;
            gp[4] = W * gX2; gp[5] = -H * gY2;
        }
    }
    // runs of neighbouring pixels with the same (view, triangle)
    const uint32_t ptri = __shfl_up_sync(0xFFFFFFFFu, tri, 1), pview = __shfl_up_sync(0xFFFFFFFFu, view, 1);
    const bool head = lane == 0 || ptri != tri || pview != view;
    const uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
    const uint32_t later = heads & ~((2u << lane) - 1u);
    const int end = later ? __ffs(later) - 2 : 31;
    if (d.grad_colors) run_sum(gc, lane, end);
    if (d.grad_positions) run_sum(gp, lane, end);
    if (!(head && live)) return;
    if (d.grad_colors) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float *g = d.grad_colors + 3 * (size_t)e.vi[k];
            atomicAdd(g, gc[3 * k]);
            atomicAdd(g + 1, gc[3 * k + 1]);
            atomicAdd(g + 2, gc[3 * k + 2]);
        }
    }
    if (d.grad_positions) {
        float2 *gpos = reinterpret_cast<float2 *>(d.grad_positions + (size_t)view * d.n_verts * 2);
#pragma unroll
        for (int k = 0; k < 3; ++k) atomicAdd(gpos + e.vi[k], make_float2(gp[2 * k], gp[2 * k + 1]));
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
    if (((uintptr_t)d->positions | (uintptr_t)d->uvs | (uintptr_t)d->barycentrics | (uintptr_t)d->grad_positions) & 7u ||
        ((uintptr_t)d->texture | (uintptr_t)d->grad_texture) & 15u) {
        set_last_error("positions, uvs, barycentrics, grad_positions need 8-byte alignment, texture, grad_texture 16-byte");
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
