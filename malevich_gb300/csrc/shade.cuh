// Device-side shader math: vertex shaders, pixel shaders, texture sampling, colour packing.
// Compiled with --fmad=false so that every a*b+c below is the reference's two rounded float
// operations (the reference's AVX code issues separate mul and add instructions); the two places
// where the reference itself fuses (_mm256_fmadd_ps in passthrough_vs.c:20-21 and
// fullscreen_vs.c:28-29) call fmaf explicitly.
#pragma once
#include <cuda_fp16.h>
#include <cstdint>

#include "internal.h"

namespace mlv {

__device__ __forceinline__ float fmax_ref(float x, float y) { return (x > y) ? x : y; }  // MAX, math.h:29-30
__device__ __forceinline__ float fmin_ref(float x, float y) { return (x < y) ? x : y; }  // MIN, math.h:26-27

// v4f256_dot (math.h:142-146): (x*x' + y*y') + (z*z' + w*w')
__device__ __forceinline__ float dot4_pairwise(const float *a, float b0, float b1, float b2, float b3) {
    float xy = a[0] * b0 + a[1] * b1;
    float zw = a[2] * b2 + a[3] * b3;
    return xy + zw;
}

// v4f32_dot (math.h:137-140): left to right
__device__ __forceinline__ float dot4_lr(const float *a, float b0, float b1, float b2, float b3) {
    return a[0] * b0 + a[1] * b1 + a[2] * b2 + a[3] * b3;
}

// v3f256_dot (math.h:153-157)
__device__ __forceinline__ float dot3(float a0, float a1, float a2, float b0, float b1, float b2) {
    float r = a0 * b0 + a1 * b1;
    return r + a2 * b2;
}

// v3f256_normalize (math.h:277-280) with a correctly rounded reciprocal square root (the
// reference's _mm256_rsqrt_ps is an approximate, CPU-model specific instruction).
__device__ __forceinline__ void normalize3(float &x, float &y, float &z) {
    float r = 1.0f / sqrtf(dot3(x, y, z, x, y, z));
    x = x * r; y = y * r; z = z * r;
}

// _mm256_cvtps_epi32 under the default MXCSR: round to nearest even; NaN and out-of-range
// values give 0x80000000.
__device__ __forceinline__ int32_t cvt_rn(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return (int32_t)0x80000000u;
    return __float2int_rn(x);
}

// main.c:843-848: floor(x_ss * 16 + 0.5) with the add in double. For |v| < 2^23 the float sum
// v + 0.5 is exact (the unit in the last place of v is at most 0.5), so it is floored in float.
__device__ __forceinline__ int32_t snap28_4(float x_ss) {
    float v = x_ss * 16.0f;
    if (!(fabsf(v) < 8388608.0f)) {
        if (!(v >= -2147483648.0f && v < 2147483648.0f)) return (int32_t)0x80000000u;
        return (int32_t)v;
    }
    return __float2int_rd(v + 0.5f);
}

// encode_color_as_u32 (math.h:322-324): R in the low byte, truncating conversions
__device__ __host__ __forceinline__ uint32_t trunc_u32(float x) {
    if (!(x > -9.2e18f && x < 9.2e18f)) return 0u;
    return (uint32_t)(long long)x;
}

// output merger packing (main.c:1176-1178): R<<16 + G<<8 + B, rounded, not clamped
__device__ __forceinline__ uint32_t pack_color(float r, float g, float b) {
    return ((uint32_t)cvt_rn(r * 255.0f) << 16) + ((uint32_t)cvt_rn(g * 255.0f) << 8) + (uint32_t)cvt_rn(b * 255.0f);
}

// ------------------------------------------------------------------ texture sampling

// clamp-to-edge addressing, common_shader_core.h:30-36,42-46
__device__ __forceinline__ uint32_t texel_index(const TexDesc &t, int32_t s, int32_t u) {
    int32_t w1 = (int32_t)t.width - 1, h1 = (int32_t)t.height - 1;
    s = s < w1 ? s : w1; s = s > 0 ? s : 0;
    u = u < h1 ? u : h1; u = u > 0 ? u : 0;
    return (uint32_t)u * t.width + (uint32_t)s;
}

// decode_u32_as_color_x8 (math.h:336-344): byte * (float)(1/255)
__device__ __forceinline__ float4 fetch_rgba8(const TexDesc &t, int32_t s, int32_t u) {
    uint32_t c = __ldg((const uint32_t *)t.data + texel_index(t, s, u));
    const float k = (float)(1.0 / 255.0);
    return make_float4((float)(int32_t)(c & 0xFFu) * k, (float)(int32_t)((c >> 8) & 0xFFu) * k,
                       (float)(int32_t)((c >> 16) & 0xFFu) * k, (float)(int32_t)(c >> 24) * k);
}

__device__ __forceinline__ float4 fetch_float(const TexDesc &t, int32_t s, int32_t u) {
    uint32_t i = texel_index(t, s, u);
    if (t.format == 3) return __ldg((const float4 *)t.data + i);
    uint2 h = __ldg((const uint2 *)t.data + i);   // RGBA16F widened exactly
    __half2 lo = *reinterpret_cast<__half2 *>(&h.x), hi = *reinterpret_cast<__half2 *>(&h.y);
    float2 a = __half22float2(lo), b = __half22float2(hi);
    return make_float4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ float4 fetch(const TexDesc &t, int32_t s, int32_t u) {
    return t.format == 1 ? fetch_rgba8(t, s, u) : fetch_float(t, s, u);
}

// v4f256_lerp (math.h:381-384)
__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t) {
    float omt = 1.0f - t;
    return make_float4(a.x * omt + b.x * t, a.y * omt + b.y * t, a.z * omt + b.z * t, a.w * omt + b.w * t);
}

// bilinear_u_x8 / bilinear_f_x8 (common_shader_core.h:103-121,143-161)
__device__ __forceinline__ float4 bilinear(const TexDesc &t, float u, float v) {
    float s_f = (float)t.width * u + (-0.5f);
    float t_f = (float)t.height * (1.0f - v) + (-0.5f);
    int32_t s = cvt_rn(floorf(s_f));
    int32_t tt = cvt_rn(floorf(t_f));
    float fs = s_f - (float)s;
    float ft = t_f - (float)tt;
    float4 t00 = fetch(t, s, tt), t10 = fetch(t, s + 1, tt);
    float4 t01 = fetch(t, s, tt + 1), t11 = fetch(t, s + 1, tt + 1);
    float4 a = lerp4(t00, t10, fs);
    float4 b = lerp4(t01, t11, fs);
    return lerp4(a, b, ft);
}

// sample_2D_latlon_x8 (common_shader_core.h:226-244). The normalised axes are exact: with a
// correctly rounded rsqrt, normalize((0,0,1)) == (0,0,1).
__device__ __forceinline__ float4 sample_latlon(const TexDesc &t, float dx, float dy, float dz) {
    float cos_theta = dot3(0.0f, 0.0f, 1.0f, dx, dy, dz);
    float cx = dx, cy = dy, cz = 0.0f;
    normalize3(cx, cy, cz);
    float cos_x = dot3(1.0f, 0.0f, 0.0f, cx, cy, cz);
    float cos_y = dot3(0.0f, 1.0f, 0.0f, cx, cy, cz);
    float ax = acosf(cos_x) * (float)(1.0 / 6.283185307f);
    float uv_x = (cos_y >= 0.0f) ? ax : (1.0f - ax);
    float uv_y = acosf(cos_theta) * (float)(1.0 / 3.141592654f);
    bool pos = cos_theta > (float)0.999;
    bool neg = cos_theta < (float)-0.999;
    if (pos || neg) uv_x = 0.5f;
    if (pos) uv_y = 0.0f;
    if (neg) uv_y = 1.0f;
    uv_y = 1.0f - uv_y;
    return bilinear(t, uv_x, uv_y);
}

// The colour-only transcendentals below use CUDA's fast intrinsics (__expf, __powf: a few ulp,
// i.e. about 1e-3 of an 8-bit step after packing), as the reference uses SVML's approximations
// (math.h:21-23); they feed nothing but UNORM8 colour, which is compared within +-1 LSB.

// vertex_lighting_vs.c:34-35 and env_lighting_ps.c:20-21: (1 - e^(-c))^(1/2.2)
__device__ __forceinline__ float tonemap(float c) {
    return __powf(1.0f - __expf(c * -1.0f), (float)(1.0 / 2.2));
}

// f256_srgb_from_linear_approx (math.h:419-422)
__device__ __forceinline__ float srgb_approx(float c) {
    float v = (float)1.055 * __powf(c, (float)0.416666667) + (float)-0.055;
    return (v > 0.0f) ? v : 0.0f;
}

// ------------------------------------------------------------------ vertex shaders

// Runs vertex shader `vs` on the 8 input floats of one vertex. Outputs the registers the rest of
// the pipeline reads: o0..o3 = SV_POSITION, o4..o6 = reg1.xyz, o7 = reg1.w (U), o8 = reg2.x (V).
// basic_vs.c:22-33, vertex_lighting_vs.c:22-39, passthrough_vs.c:16-25, fullscreen_vs.c:22-39.
__device__ __forceinline__ void run_vs(int vs, const float *in, const float *cb, const TexDesc &tex, float *o) {
    o[7] = 0.0f; o[8] = 0.0f;
    if (vs == 1 || vs == 2) {
        for (int k = 0; k < 4; ++k) o[k] = dot4_pairwise(cb + 4 * k, in[0], in[1], in[2], 1.0f);
        float nx = in[3], ny = in[4], nz = in[5];
        normalize3(nx, ny, nz);
        if (vs == 1) {
            o[4] = nx; o[5] = ny; o[6] = nz;
        } else {
            float4 c = sample_latlon(tex, nx, ny, nz);
            o[4] = tonemap(c.x); o[5] = tonemap(c.y); o[6] = tonemap(c.z);
        }
        o[7] = in[6]; o[8] = in[7];
    } else if (vs == 3) {
        o[0] = fmaf(in[0], 2.0f, -1.0f); o[1] = fmaf(in[1], 2.0f, -1.0f);
        o[2] = in[2]; o[3] = in[3];
        o[4] = in[4]; o[5] = in[5]; o[6] = in[6];
    } else if (vs == 4) {
        float p0 = fmaf(in[0], 2.0f, -1.0f), p1 = fmaf(in[1], 2.0f, -1.0f), p2 = in[2], p3 = in[3];
        float dv[3];
        for (int k = 0; k < 3; ++k) dv[k] = dot4_pairwise(cb + 16 + 4 * k, p0, p1, p2, p3);
        for (int k = 0; k < 3; ++k) o[4 + k] = dot4_pairwise(cb + 32 + 4 * k, dv[0], dv[1], dv[2], 0.0f);
        o[0] = p0; o[1] = p1; o[2] = p2; o[3] = p3;
    } else {  // 5: passthrough with UV (new)
        o[0] = fmaf(in[0], 2.0f, -1.0f); o[1] = fmaf(in[1], 2.0f, -1.0f);
        o[2] = in[2]; o[3] = 1.0f;
        o[4] = in[3]; o[5] = in[4]; o[6] = in[5];
        o[7] = in[6]; o[8] = in[7];
    }
}

// ------------------------------------------------------------------ pixel shaders

// basic_ps.c:16-27, passthrough_ps.c:13-20, env_lighting_ps.c:13-24, COLOR_TIMES_TEXEL (new).
// a = reg1.xyz, u = reg1.w, v = reg2.x of the interpolated fragment.
__device__ __forceinline__ float3 run_ps(int ps, float a0, float a1, float a2, float u, float v, const TexDesc &tex) {
    if (ps == 1) {
        float4 c = bilinear(tex, u, v);
        return make_float3(srgb_approx(c.x), srgb_approx(c.y), srgb_approx(c.z));
    } else if (ps == 2) {
        return make_float3(a0, a1, a2);
    } else if (ps == 3) {
        float nx = a0, ny = a1, nz = a2;
        normalize3(nx, ny, nz);
        float4 c = sample_latlon(tex, nx, ny, nz);
        return make_float3(tonemap(c.x), tonemap(c.y), tonemap(c.z));
    } else {
        float4 c = bilinear(tex, u, v);
        return make_float3(a0 * c.x, a1 * c.y, a2 * c.z);
    }
}

}  // namespace mlv
