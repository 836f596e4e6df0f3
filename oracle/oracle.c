/* Malevich draw-path oracle (TEST INFRASTRUCTURE ONLY; see oracle.h for the contract).
 * Every function names the reference lines it restates. Build with -ffp-contract=off -fwrapv:
 * the reference's arithmetic is unfused float ops and wrapping int32. */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define TILE 8
#define SUBPIX 4
#define MAX_CLIP_VERTICES 16

typedef struct vtx { float r[3][4]; } vtx;   /* 3 output registers of a vertex (main.c:117-119) */

typedef struct tri_rec {                       /* Triangle + Setup (main.c:121-139) */
    uint32_t input;                            /* input triangle index within the draw */
    int32_t e[3][3];                           /* edge functions a, b, c */
    float rw[3], inv_area, zbound;
    int32_t minx, miny, maxx, maxy;
    float attrs[3][3][4];
} tri_rec;

void orc_set_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n > 0 ? n : 1);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------------------------------------------------------- math helpers (math.h) */

static inline float mx(float x, float y) { return (x > y) ? x : y; }   /* MAX, math.h:29-30 */
static inline float mn(float x, float y) { return (x < y) ? x : y; }   /* MIN, math.h:26-27 */

/* v4f32_dot, math.h:137-140: left to right */
static inline float dot4_lr(const float a[4], const float b[4]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
}

/* v4f256_dot, math.h:142-146: pairwise */
static inline float dot4_pw(const float a[4], const float b[4]) {
    float xy = a[0] * b[0] + a[1] * b[1];
    float zw = a[2] * b[2] + a[3] * b[3];
    return xy + zw;
}

/* v3f256_dot, math.h:153-157 */
static inline float dot3(const float a[3], const float b[3]) {
    float r = a[0] * b[0] + a[1] * b[1];
    return r + a[2] * b[2];
}

/* _mm256_rsqrt_ps stand-in (math.h:278): correctly rounded, see oracle.h */
static inline float rsqrt_(float x) { return 1.0f / sqrtf(x); }

/* v3f256_normalize, math.h:277-280 */
static inline void normalize3(const float v[3], float out[3]) {
    float r = rsqrt_(dot3(v, v));
    out[0] = v[0] * r; out[1] = v[1] * r; out[2] = v[2] * r;
}

/* m4x4f32_mul_v4f256, math.h:174-177 (row-major matrix, pairwise dots) */
static inline void mat_vec_pw(const float *m, const float v[4], float out[4]) {
    for (int k = 0; k < 4; ++k) out[k] = dot4_pw(m + 4 * k, v);
}

/* _mm256_cvtps_epi32 under the default MXCSR: round to nearest even; NaN and values outside the
 * int32 range give the "integer indefinite" 0x80000000. */
int32_t orc_cvt_rn(float x) {
    if (!(x >= -2147483648.0f && x < 2147483648.0f)) return (int32_t)0x80000000u;
    return (int32_t)rintf(x);
}

/* encode_color_as_u32, math.h:322-324: R in the low byte, truncating conversions */
static inline uint32_t trunc_u32(float x) {
    if (!(x > -9.2e18f && x < 9.2e18f)) return 0u;
    return (uint32_t)(int64_t)x;
}

uint32_t orc_encode_clear_color(const float c[4]) {
    return (trunc_u32(c[3] * 255.f) << 24) + (trunc_u32(c[2] * 255.f) << 16) +
           (trunc_u32(c[1] * 255.f) << 8) + trunc_u32(c[0] * 255.f);
}

/* main.c:843-848: x = floor(x_ss * 16 + 0.5), the product in float, the add and floor in double */
int32_t orc_snap(float x_ss) {
    double v = floor((double)(x_ss * (float)(1 << SUBPIX)) + 0.5);
    if (!(v >= -2147483648.0 && v < 2147483648.0)) return (int32_t)0x80000000u;
    return (int32_t)v;
}

static inline float half_to_float(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu, bits;
    if (e == 0) {
        if (m == 0) {
            bits = sign;
        } else {               /* subnormal: renormalise */
            e = 113;
            while (!(m & 0x400u)) { m <<= 1; --e; }
            bits = sign | (e << 23) | ((m & 0x3FFu) << 13);
        }
    } else if (e == 31) {
        bits = sign | 0x7F800000u | (m << 13);
    } else {
        bits = sign | ((e + 112) << 23) | (m << 13);
    }
    float f;
    memcpy(&f, &bits, 4);
    return f;
}

/* ---------------------------------------------------------------- texture sampling */

/* get_texel_f_x8 / get_texel_u_x8 addressing, common_shader_core.h:30-53: clamp to edge */
static inline uint32_t texel_index(const orc_texture *t, int32_t s, int32_t u) {
    int32_t w1 = (int32_t)t->width - 1, h1 = (int32_t)t->height - 1;
    s = s < w1 ? s : w1; s = s > 0 ? s : 0;
    u = u < h1 ? u : h1; u = u > 0 ? u : 0;
    return (uint32_t)u * t->width + (uint32_t)s;
}

static inline void fetch_f(const orc_texture *t, int32_t s, int32_t u, float out[4]) {
    uint32_t i = texel_index(t, s, u);
    if (t->format == ORC_FMT_RGBA32F) {
        const float *p = (const float *)t->data + 4 * (size_t)i;
        out[0] = p[0]; out[1] = p[1]; out[2] = p[2]; out[3] = p[3];
    } else {
        const uint16_t *p = (const uint16_t *)t->data + 4 * (size_t)i;
        out[0] = half_to_float(p[0]); out[1] = half_to_float(p[1]);
        out[2] = half_to_float(p[2]); out[3] = half_to_float(p[3]);
    }
}

/* decode_u32_as_color_x8, math.h:336-344: R in the low byte, times (float)(1/255) */
static inline void fetch_u(const orc_texture *t, int32_t s, int32_t u, float out[4]) {
    uint32_t c = ((const uint32_t *)t->data)[texel_index(t, s, u)];
    const float k = (float)(1.0 / 255.0);
    out[0] = (float)(int32_t)(c & 0xFFu) * k;
    out[1] = (float)(int32_t)((c & 0xFF00u) >> 8) * k;
    out[2] = (float)(int32_t)((c & 0xFF0000u) >> 16) * k;
    out[3] = (float)(int32_t)((c & 0xFF000000u) >> 24) * k;
}

/* v4f256_lerp, math.h:381-384 */
static inline void lerp4(const float a[4], const float b[4], float t, float out[4]) {
    float omt = 1.0f - t;
    for (int k = 0; k < 4; ++k) out[k] = a[k] * omt + b[k] * t;
}

/* bilinear_u_x8 / bilinear_f_x8, common_shader_core.h:103-121,143-161 */
static void bilinear(const orc_texture *t, float u, float v, float out[4]) {
    float s_f = (float)t->width * u + (-0.5f);
    float t_f = (float)t->height * (1.0f - v) + (-0.5f);
    int32_t s = orc_cvt_rn(floorf(s_f));
    int32_t tt = orc_cvt_rn(floorf(t_f));
    float fs = s_f - (float)s;
    float ft = t_f - (float)tt;
    float t00[4], t10[4], t01[4], t11[4], a[4], b[4];
    if (t->format == ORC_FMT_RGBA8) {
        fetch_u(t, s, tt, t00); fetch_u(t, s + 1, tt, t10);
        fetch_u(t, s, tt + 1, t01); fetch_u(t, s + 1, tt + 1, t11);
    } else {
        fetch_f(t, s, tt, t00); fetch_f(t, s + 1, tt, t10);
        fetch_f(t, s, tt + 1, t01); fetch_f(t, s + 1, tt + 1, t11);
    }
    lerp4(t00, t10, fs, a);
    lerp4(t01, t11, fs, b);
    lerp4(a, b, ft, out);
}

/* sample_2D_latlon_x8, common_shader_core.h:226-244 */
static void sample_latlon(const orc_texture *t, const float dir[3], float out[4]) {
    static const float zax[3] = {0.f, 0.f, 1.f}, xax[3] = {1.f, 0.f, 0.f}, yax[3] = {0.f, 1.f, 0.f};
    float nz[3], nx[3], ny[3], cxy[3];
    normalize3(zax, nz);
    float cos_theta = dot3(nz, dir);
    float dxy[3] = {dir[0], dir[1], 0.f};
    normalize3(dxy, cxy);
    normalize3(xax, nx);
    normalize3(yax, ny);
    float cos_x = dot3(nx, cxy);
    float cos_y = dot3(ny, cxy);
    float ax = acosf(cos_x) * (float)(1.0 / 6.283185307f);
    float uv_x = (cos_y >= 0.0f) ? ax : (1.0f - ax);
    float uv_y = acosf(cos_theta) * (float)(1.0 / 3.141592654f);
    int pos = cos_theta > (float)0.999;
    int neg = cos_theta < (float)-0.999;
    if (pos || neg) uv_x = 0.5f;
    if (pos) uv_y = 0.0f;
    if (neg) uv_y = 1.0f;
    uv_y = 1.0f - uv_y;
    bilinear(t, uv_x, uv_y, out);
}

/* the tonemap shared by vertex_lighting_vs.c:34-35 and env_lighting_ps.c:20-21 */
static inline float tonemap(float c) {
    return powf(1.0f - expf(c * -1.0f), (float)(1.0 / 2.2));
}

/* f256_srgb_from_linear_approx, math.h:419-422 */
static inline float srgb_approx(float c) {
    float v = (float)1.055 * powf(c, (float)0.416666667) + (float)-0.055;
    return (v > 0.0f) ? v : 0.0f;
}

/* ---------------------------------------------------------------- shaders */

/* Vertex shaders: 8 input floats, 12 output floats (r0 = SV_POSITION, r1 = xyz + U, r2 = V + pad).
 * basic_vs.c:22-33, vertex_lighting_vs.c:22-39, passthrough_vs.c:16-25, fullscreen_vs.c:22-39.
 * Outputs the reference leaves uninitialised are zero here. */
void orc_run_vs(int32_t vs, const float in[8], const float *cb, const orc_texture *tex, float o[12]) {
    memset(o, 0, 12 * sizeof(float));
    switch (vs) {
        case ORC_VS_BASIC:
        case ORC_VS_VERTEX_LIGHTING: {
            float p[4] = {in[0], in[1], in[2], 1.0f};
            mat_vec_pw(cb, p, o);
            float n[3];
            normalize3(in + 3, n);
            if (vs == ORC_VS_BASIC) {
                o[4] = n[0]; o[5] = n[1]; o[6] = n[2];
            } else {
                float c[4];
                sample_latlon(tex, n, c);
                o[4] = tonemap(c[0]); o[5] = tonemap(c[1]); o[6] = tonemap(c[2]);
            }
            o[7] = in[6]; o[8] = in[7];
            break;
        }
        case ORC_VS_PASSTHROUGH:
            o[0] = fmaf(in[0], 2.0f, -1.0f); o[1] = fmaf(in[1], 2.0f, -1.0f);
            o[2] = in[2]; o[3] = in[3];
            o[4] = in[4]; o[5] = in[5]; o[6] = in[6];
            break;
        case ORC_VS_FULLSCREEN: {
            float p[4] = {fmaf(in[0], 2.0f, -1.0f), fmaf(in[1], 2.0f, -1.0f), in[2], in[3]};
            float dv[4], dw[4];
            mat_vec_pw(cb + 16, p, dv);
            float d0[4] = {dv[0], dv[1], dv[2], 0.0f};
            mat_vec_pw(cb + 32, d0, dw);
            o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; o[3] = p[3];
            o[4] = dw[0]; o[5] = dw[1]; o[6] = dw[2];
            break;
        }
        case ORC_VS_PASSTHROUGH_UV:    /* new: {x, y, z, r, g, b, u, v}, w = 1 */
            o[0] = fmaf(in[0], 2.0f, -1.0f); o[1] = fmaf(in[1], 2.0f, -1.0f);
            o[2] = in[2]; o[3] = 1.0f;
            o[4] = in[3]; o[5] = in[4]; o[6] = in[5];
            o[7] = in[6]; o[8] = in[7];
            break;
        default:
            break;
    }
}

/* Pixel shaders on the 12 interpolated floats (Ps_Input: pos4, xyz, U, V).
 * basic_ps.c:16-27, passthrough_ps.c:13-20, env_lighting_ps.c:13-24; COLOR_TIMES_TEXEL is new. */
void orc_run_ps(int32_t ps, const float a[12], const orc_texture *tex, float out[3]) {
    switch (ps) {
        case ORC_PS_BASIC: {
            float c[4];
            bilinear(tex, a[7], a[8], c);
            out[0] = srgb_approx(c[0]); out[1] = srgb_approx(c[1]); out[2] = srgb_approx(c[2]);
            break;
        }
        case ORC_PS_PASSTHROUGH:
            out[0] = a[4]; out[1] = a[5]; out[2] = a[6];
            break;
        case ORC_PS_ENV_LIGHTING: {
            float n[3], c[4];
            normalize3(a + 4, n);
            sample_latlon(tex, n, c);
            out[0] = tonemap(c[0]); out[1] = tonemap(c[1]); out[2] = tonemap(c[2]);
            break;
        }
        case ORC_PS_COLOR_TIMES_TEXEL: {
            float c[4];
            bilinear(tex, a[7], a[8], c);
            out[0] = a[4] * c[0]; out[1] = a[5] * c[1]; out[2] = a[6] * c[2];
            break;
        }
        default:
            out[0] = out[1] = out[2] = 0.f;
    }
}

/* Output merger packing, main.c:1176-1178: R<<16 + G<<8 + B, rounded, not clamped */
static inline uint32_t pack_color(const float c[3]) {
    return ((uint32_t)orc_cvt_rn(c[0] * 255.0f) << 16) + ((uint32_t)orc_cvt_rn(c[1] * 255.0f) << 8) +
           (uint32_t)orc_cvt_rn(c[2] * 255.0f);
}

/* ---------------------------------------------------------------- clears (main.c:1191-1217) */

static uint32_t tiles_x(const orc_target *t) { return (t->width + TILE - 1) / TILE; }
static uint32_t tiles_y(const orc_target *t) { return (t->height + TILE - 1) / TILE; }

void orc_clear_color(orc_target *t, const float rgba[4]) {
    uint32_t v = orc_encode_clear_color(rgba);
    size_t n = (size_t)t->width * t->height;
    for (size_t i = 0; i < n; ++i) t->color[i] = v;
    if (t->vis_tri) for (size_t i = 0; i < n; ++i) t->vis_tri[i] = 0xFFFFFFFFu;
    if (t->vis_draw) for (size_t i = 0; i < n; ++i) t->vis_draw[i] = 0xFFFFFFFFu;
    if (t->vis_prim) for (size_t i = 0; i < n; ++i) t->vis_prim[i] = 0xFFFFFFFFu;
    if (t->vis_bary) for (size_t i = 0; i < 2 * n; ++i) t->vis_bary[i] = 0.f;
}

void orc_clear_depth(orc_target *t, float depth) {
    size_t n = (size_t)t->width * t->height;
    for (size_t i = 0; i < n; ++i) t->depth[i] = depth;
    size_t nt = (size_t)tiles_x(t) * tiles_y(t);
    for (size_t i = 0; i < nt; ++i) { t->tile_min[i] = 0.0f; t->tile_max[i] = 1.0f; }
}

/* ---------------------------------------------------------------- clipping (main.c:609-660) */

static float g_plane[6][4];
static int g_planes_ready;

static void init_planes(void) {
    /* v4f32_normalize, math.h:267-270: length via double sqrt returned as float, 1.0/length in
     * double stored as float, then a float multiply */
    static const float raw[6][4] = {{1, 0, 0, 1}, {-1, 0, 0, 1}, {0, 1, 0, 1},
                                    {0, -1, 0, 1}, {0, 0, 1, 1}, {0, 0, -1, 1}};
    for (int p = 0; p < 6; ++p) {
        float len = (float)sqrt((double)dot4_lr(raw[p], raw[p]));
        float inv = (float)(1.0 / (double)len);
        for (int k = 0; k < 4; ++k) g_plane[p][k] = raw[p][k] * inv;
    }
    g_planes_ready = 1;
}

static void clip_by_plane(vtx *v, const float n[4], int *count) {
    vtx res[MAX_CLIP_VERTICES];
    int out = 0, nv = *count;
    if (nv <= 0) return;
    float cd = dot4_lr(n, v[0].r[0]);
    int cin = cd > -0.0f;
    for (int i = 0; i < nv; ++i) {
        int next = (i + 1) % nv;
        if (cin && out < MAX_CLIP_VERTICES) res[out++] = v[i];
        float nd = dot4_lr(n, v[next].r[0]);
        int nin = nd > -0.0f;
        if (cin != nin && out < MAX_CLIP_VERTICES) {
            float t = (0.0f + cd) / (cd - nd);
            float omt = 1.f - t;
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < 4; ++k) res[out].r[a][k] = v[i].r[a][k] * omt + v[next].r[a][k] * t;
            ++out;
        }
        cd = nd;
        cin = nin;
    }
    *count = out;
    memcpy(v, res, sizeof(vtx) * (size_t)out);
}

/* ---------------------------------------------------------------- primitive assembly */

static inline void set_edge(int32_t e[3], int32_t area, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
    /* main.c:563-575 (wrapping int32 arithmetic) */
    uint32_t a = (uint32_t)y0 - (uint32_t)y1;
    uint32_t b = (uint32_t)x1 - (uint32_t)x0;
    if (area < 0) { a = 0u - a; b = 0u - b; }
    uint32_t c = (0u - a) * (uint32_t)x0 - b * (uint32_t)y0;
    e[0] = (int32_t)a; e[1] = (int32_t)b; e[2] = (int32_t)c;
}

typedef struct tri_buf { tri_rec *v; size_t n, cap; } tri_buf;

static void push_tri(tri_buf *b, const tri_rec *r) {
    if (b->n == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 256;
        b->v = (tri_rec *)realloc(b->v, sizeof(tri_rec) * b->cap);
    }
    b->v[b->n++] = *r;
}

/* primitive_assembly_stage body for one input triangle, main.c:753-907 */
static int assemble(const orc_draw *d, const float vout[3][12], uint32_t input, tri_buf *out) {
    const float *p0 = vout[0], *p1 = vout[1], *p2 = vout[2];
    if (p0[3] == 0 || p1[3] == 0 || p2[3] == 0) return 0;
    if ((p0[0] < -p0[3] && p1[0] < -p1[3] && p2[0] < -p2[3]) ||
        (p0[0] > +p0[3] && p1[0] > +p1[3] && p2[0] > +p2[3]) ||
        (p0[1] < -p0[3] && p1[1] < -p1[3] && p2[1] < -p2[3]) ||
        (p0[1] > +p0[3] && p1[1] > +p1[3] && p2[1] > +p2[3]) ||
        (p0[2] < 0.f && p1[2] < 0.f && p2[2] < 0.f) ||
        (p0[2] > +p0[3] && p1[2] > +p1[3] && p2[2] > +p2[3]))
        return 0;
    int clip = !((p0[0] >= -p0[3] && p1[0] >= -p1[3] && p2[0] >= -p2[3]) &&
                 (p0[0] <= +p0[3] && p1[0] <= +p1[3] && p2[0] <= +p2[3]) &&
                 (p0[1] >= -p0[3] && p1[1] >= -p1[3] && p2[1] >= -p2[3]) &&
                 (p0[1] <= +p0[3] && p1[1] <= +p1[3] && p2[1] <= +p2[3]) &&
                 (p0[2] >= 0.f && p1[2] >= 0.f && p2[2] >= 0.f) &&
                 (p0[2] <= +p0[3] && p1[2] <= +p1[3] && p2[2] <= +p2[3]));
    vtx poly[MAX_CLIP_VERTICES];
    for (int v = 0; v < 3; ++v) memcpy(poly[v].r, vout[v], 12 * sizeof(float));
    int count = 3;
    if (clip)
        for (int p = 0; p < 6; ++p) clip_by_plane(poly, g_plane[p], &count);

    const float *vp = d->viewport;
    /* screen_from_ndc, main.c:825-830 */
    float m[16] = {(float)(vp[2] * 0.5), 0, 0, (float)(vp[2] * 0.5 + vp[0]),
                   0, (float)(-vp[3] * 0.5), 0, (float)(vp[3] * 0.5 + vp[1]),
                   0, 0, vp[5] - vp[4], vp[4],
                   0, 0, 0, 1};
    int32_t vw = (int32_t)vp[2], vh = (int32_t)vp[3];
    for (int f = 1; f < count - 1; ++f) {
        const vtx *tv[3] = {&poly[0], &poly[f], &poly[f + 1]};
        float pos[3][4], rw[3], ss[3][4];
        for (int k = 0; k < 3; ++k) {
            memcpy(pos[k], tv[k]->r[0], 16);
            rw[k] = (float)(1.0 / (double)pos[k][3]);
            for (int c = 0; c < 4; ++c) pos[k][c] *= rw[k];
            for (int r = 0; r < 4; ++r) ss[k][r] = dot4_lr(m + 4 * r, pos[k]);
        }
        int32_t x[3], y[3];
        for (int k = 0; k < 3; ++k) { x[k] = orc_snap(ss[k][0]); y[k] = orc_snap(ss[k][1]); }
        int32_t area = (int32_t)(((uint32_t)x[1] - (uint32_t)x[0]) * ((uint32_t)y[2] - (uint32_t)y[0]) -
                                 ((uint32_t)x[2] - (uint32_t)x[0]) * ((uint32_t)y[1] - (uint32_t)y[0]));
        if (d->cull == ORC_CULL_BACK && area > 0) continue;
        if (d->cull == ORC_CULL_FRONT && area < 0) continue;
        tri_rec r;
        r.input = input;
        set_edge(r.e[2], area, x[0], y[0], x[1], y[1]);
        set_edge(r.e[0], area, x[1], y[1], x[2], y[2]);
        set_edge(r.e[1], area, x[2], y[2], x[0], y[0]);
        if (d->sample_center) /* E at (x + 1/2, y + 1/2): ((a x) << 4) + 8 a + ((b y) << 4) + 8 b + c */
            for (int e = 0; e < 3; ++e)
                r.e[e][2] = (int32_t)((uint32_t)r.e[e][2] + (((uint32_t)r.e[e][0] + (uint32_t)r.e[e][1]) << 3));
        float af = (float)(area >> (SUBPIX * 2));
        if (af == 0.0f) af = 1.0f;
        r.inv_area = fabsf(1.f / af);
        r.rw[0] = rw[0]; r.rw[1] = rw[1]; r.rw[2] = rw[2];
        if (d->depth_func == ORC_DEPTH_LESS)
            r.zbound = mn(ss[0][2], mn(ss[1][2], ss[2][2]));
        else
            r.zbound = mx(ss[0][2], mx(ss[1][2], ss[2][2]));
        for (int k = 0; k < 3; ++k) {
            memcpy(r.attrs[k], tv[k]->r, sizeof(r.attrs[k]));
            memcpy(r.attrs[k][0], ss[k], 16);
        }
        int32_t minx = (x[0] < (x[1] < x[2] ? x[1] : x[2]) ? x[0] : (x[1] < x[2] ? x[1] : x[2])) >> SUBPIX;
        int32_t miny = (y[0] < (y[1] < y[2] ? y[1] : y[2]) ? y[0] : (y[1] < y[2] ? y[1] : y[2])) >> SUBPIX;
        int32_t maxx = (x[0] > (x[1] > x[2] ? x[1] : x[2]) ? x[0] : (x[1] > x[2] ? x[1] : x[2])) >> SUBPIX;
        int32_t maxy = (y[0] > (y[1] > y[2] ? y[1] : y[2]) ? y[0] : (y[1] > y[2] ? y[1] : y[2])) >> SUBPIX;
        minx = minx > 0 ? minx : 0; minx = minx < vw - 1 ? minx : vw - 1;
        miny = miny > 0 ? miny : 0; miny = miny < vh - 1 ? miny : vh - 1;
        maxx = maxx + 1 < vw - 1 ? maxx + 1 : vw - 1;
        maxy = maxy + 1 < vh - 1 ? maxy + 1 : vh - 1;
        r.minx = minx; r.miny = miny; r.maxx = maxx; r.maxy = maxy;
        push_tri(out, &r);
    }
    return clip;
}

static int vertex_fetch(const orc_draw *d, uint32_t idx_pos, float in[8]) {
    int64_t idx = d->ib ? (int64_t)d->ib[idx_pos] : (int64_t)idx_pos;
    idx += d->base_vertex;
    if (idx < 0 || idx >= (int64_t)d->vertex_count) return -1;
    memcpy(in, (const uint8_t *)d->vb + (size_t)idx * d->vb_stride, 8 * sizeof(float));
    return 0;
}

/* ---------------------------------------------------------------- draw */

static int texture_ok(const orc_texture *t, int want_float, int any) {
    if (!t->data || t->width == 0 || t->height == 0) return 0;
    if (any) return 1;
    return want_float ? (t->format == ORC_FMT_RGBA32F || t->format == ORC_FMT_RGBA16F)
                      : (t->format == ORC_FMT_RGBA8);
}

static int validate(const orc_draw *d) {
    if (d->vs < ORC_VS_BASIC || d->vs > ORC_VS_PASSTHROUGH_UV) return -1;
    if (d->ps < ORC_PS_BASIC || d->ps > ORC_PS_NONE) return -1;
    if (d->vb_stride < 32 || !d->vb) return -1;
    if ((d->vs == ORC_VS_BASIC || d->vs == ORC_VS_VERTEX_LIGHTING || d->vs == ORC_VS_FULLSCREEN) && !d->cb)
        return -1;
    if (d->vs == ORC_VS_VERTEX_LIGHTING && !texture_ok(&d->vs_tex, 1, 0)) return -1;
    if (d->ps == ORC_PS_BASIC && !texture_ok(&d->ps_tex, 0, 0)) return -1;
    if (d->ps == ORC_PS_ENV_LIGHTING && !texture_ok(&d->ps_tex, 1, 0)) return -1;
    if (d->ps == ORC_PS_COLOR_TIMES_TEXEL && !texture_ok(&d->ps_tex, 0, 1)) return -1;
    return 0;
}

#define CHUNK 2048

int orc_draw_indexed(orc_target *t, const orc_draw *d, uint32_t draw_seq, orc_stats *st, orc_capture *cap) {
    if (!g_planes_ready) init_planes();
    if (validate(d)) return -1;
    const uint32_t ntri = d->index_count / 3;
    const uint32_t nchunks = (ntri + CHUNK - 1) / CHUNK;

    /* input assembler + vertex shader + primitive assembly (main.c:662-913); per-index shading as
     * in the reference; chunk-local output keeps the serial (input triangle, fan) order */
    tri_buf *chunks = (tri_buf *)calloc(nchunks ? nchunks : 1, sizeof(tri_buf));
    int bad = 0;
    uint64_t nclipped = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad) reduction(+ : nclipped)
    for (uint32_t c = 0; c < nchunks; ++c) {
        uint32_t end = (c + 1) * CHUNK < ntri ? (c + 1) * CHUNK : ntri;
        for (uint32_t i = c * CHUNK; i < end; ++i) {
            float vin[8], vout[3][12];
            for (int k = 0; k < 3; ++k) {
                if (vertex_fetch(d, d->start_index + 3 * i + k, vin)) { bad = 1; break; }
                orc_run_vs(d->vs, vin, d->cb, &d->vs_tex, vout[k]);
            }
            if (bad) break;
            nclipped += (uint64_t)assemble(d, (const float(*)[12])vout, i, &chunks[c]);
        }
    }
    if (bad) {
        for (uint32_t c = 0; c < nchunks; ++c) free(chunks[c].v);
        free(chunks);
        return -1;
    }
    size_t nasm = 0;
    size_t *coff = (size_t *)malloc(sizeof(size_t) * (nchunks + 1));
    for (uint32_t c = 0; c < nchunks; ++c) { coff[c] = nasm; nasm += chunks[c].n; }
    tri_rec *tris = (tri_rec *)malloc(sizeof(tri_rec) * (nasm ? nasm : 1));
#pragma omp parallel for schedule(dynamic, 1)
    for (uint32_t c = 0; c < nchunks; ++c) {
        if (chunks[c].n) memcpy(tris + coff[c], chunks[c].v, sizeof(tri_rec) * chunks[c].n);
        free(chunks[c].v);
    }
    free(chunks);
    free(coff);

    /* binner, main.c:915-981 (serial, like the reference) */
    const int32_t tx = (int32_t)tiles_x(t), ty = (int32_t)tiles_y(t);
    const size_t nbins = (size_t)tx * ty;
    uint32_t *cnt = (uint32_t *)calloc(nbins + 1, sizeof(uint32_t));
    for (size_t i = 0; i < nasm; ++i) {
        const tri_rec *r = tris + i;
        int32_t bx0 = r->minx / TILE; bx0 = bx0 > 0 ? bx0 : 0;
        int32_t by0 = r->miny / TILE; by0 = by0 > 0 ? by0 : 0;
        int32_t bx1 = r->maxx / TILE; bx1 = bx1 < tx - 1 ? bx1 : tx - 1;
        int32_t by1 = r->maxy / TILE; by1 = by1 < ty - 1 ? by1 : ty - 1;
        for (int32_t y = by0; y <= by1; ++y)
            for (int32_t x = bx0; x <= bx1; ++x) cnt[(size_t)y * tx + x]++;
    }
    uint32_t *upto = (uint32_t *)malloc(sizeof(uint32_t) * (nbins + 1));
    size_t total = 0, active = 0;
    for (size_t b = 0; b < nbins; ++b) {
        upto[b] = (uint32_t)total;
        total += cnt[b];
        if (cnt[b]) ++active;
    }
    upto[nbins] = (uint32_t)total;
    uint32_t *ids = (uint32_t *)malloc(sizeof(uint32_t) * (total ? total : 1));
    uint32_t *cur = (uint32_t *)calloc(nbins, sizeof(uint32_t));
    for (size_t i = 0; i < nasm; ++i) {
        const tri_rec *r = tris + i;
        int32_t bx0 = r->minx / TILE; bx0 = bx0 > 0 ? bx0 : 0;
        int32_t by0 = r->miny / TILE; by0 = by0 > 0 ? by0 : 0;
        int32_t bx1 = r->maxx / TILE; bx1 = bx1 < tx - 1 ? bx1 : tx - 1;
        int32_t by1 = r->maxy / TILE; by1 = by1 < ty - 1 ? by1 : ty - 1;
        for (int32_t y = by0; y <= by1; ++y)
            for (int32_t x = bx0; x <= bx1; ++x) {
                size_t b = (size_t)y * tx + x;
                ids[upto[b] + cur[b]++] = (uint32_t)i;
            }
    }
    free(cur);
    uint32_t *active_list = (uint32_t *)malloc(sizeof(uint32_t) * (active ? active : 1));
    {
        size_t k = 0;
        for (size_t b = 0; b < nbins; ++b)
            if (cnt[b]) active_list[k++] = (uint32_t)b;
    }
    uint64_t *masks = cap ? (uint64_t *)malloc(sizeof(uint64_t) * (total ? total : 1)) : NULL;

    /* rasteriser + pixel stage + output merger, per bin (main.c:983-1189, 577-603). The
     * hierarchical-Z value read here is the one the previous draws left: only this bin writes it. */
    const int less = d->depth_func == ORC_DEPTH_LESS;
    uint64_t frags = 0;
#pragma omp parallel for schedule(dynamic, 32) reduction(+ : frags)
    for (size_t k = 0; k < active; ++k) {
        const uint32_t b = active_list[k];
        const int32_t x0 = (int32_t)(b % (uint32_t)tx) * TILE, y0 = (int32_t)(b / (uint32_t)tx) * TILE;
        uint32_t tcol[64], ttri[64], tdraw[64], tprim[64];
        float tdep[64], tbary[128];
        uint8_t valid[64];
        for (int j = 0; j < 8; ++j)
            for (int i = 0; i < 8; ++i) {
                int p = j * 8 + i;
                int32_t x = x0 + i, y = y0 + j;
                valid[p] = (x < (int32_t)t->width && y < (int32_t)t->height);
                size_t o = valid[p] ? (size_t)y * t->width + x : 0;
                tcol[p] = valid[p] ? t->color[o] : 0;
                tdep[p] = valid[p] ? t->depth[o] : 0.f;
                if (t->vis_tri) ttri[p] = valid[p] ? t->vis_tri[o] : 0;
                if (t->vis_draw) tdraw[p] = valid[p] ? t->vis_draw[o] : 0;
                if (t->vis_prim) tprim[p] = valid[p] ? t->vis_prim[o] : 0;
                if (t->vis_bary) { tbary[2 * p] = valid[p] ? t->vis_bary[2 * o] : 0; tbary[2 * p + 1] = valid[p] ? t->vis_bary[2 * o + 1] : 0; }
            }
        const float hiz = less ? t->tile_max[b] : t->tile_min[b];
        for (uint32_t q = upto[b]; q < upto[b + 1]; ++q) {
            const tri_rec *r = tris + ids[q];
            uint64_t mask = 0;
            int rejected = less ? (r->zbound > hiz) : (r->zbound < hiz);
            if (!rejected) {
                for (int j = 0; j < 8; ++j)
                    for (int i = 0; i < 8; ++i) {
                        uint32_t x = (uint32_t)(x0 + i), y = (uint32_t)(y0 + j);
                        uint32_t ev[3];
                        for (int e = 0; e < 3; ++e)
                            ev[e] = (((uint32_t)r->e[e][0] * x) << SUBPIX) + (((uint32_t)r->e[e][1] * y) << SUBPIX) +
                                    (uint32_t)r->e[e][2];
                        int cov;
                        if (d->fill_rule) {
                            /* top-left: E > 0, or E == 0 on a left edge (interior to its right, a > 0)
                             * or a top edge (horizontal, interior below it, a == 0 and b > 0) */
                            uint32_t bias[3];
                            for (int e = 0; e < 3; ++e)
                                bias[e] = (r->e[e][0] > 0 || (r->e[e][0] == 0 && r->e[e][1] > 0)) ? 0u : 1u;
                            cov = (int32_t)((ev[0] - bias[0]) | (ev[1] - bias[1]) | (ev[2] - bias[2])) >= 0;
                        } else {
                            cov = (int32_t)(ev[0] | ev[1] | ev[2]) > 0;
                        }
                        if (cov && valid[j * 8 + i]) mask |= (uint64_t)1 << (j * 8 + i);
                    }
            }
            if (masks) masks[q] = mask;
            if (!mask) continue;
            for (int p = 0; p < 64; ++p) {
                if (!(mask >> p & 1)) continue;
                uint32_t x = (uint32_t)(x0 + (p & 7)), y = (uint32_t)(y0 + (p >> 3));
                int32_t e1 = (int32_t)((((uint32_t)r->e[1][0] * x) << SUBPIX) + (((uint32_t)r->e[1][1] * y) << SUBPIX) +
                                       (uint32_t)r->e[1][2]);
                int32_t e2 = (int32_t)((((uint32_t)r->e[2][0] * x) << SUBPIX) + (((uint32_t)r->e[2][1] * y) << SUBPIX) +
                                       (uint32_t)r->e[2][2]);
                float b1 = (float)(e1 >> (SUBPIX * 2)) * r->inv_area;
                float b2 = (float)(e2 >> (SUBPIX * 2)) * r->inv_area;
                float den = (1.0f - (b1 + b2)) * r->rw[0];
                den = den + b1 * r->rw[1];
                den = den + b2 * r->rw[2];
                den = 1.0f / den;
                float pb1 = (b1 * r->rw[1]) * den;
                float pb2 = (b2 * r->rw[2]) * den;
                float at[12];
                for (int a = 0; a < 3; ++a) {
                    float u = a ? pb1 : b1, v = a ? pb2 : b2;
                    for (int c = 0; c < 4; ++c) {
                        float v0 = r->attrs[0][a][c], v1 = r->attrs[1][a][c], v2 = r->attrs[2][a][c];
                        float tmp = v0 + (v1 - v0) * u;
                        at[a * 4 + c] = tmp + (v2 - v0) * v;
                    }
                }
                float z = at[2];
                int pass = less ? (z < tdep[p]) : (z >= tdep[p]);
                if (!pass) continue;
                if (d->ps != ORC_PS_NONE) { /* a null pixel shader leaves the colour */
                    float col[3];
                    orc_run_ps(d->ps, at, &d->ps_tex, col);
                    tcol[p] = pack_color(col);
                }
                tdep[p] = z;
                ttri[p] = ids[q];
                tdraw[p] = draw_seq;
                tprim[p] = r->input;
                tbary[2 * p] = b1; tbary[2 * p + 1] = b2;
                ++frags;
            }
        }
        float mnz = 1.0f, mxz = 0.0f;
        for (int j = 0; j < 8; ++j)
            for (int i = 0; i < 8; ++i) {
                int p = j * 8 + i;
                if (!valid[p]) continue;
                size_t o = (size_t)(y0 + j) * t->width + (x0 + i);
                t->color[o] = tcol[p];
                t->depth[o] = tdep[p];
                if (t->vis_tri) t->vis_tri[o] = ttri[p];
                if (t->vis_draw) t->vis_draw[o] = tdraw[p];
                if (t->vis_prim) t->vis_prim[o] = tprim[p];
                if (t->vis_bary) { t->vis_bary[2 * o] = tbary[2 * p]; t->vis_bary[2 * o + 1] = tbary[2 * p + 1]; }
                mnz = mn(mnz, tdep[p]);
                mxz = mx(mxz, tdep[p]);
            }
        t->tile_min[b] = mnz;
        t->tile_max[b] = mxz;
    }

    if (st) {
        st->vertex_count += d->index_count;
        st->input_triangle_count += ntri;
        st->assembled_triangle_count += nasm;
        st->active_bin_count += active;
        st->total_triangle_count_in_bins += total;
        st->fragments_written += frags;
        st->clipped_triangle_count += nclipped;
    }
    if (cap) {
        orc_capture_free(cap);
        cap->n_tris = (uint32_t)nasm;
        size_t n = nasm ? nasm : 1;
        cap->edges = (int32_t *)malloc(sizeof(int32_t) * 9 * n);
        cap->rw = (float *)malloc(sizeof(float) * 3 * n);
        cap->inv_area = (float *)malloc(sizeof(float) * n);
        cap->depth_bound = (float *)malloc(sizeof(float) * n);
        cap->bounds = (int32_t *)malloc(sizeof(int32_t) * 4 * n);
        cap->attrs = (float *)malloc(sizeof(float) * 36 * n);
        for (size_t i = 0; i < nasm; ++i) {
            const tri_rec *r = tris + i;
            memcpy(cap->edges + 9 * i, r->e, sizeof(r->e));
            memcpy(cap->rw + 3 * i, r->rw, sizeof(r->rw));
            cap->inv_area[i] = r->inv_area;
            cap->depth_bound[i] = r->zbound;
            cap->bounds[4 * i + 0] = r->minx; cap->bounds[4 * i + 1] = r->miny;
            cap->bounds[4 * i + 2] = r->maxx; cap->bounds[4 * i + 3] = r->maxy;
            memcpy(cap->attrs + 36 * i, r->attrs, sizeof(r->attrs));
        }
        cap->n_infos = (uint32_t)total;
        size_t m = total ? total : 1;
        cap->info_bin = (uint32_t *)malloc(sizeof(uint32_t) * m);
        cap->info_tri = (uint32_t *)malloc(sizeof(uint32_t) * m);
        cap->info_mask = masks;
        masks = NULL;
        for (size_t b = 0; b < nbins; ++b)
            for (uint32_t q = upto[b]; q < upto[b + 1]; ++q) { cap->info_bin[q] = (uint32_t)b; cap->info_tri[q] = ids[q]; }
    }
    free(masks);
    free(active_list);
    free(ids);
    free(upto);
    free(cnt);
    free(tris);
    return 0;
}

void orc_capture_free(orc_capture *cap) {
    if (!cap) return;
    free(cap->edges); free(cap->rw); free(cap->inv_area); free(cap->depth_bound);
    free(cap->bounds); free(cap->attrs); free(cap->info_bin); free(cap->info_tri); free(cap->info_mask);
    memset(cap, 0, sizeof(*cap));
}
