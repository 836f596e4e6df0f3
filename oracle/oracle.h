/* Malevich draw-path oracle: a scalar C restatement of the reference's pipeline core.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py may load this code, and only as the checker or the timed CPU baseline; the product
 * (malevich_gb300) never calls it.
 *
 * It follows source/main.c:563-1217 (clip, IA/VS, primitive assembly, binner, rasteriser, pixel
 * stage, clears), source/common_shader_core.h:26-53,83-161,226-244 (texel fetch, bilinear and
 * lat-long sampling), source/math.h:137-177,277-280,322-344,376-427 and the seven shader files,
 * in the same floating-point operation order (compile with -ffp-contract=off). Parity is pinned
 * against the reference itself, compiled headless from its sources by oracle/ref_build.py.
 *
 * Deliberate, documented departures (each one is a mode the reference lacks, or a reference
 * behaviour that cannot be reproduced):
 *   - rsqrt: the reference normalises with _mm256_rsqrt_ps (an approximate, CPU-model specific
 *     instruction, math.h:277-280). The oracle uses the correctly rounded 1.0f/sqrtf(x).
 *   - acos/exp/pow: the reference links Intel SVML (closed). The oracle calls libm acosf/expf/powf.
 *   - Depth LESS with a mirrored hierarchical-Z (tile maximum), cull modes NONE/FRONT,
 *     RGBA16F textures, the PASSTHROUGH_UV vertex shader and COLOR_TIMES_TEXEL pixel shader,
 *     start-index/base-vertex offsets, arbitrary render-target sizes (partial edge tiles) and
 *     index counts that are not a multiple of 8.
 * Assembled triangles keep the serial order (input triangle, clip-fan index); the reference is
 * only deterministic in that order with one OpenMP thread (main.c:874-875).
 */
#ifndef MALEVICH_ORACLE_H
#define MALEVICH_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_FMT_RGBA8 = 1, ORC_FMT_RGBA16F = 2, ORC_FMT_RGBA32F = 3 };
enum { ORC_VS_BASIC = 1, ORC_VS_VERTEX_LIGHTING = 2, ORC_VS_PASSTHROUGH = 3, ORC_VS_FULLSCREEN = 4,
       ORC_VS_PASSTHROUGH_UV = 5 };
enum { ORC_PS_BASIC = 1, ORC_PS_PASSTHROUGH = 2, ORC_PS_ENV_LIGHTING = 3, ORC_PS_COLOR_TIMES_TEXEL = 4, ORC_PS_NONE = 5 };
enum { ORC_CULL_NONE = 0, ORC_CULL_BACK = 1, ORC_CULL_FRONT = 2 };
enum { ORC_DEPTH_GREATER_EQUAL = 0, ORC_DEPTH_LESS = 1 };

typedef struct orc_texture {
    const void *data;
    uint32_t width, height;
    int32_t format;
} orc_texture;

typedef struct orc_draw {
    int32_t vs, ps;
    const void *vb;
    uint32_t vb_stride;          /* bytes; the VS reads the first 32 bytes of each vertex */
    uint32_t vertex_count;       /* vertices available in vb (indices are checked against it) */
    const uint32_t *ib;          /* NULL: Draw() with implicit indices start..start+count-1 */
    uint32_t index_count, start_index;
    int32_t base_vertex;
    const float *cb;             /* 48 floats: clip_from_world, view_from_clip, world_from_view */
    orc_texture vs_tex, ps_tex;
    float viewport[6];           /* top_left_x, top_left_y, width, height, min_depth, max_depth */
    int32_t cull, depth_func;
    /* Modes the reference lacks (0 = the reference): fill_rule 1 = top-left (an edge value of 0
     * covers only on a top or left edge, instead of the inclusive (E0|E1|E2) > 0 of main.c:1028);
     * sample_center 1 = test and interpolate at the pixel centre instead of its corner (main.c:1014). */
    int32_t fill_rule, sample_center;
} orc_draw;

typedef struct orc_target {
    uint32_t *color;
    float *depth;
    uint32_t width, height;
    float *tile_min, *tile_max;  /* per 8x8 tile, ceil(w/8)*ceil(h/8) */
    uint32_t *vis_tri;           /* optional: assembled triangle index of the last writer */
    uint32_t *vis_draw;          /* optional: draw sequence number of the last writer */
    float *vis_bary;             /* optional: 2 floats per pixel, quantised (b1, b2) */
    uint32_t *vis_prim;          /* optional: input triangle index (within its draw) of the last writer */
} orc_target;

typedef struct orc_stats {
    uint64_t vertex_count, input_triangle_count, assembled_triangle_count;
    uint64_t active_bin_count, total_triangle_count_in_bins, fragments_written;
    uint64_t clipped_triangle_count;  /* input triangles that went through the clipper */
} orc_stats;

/* Optional capture of one draw's intermediate results. Arrays are (re)allocated by the oracle
 * and released with orc_capture_free. */
typedef struct orc_capture {
    uint32_t n_tris;
    int32_t *edges;       /* n*9: edge0 a,b,c, edge1 a,b,c, edge2 a,b,c */
    float *rw;            /* n*3 */
    float *inv_area;      /* n */
    float *depth_bound;   /* n: max z (GREATER_EQUAL) or min z (LESS) */
    int32_t *bounds;      /* n*4: min x, min y, max x, max y */
    float *attrs;         /* n*36: 3 vertices x 3 registers x float4 */
    uint32_t n_infos;
    uint32_t *info_bin, *info_tri;
    uint64_t *info_mask;  /* coverage AND hierarchical-Z pass, bit (row*8+col) */
} orc_capture;

void orc_set_threads(int n);
int orc_max_threads(void);
void orc_clear_color(orc_target *t, const float rgba[4]);
void orc_clear_depth(orc_target *t, float depth);
/* Returns 0, or -1 on invalid arguments (an index outside the vertex buffer, a texture of the
 * wrong format, an unknown shader). */
int orc_draw_indexed(orc_target *t, const orc_draw *d, uint32_t draw_seq, orc_stats *stats,
                     orc_capture *cap);
void orc_capture_free(orc_capture *cap);

/* Differentiable shading model in FP64 (oracle_adjoint.c): vertex colour times a bilinear RGBA32F
 * texel, continuous barycentrics at the pixel corner under fixed visibility (prim). */
typedef struct orc_diff_scene {
    uint32_t n_verts, n_tris;
    const uint32_t *ib;          /* 3 * n_tris */
    const double *col;           /* 3 * n_verts */
    const double *uv;            /* 2 * n_verts */
    const double *tex;           /* th * tw * 4 */
    uint32_t tw, th;
} orc_diff_scene;

typedef struct orc_diff_view {
    uint32_t width, height;
    const double *pos;           /* 2 * n_verts: passthrough x, y in [0,1] */
    const uint32_t *prim;        /* width * height: input triangle or 0xFFFFFFFF */
    const double *target;        /* width * height * 3 */
    const int32_t *cells;        /* optional frozen bilinear cells (s0, t0) per pixel */
} orc_diff_view;

double orc_diff_loss(const orc_diff_scene *s, const orc_diff_view *views, uint32_t nviews, double *image);
void orc_diff_cells(const orc_diff_scene *s, const orc_diff_view *v, int32_t *cells);
/* The same cells chosen with the GPU kernels' single-precision operation sequence. */
void orc_diff_cells_f32(const orc_diff_scene *s, const orc_diff_view *v, int32_t *cells);
void orc_diff_grad(const orc_diff_scene *s, const orc_diff_view *views, uint32_t nviews, double *g_col,
                   double *g_tex, double *g_pos);

/* Building blocks exposed for the known-answer tests. */
uint32_t orc_encode_clear_color(const float rgba[4]);
int32_t orc_cvt_rn(float x);
int32_t orc_snap(float x_ss);
void orc_run_vs(int32_t vs, const float in[8], const float *cb, const orc_texture *tex, float out[12]);
void orc_run_ps(int32_t ps, const float attrs[12], const orc_texture *tex, float out[3]);

#ifdef __cplusplus
}
#endif
#endif
