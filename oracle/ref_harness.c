/* Test infrastructure only: a headless driver around the reference's own pipeline core.
 *
 * It is compiled together with the patched copy of source/main.c that oracle/ref_build.py writes
 * into oracle/_ref/src (the copy is included below), and it does what the reference's render()
 * does for one draw (source/main.c:1276-1295): sets the global Pipeline fields, the VS/PS
 * function pointers and SRV slot 0, then calls draw_indexed(). Clears go through
 * clear_render_target_view / clear_depth_stencil_view (main.c:1191-1217). The instrumentation
 * hooks defined here receive the assembled triangles, the per-(bin, triangle) TileInfo masks and
 * the triangle id of every colour store, so tests can compare them with the GPU path. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

void ref_hook_triangles(const void *tris, unsigned n, const void *attrs);
void ref_hook_tile_infos(const void *infos, unsigned n, const void *bins, unsigned nbins, const unsigned *ids);
void ref_hook_read_ids(unsigned bin_index, uint64_t *ids);
void ref_hook_store_id(uint64_t *row, const void *mask, unsigned tri);
void ref_hook_write_ids(unsigned bin_index, const uint64_t *ids);

#define REF_HOOK_TRIANGLES(tris, n, attrs) ref_hook_triangles((tris), (n), (attrs))
#define REF_HOOK_TILE_INFOS(infos, n, bins, nbins, ids) ref_hook_tile_infos((infos), (n), (bins), (nbins), (ids))
#define REF_HOOK_READ_IDS(bin_index, ids) ref_hook_read_ids((bin_index), (ids))
#define REF_HOOK_STORE_ID(row, mask, tri) ref_hook_store_id((row), &(mask), (tri))
#define REF_HOOK_WRITE_IDS(bin_index, ids) ref_hook_write_ids((bin_index), (ids))

#include "main_core.c"

#define EXPORT __attribute__((visibility("default")))

static uint64_t g_ids[WIDTH * HEIGHT];   /* (draw sequence << 32) | assembled triangle id */
static uint32_t g_draw_seq;
static Texture2D g_vs_tex, g_ps_tex;

/* capture of the last draw */
static Triangle *g_tris; static float *g_attrs; static unsigned g_ntris, g_cap_tris;
static uint32_t *g_ti_bin, *g_ti_tri; static uint64_t *g_ti_mask; static unsigned g_nti, g_cap_ti;

void ref_hook_triangles(const void *tris, unsigned n, const void *attrs) {
    if (n > g_cap_tris) {
        g_cap_tris = n;
        g_tris = realloc(g_tris, sizeof(Triangle) * n);
        g_attrs = realloc(g_attrs, sizeof(float) * 36 * (size_t)n);
    }
    g_ntris = n;
    const Triangle *t = (const Triangle *)tris;
    for (unsigned i = 0; i < n; ++i) {
        g_tris[i] = t[i];
        memcpy(g_attrs + 36 * (size_t)i, t[i].p_attributes, sizeof(float) * 36);
    }
    (void)attrs;
}

void ref_hook_tile_infos(const void *infos, unsigned n, const void *bins, unsigned nbins, const unsigned *ids) {
    if (n > g_cap_ti) {
        g_cap_ti = n;
        g_ti_bin = realloc(g_ti_bin, 4 * (size_t)n);
        g_ti_tri = realloc(g_ti_tri, 4 * (size_t)n);
        g_ti_mask = realloc(g_ti_mask, 8 * (size_t)n);
    }
    const TileInfo *ti = (const TileInfo *)infos;
    const CompactedBin *cb = (const CompactedBin *)bins;
    unsigned k = 0;
    for (unsigned b = 0; b < nbins; ++b) {
        for (unsigned j = 0; j < cb[b].num_triangles_self; ++j) {
            const TileInfo *e = ti + cb[b].num_triangles_upto + j;
            g_ti_bin[k] = cb[b].bin_index;
            g_ti_tri[k] = e->triangle_id;
            g_ti_mask[k] = e->fragment_mask;
            ++k;
        }
    }
    g_nti = k;
    (void)ids;
}

void ref_hook_read_ids(unsigned bin_index, uint64_t *ids) {
    int x0 = TILE_WIDTH * (bin_index % WIDTH_IN_TILES), y0 = TILE_HEIGHT * (bin_index / WIDTH_IN_TILES);
    for (int j = 0; j < 8; ++j)
        for (int i = 0; i < 8; ++i) ids[j * 8 + i] = g_ids[(y0 + j) * WIDTH + x0 + i];
}

void ref_hook_store_id(uint64_t *row, const void *mask, unsigned tri) {
    int32_t m[8];
    memcpy(m, mask, sizeof(m));
    for (int k = 0; k < 8; ++k)
        if (m[k]) row[k] = ((uint64_t)g_draw_seq << 32) | tri;
}

void ref_hook_write_ids(unsigned bin_index, const uint64_t *ids) {
    int x0 = TILE_WIDTH * (bin_index % WIDTH_IN_TILES), y0 = TILE_HEIGHT * (bin_index / WIDTH_IN_TILES);
    for (int j = 0; j < 8; ++j)
        for (int i = 0; i < 8; ++i) g_ids[(y0 + j) * WIDTH + x0 + i] = ids[j * 8 + i];
}

EXPORT int ref_width(void) { return WIDTH; }
EXPORT int ref_height(void) { return HEIGHT; }
EXPORT void ref_set_threads(int n) { omp_set_num_threads(n); }

EXPORT void ref_clear(const float *rgba, float depth) {
    clear_render_target_view(rgba);
    clear_depth_stencil_view(depth);
    memset(g_ids, 0xFF, sizeof(g_ids));
    g_draw_seq = 0;
}

EXPORT void ref_set_viewport(const float *vp) {
    Viewport v = {vp[0], vp[1], vp[2], vp[3], vp[4], vp[5]};
    graphics_pipeline.rs.viewport = v;
}

static VertexShader *vs_by_id(int id) {
    switch (id) {
        case 1: return &basic_vs;
        case 2: return &vertex_lighting_vs;
        case 3: return &passthrough_vs;
        case 4: return &fullscreen_vs;
        default: return NULL;
    }
}

static PixelShader *ps_by_id(int id) {
    switch (id) {
        case 1: return &basic_ps;
        case 2: return &passthrough_ps;
        case 3: return &env_lighting_ps;
        default: return NULL;
    }
}

/* Shader ids: VS 1 basic, 2 vertex_lighting, 3 passthrough, 4 fullscreen; PS 1 basic,
 * 2 passthrough, 3 env_lighting. Returns 0 on success. */
EXPORT int ref_set_shaders(int vs_id, int ps_id) {
    VertexShader *vs = vs_by_id(vs_id);
    PixelShader *ps = ps_by_id(ps_id);
    if (!vs || !ps) return -1;
    graphics_pipeline.ia.input_layout = vs->in_vertex_size / VECTOR_WIDTH;
    graphics_pipeline.vs.output_register_count = vs->out_vertex_size / (sizeof(v4f32) * VECTOR_WIDTH);
    graphics_pipeline.vs.shader = vs->vs_main;
    graphics_pipeline.ps.shader = ps->ps_main;
    return 0;
}

EXPORT void ref_set_cb(const void *cb) { memcpy(&per_frame_cb, cb, sizeof(per_frame_cb)); }

EXPORT void ref_set_vs_texture(void *data, unsigned w, unsigned h) {
    g_vs_tex.p_data = data; g_vs_tex.width = w; g_vs_tex.height = h;
}

EXPORT void ref_set_ps_texture(void *data, unsigned w, unsigned h) {
    g_ps_tex.p_data = data; g_ps_tex.width = w; g_ps_tex.height = h;
}

EXPORT void ref_draw_indexed(void *vb, unsigned *ib, unsigned index_count) {
    graphics_pipeline.ia.primitive_topology = PRIMITIVE_TOPOLOGY_TRIANGLELIST;
    graphics_pipeline.om.p_colors = &frame_buffer[0][0];
    graphics_pipeline.om.p_depth = &depth_buffer[0][0];
    graphics_pipeline.vs.p_constant_buffers[0] = &per_frame_cb;
    graphics_pipeline.ia.p_index_buffer = ib;
    graphics_pipeline.ia.p_vertex_buffer = vb;
    graphics_pipeline.vs.p_shader_resource_views[0] = &g_vs_tex;
    graphics_pipeline.ps.p_shader_resource_views[0] = &g_ps_tex;
    draw_indexed(index_count);
    ++g_draw_seq;
}

EXPORT void ref_reset_stats(void) { memset(&stats, 0, sizeof(stats)); }

/* vertex_count, input_triangle_count, assembled_triangle_count, active_bin_count,
 * total_triangle_count_in_bins (main.c:199-206) */
EXPORT void ref_get_stats(unsigned *out) {
    out[0] = stats.vertex_count; out[1] = stats.input_triangle_count;
    out[2] = stats.assembled_triangle_count; out[3] = stats.active_bin_count;
    out[4] = stats.total_triangle_count_in_bins;
}

EXPORT const unsigned *ref_color(void) { return &frame_buffer[0][0]; }
EXPORT const float *ref_depth(void) { return &depth_buffer[0][0]; }
EXPORT const uint64_t *ref_ids(void) { return g_ids; }
EXPORT const float *ref_tile_min(void) { return a_tile_min_depths; }

EXPORT unsigned ref_last_triangle_count(void) { return g_ntris; }

/* edges: n*9 ints (edge0 a,b,c, edge1 a,b,c, edge2 a,b,c); rw: n*3; inv_area, max_depth: n;
 * bounds: n*4 (min x, min y, max x, max y); attrs: n*36 (3 vertices x 3 registers x float4) */
EXPORT void ref_last_triangles(int *edges, float *rw, float *inv_area, float *max_depth, int *bounds, float *attrs) {
    for (unsigned i = 0; i < g_ntris; ++i) {
        const Triangle *t = g_tris + i;
        for (int e = 0; e < 3; ++e) {
            edges[9 * i + 3 * e + 0] = t->setup.a_edge_functions[e].a;
            edges[9 * i + 3 * e + 1] = t->setup.a_edge_functions[e].b;
            edges[9 * i + 3 * e + 2] = t->setup.a_edge_functions[e].c;
            rw[3 * i + e] = t->setup.a_reciprocal_ws[e];
        }
        inv_area[i] = t->setup.one_over_area;
        max_depth[i] = t->setup.max_depth;
        bounds[4 * i + 0] = t->min_bounds.x; bounds[4 * i + 1] = t->min_bounds.y;
        bounds[4 * i + 2] = t->max_bounds.x; bounds[4 * i + 3] = t->max_bounds.y;
    }
    memcpy(attrs, g_attrs, sizeof(float) * 36 * (size_t)g_ntris);
}

EXPORT unsigned ref_last_tile_info_count(void) { return g_nti; }

EXPORT void ref_last_tile_infos(unsigned *bin_index, unsigned *tri_id, uint64_t *mask) {
    memcpy(bin_index, g_ti_bin, 4 * (size_t)g_nti);
    memcpy(tri_id, g_ti_tri, 4 * (size_t)g_nti);
    memcpy(mask, g_ti_mask, 8 * (size_t)g_nti);
}
