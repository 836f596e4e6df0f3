/* malevich.h: C ABI of the GB300-native Malevich draw path.
 *
 * A Direct3D-11-flavoured API over hand-written CUDA kernels for sm_103a. The reference
 * (OzgurCerlet/Malevich) has no device, context or resource objects: it draws through one global
 * `Pipeline graphics_pipeline` whose fields are assigned directly (source/main.c:109-115,222,
 * 1276-1294) and three functions, draw_indexed (main.c:1219), clear_render_target_view
 * (main.c:1191) and clear_depth_stencil_view (main.c:1204). Every entry point below names the
 * reference field or function it replaces. Each function returns an mlv_status; nothing aborts.
 *
 * Threading: a device may be used from several threads for resource creation; a context is
 * one CUDA stream and, like an ID3D11DeviceContext, is not thread-safe. Work is queued
 * asynchronously; readbacks and mlv_finish synchronise and report device-side errors.
 */
#ifndef MALEVICH_H
#define MALEVICH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MLV_API __attribute__((visibility("default")))
#else
#define MLV_API
#endif

#define MLV_ABI_VERSION 5

/* ------------------------------------------------------------------ status */

typedef enum mlv_status {
    MLV_OK = 0,
    MLV_ERROR_INVALID_ARG = 1,        /* a NULL handle, a size or format the call cannot take */
    MLV_ERROR_OUT_OF_MEMORY = 2,
    MLV_ERROR_CAPACITY_EXCEEDED = 3,  /* an internal buffer overflowed and could not be regrown */
    MLV_ERROR_DEVICE = 4,             /* a CUDA error; see mlv_get_last_error_string */
    MLV_ERROR_TIMEOUT = 5,            /* a bounded device-side wait gave up */
    MLV_ERROR_UNSUPPORTED = 6,
    MLV_ERROR_INVALID_STATE = 7       /* e.g. a draw with no render target bound */
} mlv_status;

/* Message of the last failing call on this thread (never NULL). */
MLV_API const char *mlv_get_last_error_string(void);
MLV_API int mlv_get_abi_version(void);

/* ------------------------------------------------------------------ handles */

typedef struct mlv_device_t *mlv_device;
typedef struct mlv_context_t *mlv_context;
typedef struct mlv_buffer_t *mlv_buffer;
typedef struct mlv_texture2d_t *mlv_texture2d;
typedef struct mlv_command_list_t *mlv_command_list;

/* ------------------------------------------------------------------ formats and descriptors */

typedef enum mlv_format {
    MLV_FORMAT_UNKNOWN = 0,
    /* 32-bit texel, R in the low byte (common_shader_core.h:26-36, math.h:326-344). Also the
     * render-target format: the reference's clear packs R in the low byte (math.h:322-324) and its
     * output merger stores R<<16 | G<<8 | B (main.c:1176-1178); both packings are kept. */
    MLV_FORMAT_R8G8B8A8_UNORM = 1,
    MLV_FORMAT_R16G16B16A16_FLOAT = 2,  /* new: widened exactly to float before filtering */
    MLV_FORMAT_R32G32B32A32_FLOAT = 3,  /* float4 texels (common_shader_core.h:38-53) */
    MLV_FORMAT_D32_FLOAT = 4,           /* depth buffer (main.c:36) */
    MLV_FORMAT_R32_UINT = 5,            /* index buffers (main.c:72); triangle-ID targets */
    MLV_FORMAT_R32G32_FLOAT = 6         /* barycentric targets */
} mlv_format;

typedef enum mlv_bind_flag {
    MLV_BIND_VERTEX_BUFFER = 0x1,
    MLV_BIND_INDEX_BUFFER = 0x2,
    MLV_BIND_CONSTANT_BUFFER = 0x4,
    MLV_BIND_SHADER_RESOURCE = 0x8,
    MLV_BIND_RENDER_TARGET = 0x20,
    MLV_BIND_DEPTH_STENCIL = 0x40,
    MLV_BIND_UNORDERED_ACCESS = 0x80
} mlv_bind_flag;

typedef struct mlv_buffer_desc {
    uint64_t byte_width;
    uint32_t bind_flags;
    uint32_t reserved;
} mlv_buffer_desc;

typedef struct mlv_texture2d_desc {
    uint32_t width, height;
    mlv_format format;
    uint32_t bind_flags;
} mlv_texture2d_desc;

/* Viewport, main.c:85-92 */
typedef struct mlv_viewport {
    float top_left_x, top_left_y, width, height, min_depth, max_depth;
} mlv_viewport;

/* PrimitiveTopology, main.c:66-69: triangle lists only */
typedef enum mlv_primitive_topology {
    MLV_PRIMITIVE_TOPOLOGY_UNDEFINED = 0,
    MLV_PRIMITIVE_TOPOLOGY_TRIANGLELIST = 1
} mlv_primitive_topology;

/* Culling. The reference always culls triangles whose signed screen-space area (y down, 28.4
 * fixed point) is positive (main.c:851-856): that is MLV_CULL_BACK, the default. */
typedef enum mlv_cull_mode { MLV_CULL_NONE = 1, MLV_CULL_FRONT = 2, MLV_CULL_BACK = 3 } mlv_cull_mode;

/* Coverage rule. The reference covers a pixel when (E0|E1|E2) > 0 at its sample point
 * (main.c:1028): every edge inclusive; its top-left rule is a TODO (main.c:1014,1027). TOP_LEFT
 * (new) covers a sample on an edge only for a left edge (interior to its right) or a top edge
 * (horizontal, interior below it), so a pixel on an edge shared by two triangles is covered once. */
typedef enum mlv_fill_rule { MLV_FILL_INCLUSIVE = 0, MLV_FILL_TOP_LEFT = 1 } mlv_fill_rule;

/* Sample point. The reference samples coverage and attributes at the pixel corner (x, y)
 * (main.c:1014-1025); PIXEL_CENTER (new) samples at (x + 1/2, y + 1/2). */
typedef enum mlv_sample_position { MLV_SAMPLE_PIXEL_CORNER = 0, MLV_SAMPLE_PIXEL_CENTER = 1 } mlv_sample_position;

typedef struct mlv_rasterizer_desc {
    mlv_cull_mode cull_mode;
    mlv_fill_rule fill_rule;              /* 0: the reference's rule */
    mlv_sample_position sample_position;  /* 0: the reference's sample point */
} mlv_rasterizer_desc;

/* Depth test. The reference tests GREATER_EQUAL (reversed Z, main.c:1166) against a tile
 * minimum for hierarchical Z (main.c:1005-1006). LESS is new; it keeps a mirrored tile maximum. */
typedef enum mlv_comparison_func {
    MLV_COMPARISON_LESS = 2,
    MLV_COMPARISON_GREATER_EQUAL = 7
} mlv_comparison_func;

typedef struct mlv_depth_stencil_desc {
    int32_t depth_enable;              /* must be 1 */
    mlv_comparison_func depth_func;
} mlv_depth_stencil_desc;

/* ------------------------------------------------------------------ shaders
 * The reference calls shaders through host function pointers (VS::shader, PS::shader,
 * main.c:79,99; common_shader_core.h:10-18). A GPU cannot call those, so shaders are built-in
 * and selected by id. Each keeps the reference's stage input/output layout, given below for one
 * vertex or fragment (the reference stores them 8-wide SoA: v3f256 = three __m256). */
typedef enum mlv_vertex_shader_id {
    MLV_VS_BASIC = 1,            /* basic_vs.c:22-35 */
    MLV_VS_VERTEX_LIGHTING = 2,  /* vertex_lighting_vs.c:22-41 (VS SRV 0: float lat-long map) */
    MLV_VS_PASSTHROUGH = 3,      /* passthrough_vs.c:16-27 */
    MLV_VS_FULLSCREEN = 4,       /* fullscreen_vs.c:22-41 */
    MLV_VS_PASSTHROUGH_UV = 5    /* new: passthrough with a UV, for the differentiable path */
} mlv_vertex_shader_id;

typedef enum mlv_pixel_shader_id {
    MLV_PS_BASIC = 1,            /* basic_ps.c:16-29 (PS SRV 0: RGBA8) */
    MLV_PS_PASSTHROUGH = 2,      /* passthrough_ps.c:13-22 */
    MLV_PS_ENV_LIGHTING = 3,     /* env_lighting_ps.c:13-26 (PS SRV 0: float lat-long map) */
    MLV_PS_COLOR_TIMES_TEXEL = 4, /* new: COLOR * bilinear(SRV 0, UV).xyz */
    MLV_PS_NONE = 5               /* new: no pixel shader (Direct3D 11's null PS): depth and the
                                     visibility targets are written, the render target is not */
} mlv_pixel_shader_id;

/* Vs_Input of basic_vs / vertex_lighting_vs (basic_vs.c:3-7): 32 bytes */
typedef struct mlv_vertex_basic { float position[3]; float normal[3]; float uv[2]; } mlv_vertex_basic;
/* Vs_Input of passthrough_vs (passthrough_vs.c:3-7): position already in [0,1] screen space */
typedef struct mlv_vertex_passthrough { float position[4]; float color[3]; float pad; } mlv_vertex_passthrough;
/* Vs_Input of fullscreen_vs (fullscreen_vs.c:3-7) */
typedef struct mlv_vertex_fullscreen { float position[4]; float view_dir[3]; float pad; } mlv_vertex_fullscreen;
/* Vs_Input of MLV_VS_PASSTHROUGH_UV (new): x, y in [0,1] screen space, z depth, w = 1 */
typedef struct mlv_vertex_passthrough_uv { float position[3]; float color[3]; float uv[2]; } mlv_vertex_passthrough_uv;

/* Vs_Output (basic_vs.c:9-14): three float4 registers per vertex, r0 = SV_POSITION,
 * r1 = (NORMAL|COLOR|VIEW_DIR).xyz + UV.x, r2 = UV.y + 3 pad (main.c:1286-1287: 12 floats) */
typedef struct mlv_vs_output { float sv_position[4]; float attr[3]; float uv[2]; float pad[3]; } mlv_vs_output;
/* Ps_Input (basic_ps.c:3-7) and Ps_Output (basic_ps.c:9-11) */
typedef struct mlv_ps_input { float sv_position[4]; float attr[3]; float uv[2]; } mlv_ps_input;
typedef struct mlv_ps_output { float sv_target[4]; } mlv_ps_output;

/* VS constant buffer slot 0 of the reference's shaders: PerFrameCB (main.c:169-173), row-major
 * matrices applied to column vectors. */
typedef struct mlv_per_frame_cb {
    float clip_from_world[16];
    float view_from_clip[16];
    float world_from_view[16];
} mlv_per_frame_cb;

#define MLV_CONSTANT_BUFFER_SLOT_COUNT 16   /* main.c:41 */
#define MLV_SHADER_RESOURCE_SLOT_COUNT 16   /* main.c:42 */

/* ------------------------------------------------------------------ device and contexts */

/* Creates a device on CUDA device `cuda_ordinal` (the reference has one implicit global). */
MLV_API mlv_status mlv_create_device(int cuda_ordinal, mlv_device *out_device);
/* Waits for the immediate context's work and frees it. The device's buffers, textures, deferred
 * contexts and command lists must be destroyed first (they refer to the device). */
MLV_API mlv_status mlv_destroy_device(mlv_device device);
/* The immediate context: draws execute as they are issued (main.c:1284-1296 calls
 * draw_indexed once per object). */
MLV_API mlv_status mlv_get_immediate_context(mlv_device device, mlv_context *out_context);
/* A deferred context records commands into a command list; executing the list runs all its
 * draws, across all the render targets they use, as one batched launch sequence that is captured
 * in a CUDA graph on first execution and replayed afterwards. */
MLV_API mlv_status mlv_create_deferred_context(mlv_device device, mlv_context *out_context);
MLV_API mlv_status mlv_destroy_context(mlv_context context);

/* ------------------------------------------------------------------ resources
 * The reference borrows caller pointers (IA::p_index_buffer, IA::p_vertex_buffer, Texture2D::p_data,
 * OM::p_colors/p_depth, main.c:71-107). Here resources own device memory; init data is copied.
 * Destroying a resource waits for the immediate context's queued work; a command list recorded
 * with it must not be executed afterwards (as in Direct3D 11). */
MLV_API mlv_status mlv_create_buffer(mlv_device device, const mlv_buffer_desc *desc, const void *init_data,
                                     mlv_buffer *out_buffer);
MLV_API mlv_status mlv_destroy_buffer(mlv_buffer buffer);
/* row_pitch: bytes between rows of init_data (0 = tightly packed; a pitch shorter than a row is
 * MLV_ERROR_INVALID_ARG, here and in the texture updates and readback). Depth textures carry the
 * per-8x8-tile hierarchical-Z state (main.c:230). */
MLV_API mlv_status mlv_create_texture2d(mlv_device device, const mlv_texture2d_desc *desc, const void *init_data,
                                        uint32_t row_pitch, mlv_texture2d *out_texture);
MLV_API mlv_status mlv_destroy_texture2d(mlv_texture2d texture);
/* New: a texture placed on caller-owned device memory (tightly packed rows, 16-byte aligned,
 * width * height * texel bytes long), left uninitialised and not freed by mlv_destroy_texture2d;
 * e.g. the per-view primitive-id targets of a batch laid out as one [views][height][width] array. */
MLV_API mlv_status mlv_create_texture2d_on_memory(mlv_device device, const mlv_texture2d_desc *desc,
                                                  void *device_memory, mlv_texture2d *out_texture);
/* Raw device addresses for zero-copy interop (e.g. wrapping a render target as a tensor). */
MLV_API mlv_status mlv_buffer_device_pointer(mlv_buffer buffer, void **out_ptr);
MLV_API mlv_status mlv_texture2d_device_pointer(mlv_texture2d texture, void **out_ptr);

/* Copies host data into a resource, ordered with the context's queued work. */
MLV_API mlv_status mlv_update_buffer(mlv_context context, mlv_buffer buffer, uint64_t offset, const void *data,
                                     uint64_t size);
MLV_API mlv_status mlv_update_texture2d(mlv_context context, mlv_texture2d texture, const void *data,
                                        uint32_t row_pitch);
/* New: the same copies queued without waiting (Direct3D 11 has no counterpart; compare a dynamic
 * resource's Map with NO_OVERWRITE). `data` must stay valid and unchanged until the context next
 * synchronises (mlv_finish, a readback, mlv_get_stats): with pinned host memory the copy runs in
 * the background. Queued work that was issued earlier (on the context's stream, by the library
 * or by the caller) still reads the old contents. The copy runs on the context's copy stream, and
 * later batches wait for it only at the stage that first reads the resource (vertex buffers and
 * VS textures at the vertex stage, index buffers at geometry, PS textures at the tile kernel), so
 * the later copies of a frame overlap its earlier stages. */
MLV_API mlv_status mlv_update_buffer_async(mlv_context context, mlv_buffer buffer, uint64_t offset,
                                           const void *data, uint64_t size);
MLV_API mlv_status mlv_update_texture2d_async(mlv_context context, mlv_texture2d texture, const void *data,
                                              uint32_t row_pitch);

/* New (no Direct3D 11 counterpart): several of those queued uploads from one block of host memory.
 * Each copy from host memory carries a fixed cost (about 5 us on the GB300's host link: a frame's 26
 * buffers and textures moved at 135 GB/s as separate copies, 209 GB/s as one), so the block goes to
 * the device in one copy, into a staging area of the context, and one kernel on the copy stream
 * places each range in its resource. Same ordering and lifetime rules as mlv_update_buffer_async;
 * every resource of the call is ready when the whole call is (one call per stage that reads the
 * resources lets a lone frame's earlier stages overlap the later copies; with frames pipelined, one
 * call for all was faster).
 * `src_offset` (into the block) and the destination (a buffer's `dst_offset`) must be multiples of
 * 16 bytes; a texture takes `size` = its width x height x texel bytes at `dst_offset` 0. */
typedef enum mlv_upload_kind { MLV_UPLOAD_BUFFER = 0, MLV_UPLOAD_TEXTURE2D = 1 } mlv_upload_kind;
typedef struct mlv_upload {
    uint32_t kind;          /* mlv_upload_kind */
    uint32_t pad;
    void *resource;         /* an mlv_buffer or an mlv_texture2d */
    uint64_t src_offset;    /* bytes into the block */
    uint64_t dst_offset;    /* bytes into the buffer (textures: 0) */
    uint64_t size;          /* bytes */
} mlv_upload;
MLV_API mlv_status mlv_update_resources_async(mlv_context context, const void *block, uint64_t block_bytes,
                                              const mlv_upload *uploads, uint32_t count);
/* Waits for the context's queued work, then copies the texture to host memory. */
MLV_API mlv_status mlv_read_texture2d(mlv_context context, mlv_texture2d texture, void *dst, uint32_t row_pitch);

/* ------------------------------------------------------------------ pipeline state (Pipeline, main.c:109-115) */

/* IA::primitive_topology (main.c:75) */
MLV_API mlv_status mlv_ia_set_primitive_topology(mlv_context context, mlv_primitive_topology topology);
/* IA::p_index_buffer (main.c:72); format must be MLV_FORMAT_R32_UINT, offset in bytes */
MLV_API mlv_status mlv_ia_set_index_buffer(mlv_context context, mlv_buffer buffer, mlv_format format,
                                           uint32_t offset);
/* IA::p_vertex_buffer and IA::input_layout (main.c:73-74); one slot; stride >= 32 bytes, the VS
 * reads the first 32 bytes of each vertex (main.c:684-691) */
MLV_API mlv_status mlv_ia_set_vertex_buffers(mlv_context context, uint32_t start_slot, uint32_t num_buffers,
                                             const mlv_buffer *buffers, const uint32_t *strides,
                                             const uint32_t *offsets);
/* VS::shader and VS::output_register_count (main.c:79-80, 1287-1288) */
MLV_API mlv_status mlv_vs_set_shader(mlv_context context, mlv_vertex_shader_id shader);
/* VS::p_constant_buffers (main.c:81, 1281) */
MLV_API mlv_status mlv_vs_set_constant_buffers(mlv_context context, uint32_t start_slot, uint32_t num_buffers,
                                               const mlv_buffer *buffers);
/* VS::p_shader_resource_views (main.c:82, 1293) */
MLV_API mlv_status mlv_vs_set_shader_resources(mlv_context context, uint32_t start_slot, uint32_t num_views,
                                               const mlv_texture2d *textures);
/* PS::shader (main.c:99, 1289) */
MLV_API mlv_status mlv_ps_set_shader(mlv_context context, mlv_pixel_shader_id shader);
/* PS::p_shader_resource_views (main.c:100, 1294) */
MLV_API mlv_status mlv_ps_set_shader_resources(mlv_context context, uint32_t start_slot, uint32_t num_views,
                                               const mlv_texture2d *textures);
/* RS::viewport (main.c:94-96, 1277-1278); one viewport */
MLV_API mlv_status mlv_rs_set_viewports(mlv_context context, uint32_t num_viewports, const mlv_viewport *viewports);
/* cull mode (the reference hard-codes back-face culling, main.c:856), fill rule and sample point */
MLV_API mlv_status mlv_rs_set_state(mlv_context context, const mlv_rasterizer_desc *desc);
/* depth function (the reference hard-codes GREATER_EQUAL, main.c:1166) */
MLV_API mlv_status mlv_om_set_depth_stencil_state(mlv_context context, const mlv_depth_stencil_desc *desc);
/* OM::p_colors, OM::p_depth (main.c:103-107, 1279-1280). The render target is
 * MLV_FORMAT_R8G8B8A8_UNORM, the depth target MLV_FORMAT_D32_FLOAT, of the same size. */
MLV_API mlv_status mlv_om_set_render_targets(mlv_context context, mlv_texture2d render_target,
                                             mlv_texture2d depth_stencil);
/* Optional visibility targets (new): for every pixel the last writer's triangle id (the index the
 * reference's primitive assembly gives it within its draw, main.c:873-875) in an R32_UINT texture,
 * its draw number within the bound render target's draws since the last clear in a second
 * R32_UINT texture, and its quantised barycentrics (b1, b2) (main.c:1092-1102) in an R32G32_FLOAT
 * texture. Pixels no draw wrote keep their values. Any of the three may be NULL. */
MLV_API mlv_status mlv_om_set_visibility_targets(mlv_context context, mlv_texture2d triangle_id,
                                                 mlv_texture2d draw_id, mlv_texture2d barycentrics);

/* ------------------------------------------------------------------ clears and draws */

/* clear_render_target_view, main.c:1191-1202 (R in the low byte, truncating) */
MLV_API mlv_status mlv_clear_render_target_view(mlv_context context, mlv_texture2d render_target,
                                                const float rgba[4]);
/* clear_depth_stencil_view, main.c:1204-1217: also resets the hierarchical-Z tile minima to 0
 * (and the tile maxima used by LESS to 1) */
MLV_API mlv_status mlv_clear_depth_stencil_view(mlv_context context, mlv_texture2d depth_stencil, float depth);
/* Fills a 32-bit-per-channel texture (e.g. a visibility target) with one value per channel. */
MLV_API mlv_status mlv_clear_texture_u32(mlv_context context, mlv_texture2d texture, uint32_t value);
/* draw_indexed, main.c:1219-1261; start_index_location and base_vertex_location are the
 * reference's TODO (main.c:1219). index_count need not be a multiple of 8 (main.c:670). */
MLV_API mlv_status mlv_draw_indexed(mlv_context context, uint32_t index_count, uint32_t start_index_location,
                                    int32_t base_vertex_location);
/* Non-indexed draw: vertex i of the draw is vertex start + i of the buffer. */
MLV_API mlv_status mlv_draw(mlv_context context, uint32_t vertex_count, uint32_t start_vertex_location);

/* ------------------------------------------------------------------ submission */

MLV_API mlv_status mlv_flush(mlv_context context);
/* Blocks until the context's work is done; reports device-side errors (overflows are handled by
 * regrowing buffers and re-running the affected work before returning). */
MLV_API mlv_status mlv_finish(mlv_context context);
MLV_API mlv_status mlv_finish_command_list(mlv_context deferred_context, mlv_command_list *out_list);
MLV_API mlv_status mlv_execute_command_list(mlv_context immediate_context, mlv_command_list list);
MLV_API mlv_status mlv_destroy_command_list(mlv_command_list list);
/* The CUDA stream (cudaStream_t) the context's work runs on. */
MLV_API mlv_status mlv_get_stream(mlv_context context, void **out_stream);

/* ------------------------------------------------------------------ statistics and tuning */

/* Stats, main.c:199-206, accumulated since the last reset (render() resets them per frame,
 * main.c:1268). Reading them synchronises. */
typedef struct mlv_stats {
    uint64_t vertex_count;
    uint64_t input_triangle_count;
    uint64_t assembled_triangle_count;
    uint64_t active_bin_count;
    uint64_t total_triangle_count_in_bins;
    uint64_t draw_count;
    uint64_t batch_count;
    uint64_t kernel_launches;
} mlv_stats;

MLV_API mlv_status mlv_get_stats(mlv_context context, mlv_stats *out_stats);
MLV_API mlv_status mlv_reset_stats(mlv_context context);

/* Launch-shape knobs of the tile kernel, picked by the autotuner (malevich_gb300/autotune.py).
 * The hierarchical-Z tile stays 8x8 pixels: it is observable (main.c:1005-1010). */
typedef struct mlv_tuning {
    uint32_t tile_warps_per_block;    /* warps per CTA of the tile kernel (one tile each): 2, 4 or 8 */
    uint32_t warps_per_tile;          /* 1, or 2, 4 or 8 warps sharing each tile's triangles (one tile per
                                         CTA; tile_warps_per_block is then not used): for frames whose
                                         triangles crowd into few tiles */
    uint32_t big_triangle_tiles;      /* triangles spanning more tiles are binned cooperatively */
    uint32_t geometry_block;          /* threads per CTA of the geometry kernel: 128, 256 or 512 */
    /* First sizes of the two buffers only the device can size (0 = automatic). When a batch needs
     * more, its render-target writes are skipped on the device and the next synchronisation
     * regrows the buffer and re-runs the batch, so these only trade memory for a re-run. */
    uint32_t initial_bin_entries;
    uint32_t initial_clip_fan_slots;
    /* A batch whose every view has exactly one draw, each of at most this many input triangles
     * (default: any number), with no triangle-id target and no TileInfo capture, takes the
     * small-draw path: three kernels instead of five, no binning, the vertex shader run per index
     * as the reference does. Same outputs; 0 disables it. */
    uint32_t small_draw_triangles;
    uint32_t debug_flags;             /* MLV_DEBUG_*: failure-detection tests only; 0 in normal use */
    /* 1: a batch on the binned path runs as one persistent launch instead of a kernel per stage
     * (vertex shading, geometry, clipping, bin scan, scatter, tiles): a grid of as many CTAs as the
     * GPU holds at once, with a grid-wide barrier between the stages. Same outputs. It uses 8 warps
     * (tiles) per CTA, or one tile per CTA shared by 8 warps when warps_per_tile > 1;
     * tile_warps_per_block and geometry_block do not apply. The stage timers count it as stage 4. */
    uint32_t persistent_launch;
} mlv_tuning;

/* The bin scan's first block never publishes its prefix, so the bounded waits of the blocks after
 * it run out: the batch writes nothing and the next synchronisation returns MLV_ERROR_TIMEOUT,
 * after which the context works again. Takes effect on batches with more than 16,384 bins that
 * use the binned path (a 1920x1080 target, for instance). */
#define MLV_DEBUG_STALL_LOOKBACK 0x1u
/* Persistent launch: its first CTA leaves before the first grid barrier, so the bounded waits of
 * all the others run out (shortened under this flag to milliseconds): the batch writes nothing and
 * the next synchronisation returns MLV_ERROR_TIMEOUT, after which the context works again. */
#define MLV_DEBUG_STALL_GRID 0x2u

MLV_API mlv_status mlv_get_tuning(mlv_context context, mlv_tuning *out_tuning);
MLV_API mlv_status mlv_set_tuning(mlv_context context, const mlv_tuning *tuning);

/* Per-stage device time (replaces the reference's Remotery CPU samples, main.c:663-1260).
 * When enabled, CUDA events bracket every stage on the context's stream; reading synchronises.
 * Stages: 0 clear, 1 geometry (IA + primitive assembly + bin count, and the vertex shader for
 * draws shaded per index), 2 bin scan, 3 bin scatter, 4 tile (raster+PS+OM), 5 vertex shading
 * (once per vertex). On the small-draw path (mlv_tuning::small_draw_triangles) stage 1 is the
 * raster kernel (vertex shader, setup and the small triangles' coverage and depth), 3 the queued
 * large triangles and 4 the resolve (PS + OM). Times in milliseconds, summed since the last reset. */
#define MLV_STAGE_COUNT 6
MLV_API mlv_status mlv_set_profiling(mlv_context context, int enable);
MLV_API mlv_status mlv_get_stage_times(mlv_context context, double *ms, uint64_t *launches);

/* Debug capture of the last executed single-draw batch: for every (8x8 tile, assembled triangle)
 * pair the draw binned, its 64-bit coverage mask after the hierarchical-Z test (TileInfo,
 * main.c:159-162; bit row*8+col). Entries are sorted by tile, then triangle. */
MLV_API mlv_status mlv_set_debug_capture(mlv_context context, int enable);
MLV_API mlv_status mlv_get_tile_infos(mlv_context context, uint32_t *tile_index, uint32_t *triangle_id,
                                      uint64_t *mask, uint64_t capacity, uint64_t *out_count);


/* ------------------------------------------------------------------ differentiable shading (new)
 * No reference counterpart: the reference's quantised barycentrics (main.c:1092-1102) have zero
 * gradient almost everywhere. These calls shade under a fixed visibility - the per-pixel input
 * triangle written by the rasteriser through mlv_om_set_primitive_id_target - with continuous
 * barycentrics at the reference's sample point (the pixel corner), for MLV_VS_PASSTHROUGH_UV-style
 * vertices: screen positions x, y in [0,1] (X = W x, Y = H (1 - y), w = 1), a colour and a UV per
 * vertex, and the pixel shader colour * bilinear(RGBA32F texture, uv).xyz.
 * A covered pixel whose continuous barycentrics are not all >= -1/8 is dropped (shades to 0, no
 * gradient): the 28.4 snap moves a vertex by at most 1/32 pixel, so only corners the snap pulled
 * into slivers under 1/4 pixel high are dropped, where the barycentrics extrapolate without bound.
 * mlv_diff_forward writes the image and the per-pixel barycentrics (the checkpoint);
 * mlv_diff_backward reads the checkpoint and grad_image = dL/dimage, recomputes the interpolation
 * and ADDS dL/dcolors, dL/dtexture (scattered through the bilinear weights) and dL/dpositions (the
 * barycentric terms, visibility fixed) into the gradient arrays it is given (any may be NULL).
 * All pointers are device memory (positions, uvs, barycentrics, grad_positions 8-byte aligned,
 * texture and grad_texture 16-byte);
 * both calls are asynchronous on `cuda_stream`; the backward needs the checkpoint of a forward
 * with the same positions. */
typedef struct mlv_diff_desc {
    uint32_t n_verts, n_tris;
    const uint32_t *index_buffer;     /* 3 * n_tris, each < n_verts (the kernels do not check) */
    const float *colors;              /* 3 * n_verts */
    const float *uvs;                 /* 2 * n_verts */
    const float *texture;             /* tex_height * tex_width * 4 */
    uint32_t tex_width, tex_height;
    uint32_t num_views, width, height;
    const float *positions;           /* num_views * n_verts * 2 */
    const uint32_t *primitive_ids;    /* num_views * height * width; 0xFFFFFFFF: background */
    float *barycentrics;              /* num_views * height * width * 2 (written by the forward;
                                         (-1, -1) marks a dropped pixel) */
    float *image;                     /* num_views * height * width * 3 (forward output) */
    const float *grad_image;          /* num_views * height * width * 3 (backward input) */
    float *grad_colors, *grad_texture, *grad_positions;
} mlv_diff_desc;

MLV_API mlv_status mlv_diff_forward(const mlv_diff_desc *desc, void *cuda_stream);
MLV_API mlv_status mlv_diff_backward(const mlv_diff_desc *desc, void *cuda_stream);
/* The visibility for the differentiable path: for every written pixel, the index (within its
 * draw) of the input triangle that wrote it (Direct3D's SV_PrimitiveID); R32_UINT, or NULL. */
MLV_API mlv_status mlv_om_set_primitive_id_target(mlv_context context, mlv_texture2d primitive_id);

/* ------------------------------------------------------------------ allocation-free draw
 * No counterpart in the reference: it is an addition for callers that cannot call cudaMalloc -
 * a host application that owns all device memory through its own allocator, a render loop whose
 * rule is no allocation after start-up, or code issuing work while another component of the
 * process captures a CUDA graph, where an allocation would be captured or refused. The call draws
 * one indexed (or, with index_buffer NULL, non-indexed) draw into caller-owned device memory with
 * the same results as mlv_draw_indexed (any shader pairing, MLV_PS_NONE included; no visibility
 * targets and the reference's fill rule and sample point). Its scratch (triangle records, bins, lists,
 * counters) is one static device array of MLV_NOALLOC_SCRATCH_BYTES that every GPU which loads
 * this library holds until the process exits; the call allocates nothing.
 *  - Limits: MLV_NOALLOC_MAX_TRIANGLES input triangles, MLV_NOALLOC_MAX_TILES 8x8 tiles in the
 *    render target (1024x1024 pixels), MLV_NOALLOC_MAX_CLIP_FANS clip-generated triangles and
 *    MLV_NOALLOC_MAX_BIN_ENTRIES (tile, triangle) pairs. Larger sizes are rejected with
 *    MLV_ERROR_CAPACITY_EXCEEDED (the last two are only known on the device: the call then
 *    returns that status and leaves the render target unwritten). Vertex buffers of more than
 *    MLV_NOALLOC_MAX_VERTICES vertices are shaded per index instead of once per vertex.
 *  - The first call on a device, with that device current, looks up the array's device address
 *    and loads constants; make that first call before any stream capture.
 *  - Every call shares the array and resets what must start at zero; calls that overlap on the
 *    GPU (on different streams, or from several threads) race on it and must not be issued.
 *  - The call waits for its stream before it returns, to report device-side overflows.
 *  - tile_min/tile_max are the depth target's hierarchical-Z state (float per 8x8 tile); pass
 *    MLV_NOALLOC_RESET_HIERARCHICAL_Z on the first draw after clearing the depth target. */
#define MLV_NOALLOC_MAX_TRIANGLES 32768u
#define MLV_NOALLOC_MAX_VERTICES 32768u
#define MLV_NOALLOC_MAX_TILES 16384u
#define MLV_NOALLOC_MAX_CLIP_FANS 8192u
#define MLV_NOALLOC_MAX_BIN_ENTRIES 131072u
#define MLV_NOALLOC_SCRATCH_BYTES 8849920u
#define MLV_NOALLOC_RESET_HIERARCHICAL_Z 0x1u

typedef struct mlv_noalloc_texture {
    const void *data;            /* device pointer, rows tightly packed */
    uint32_t width, height;
    mlv_format format;           /* R8G8B8A8_UNORM, R16G16B16A16_FLOAT or R32G32B32A32_FLOAT */
} mlv_noalloc_texture;

typedef struct mlv_noalloc_draw {
    const void *vertex_buffer;   /* device pointer to vertex_count vertices: the first 32 bytes of
                                    vertex vertex_count - 1, at (vertex_count - 1) * vertex_stride,
                                    must lie inside the allocation */
    uint32_t vertex_stride, vertex_count;
    const uint32_t *index_buffer;/* device pointer, or NULL for implicit indices */
    uint32_t index_buffer_count; /* 32-bit indices the index buffer holds; the call rejects
                                    start_index + index_count > index_buffer_count with
                                    MLV_ERROR_INVALID_ARG (ignored when index_buffer is NULL) */
    uint32_t index_count, start_index;
    int32_t base_vertex;
    mlv_vertex_shader_id vs;
    mlv_pixel_shader_id ps;
    const float *per_frame_cb;   /* host pointer to 48 floats (mlv_per_frame_cb), or NULL */
    mlv_noalloc_texture vs_texture, ps_texture;
    mlv_viewport viewport;
    mlv_cull_mode cull_mode;
    mlv_comparison_func depth_func;
    uint32_t *color;             /* device pointer, width*height render-target texels */
    float *depth;                /* device pointer, width*height */
    float *tile_min, *tile_max;  /* device pointers, ceil(width/8)*ceil(height/8) each */
    uint32_t width, height;
    uint32_t flags;              /* MLV_NOALLOC_RESET_HIERARCHICAL_Z */
} mlv_noalloc_draw;

/* cuda_stream: a cudaStream_t (NULL: the default stream). */
MLV_API mlv_status mlv_draw_indexed_noalloc(const mlv_noalloc_draw *draw, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif
