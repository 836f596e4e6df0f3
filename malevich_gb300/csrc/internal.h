// Internal data layout shared by the host runtime (api.cu) and the kernels (kernels.cu).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector_types.h>

#include "malevich.h"

namespace mlv {

constexpr int kTile = 8;                 // 8x8 pixel tiles: the reference's bins (main.c:24-25)
constexpr int kSubpix = 4;               // 28.4 fixed point (main.c:39)
constexpr int kPsNone = 5;               // MLV_PS_NONE: depth and visibility only
constexpr int kRasterTopLeft = 1;        // MLV_FILL_TOP_LEFT
constexpr int kRasterCenter = 2;         // MLV_SAMPLE_PIXEL_CENTER
constexpr int kDrawSharesView = 4;       // (DrawDesc::raster_flags) the view has other draws too
constexpr uint32_t kBinGhost = 0x80000000u;  // bin count bit: binned triangles without samples only
constexpr int kMaxClipVertices = 16;     // main.c:38
constexpr int kMaxViewsPerBatch = 4096;

// Error bits of the context's device status word.
enum : uint32_t {
    kErrLookbackTimeout = 1u << 0,
    kErrRecordOverflow = 1u << 1,
    kErrListOverflow = 1u << 2,
    kErrBigOverflow = 1u << 3,
    kErrBadIndex = 1u << 4,
    kErrQueueOverflow = 1u << 5,         // small-draw path: more large-triangle chunks than the queue holds
    kErrGridTimeout = 1u << 6,           // persistent launch: a grid barrier's bounded wait gave up
};

// Debug flags (mlv_tuning::debug_flags, MLV_DEBUG_*), for failure-detection tests only.
constexpr uint32_t kDebugStallLookback = 1u;
constexpr uint32_t kDebugStallGrid = 2u;     // persistent launch: CTA 0 leaves before the first grid barrier

struct TexDesc {
    const void *data;
    uint32_t width, height;
    int32_t format;                      // 1 RGBA8, 2 RGBA16F, 3 RGBA32F
    int32_t pad;
};

// One draw of a batch, as the kernels see it (the reference's Pipeline state at draw_indexed time).
struct DrawDesc {
    const uint8_t *vb;
    const uint32_t *ib;                  // nullptr: implicit indices
    uint32_t vb_stride, vertex_count;
    uint32_t start_index;
    int32_t base_vertex;
    uint32_t tri_begin;                  // first input triangle of this draw in the batch
    uint32_t tri_count;
    int32_t vs, ps, cull, depth_less;    // cull: 0 none, 1 back (reference), 2 front
    int32_t raster_flags;                // kRasterTopLeft | kRasterCenter (0: the reference) | kDrawSharesView
    uint32_t view;                       // view (render target + depth) index in the batch
    uint32_t draw_in_view;               // position among the view's draws in this batch
    uint32_t draw_seq;                   // draw number since the render target's last clear
    uint32_t vs_cached;                  // 1: vertices were shaded once by k_vertex into vs_out
    float cb[48];                        // PerFrameCB snapshot
    float screen_from_ndc[16];           // main.c:825-830, computed on the host as the reference does;
                                         // entries 1, 2, 4, 6, 8, 9, 12-14 are 0 and 15 is 1 (relied on)
    int32_t vp_w, vp_h;                  // (i32)viewport.width/height
    uint32_t vs_base, vs_count;          // this draw's range in vs_out (count 0 when not cached)
    TexDesc vs_tex, ps_tex;
};

struct ViewDesc {
    uint32_t *color;
    float *depth;
    float *tile_min, *tile_max;          // hierarchical Z per 8x8 tile
    uint32_t *vis_tri;                   // optional visibility outputs
    uint32_t *vis_draw;
    float *vis_bary;
    uint32_t *vis_prim;                  // input triangle index within its draw (differentiable path)
    uint32_t width, height, tiles_x, tiles_y;
    uint32_t tile_base;                  // first tile of this view in the batch's tile space
    uint32_t draw_begin, draw_count;     // the view's draws are contiguous in the draw array
    uint32_t bin_base;                   // bin of (tile t, draw d) = bin_base + t * draw_count + d
    // Clears folded into the tile kernel: a target the batch's segment cleared (and bound in this
    // view only) starts at its clear value in every tile, and every one of its pixels is written
    // once, instead of a separate fill (kClear* bits; the depth clear also resets hierarchical Z).
    uint32_t clear_flags;
    uint32_t clear_color, clear_tri, clear_draw, clear_prim, clear_bary;
    float clear_depth;
    uint32_t key_base;                   // small-draw path: the view's first pixel key in BatchParams::keys
};

constexpr uint32_t kClearColor = 1, kClearDepth = 2, kClearTri = 4, kClearDraw = 8, kClearPrim = 16,
                   kClearBary = 32;

// Per assembled triangle, read by the tile kernel for every (tile, triangle) pair: 64 bytes.
//   w0 = e0.a, e0.b, e0.c, e1.a      w1 = e1.b, e1.c, e2.a, e2.b
//   w2 = e2.c, inv_area, zbound, z0  w3 = z1, z2, box min (x | y << 16), box max (x | y << 16)
// The box is the reference's pixel box shrunk to the samples the triangle can cover. The slot of a
// clipped input triangle holds no record: its w0.x is the base of its fans' slots and w0.y, w0.z
// the fans' box shrinks (6 bits a fan), from which the reference's boxes are rebuilt for binning.
struct TriRaster {
    int4 w[4];
};

// Per assembled triangle, read once per shaded pixel: 80 bytes (kShadeFull float4s).
//   s0 = rw0, rw1, rw2, draw          s1..s3 = reg1 (xyzw) of vertices 0..2
//   s4 = reg2.x of vertices 0..2, pad
// In a batch whose pixel shaders read only U and V (basic_ps, or none), 48 bytes (kShadeUV):
//   s0 = rw0, rw1, rw2, draw          s1 = U of vertices 0..2, V of vertex 0
//   s2 = V of vertices 1 and 2, pad
// The records of a batch are BatchParams::shade_stride float4s apart; the workspace is sized for
// the full form.
struct TriShade {
    float4 s[5];
};
constexpr uint32_t kShadeFull = 5, kShadeUV = 3;

// Screen-space positions (reg0 after the viewport transform), for the differentiable path.
struct TriGeom {
    float x[3], y[3], z[3], w[3];
};

// One fill of a batched clear: n 32-bit words at p set to value; chunk_begin is the exclusive prefix
// of the jobs' chunk counts (kFillChunk words each), by which a block finds its job.
struct FillJob {
    uint32_t *p;
    uint64_t n;
    uint32_t value, chunk_begin;
};
constexpr uint32_t kFillChunk = 8192;

// One emitted triangle's share of the binner (main.c:924-962), rebuilt from its record's bounds
// where needed (never stored): its key and the bins of its tile rectangle,
// bin(x, y) = first_bin + y * row_stride + x * col_stride.
// One range of a grouped upload (mlv_update_resources_async): size bytes from staging + src to dst.
struct UploadJob {
    uint8_t *dst;
    uint64_t src, size;
};
constexpr uint32_t kUploadJobsPerLaunch = 64;
struct UploadJobs {
    UploadJob job[kUploadJobsPerLaunch];
};

struct BinJob {
    uint32_t key, first_bin, nx, ny;
    uint32_t col_stride, row_stride, pad0, pad1;
};

// Assembled triangles live in slots indexed by their input triangle g (draw-major across the
// batch): an unclipped triangle's record is slot g; the clip-fan triangles of a clipped input
// triangle live in an overflow region at slot total_tris + base + f (raw fan index f), with base
// stored in slot g. The 32-bit key (g << 3) | c, c = 0 for an unclipped triangle and f + 1 for
// fan f, orders triangles exactly as the reference's serial primitive assembly does
// (input triangle, then fan; main.c:751,797), with no compaction pass.
struct BatchParams {
    const DrawDesc *draws;
    const ViewDesc *views;
    uint32_t num_draws, num_views;
    uint32_t total_tris;                 // input triangles in the batch
    uint32_t total_tiles;                // sum of views' tiles
    uint32_t total_bins;                 // sum of views' tiles * draws
    uint32_t overflow_capacity;          // clip-fan slots after the total_tris primary slots
    uint32_t list_capacity;
    uint32_t big_tiles;                  // triangles spanning more tiles are binned by a whole block
    uint32_t batch_seq;
    uint32_t total_vertices;             // sum of vs_count
    uint32_t want_rank;                  // 1: compute assembled-triangle ranks (visibility, capture)
    float4 *vs_out;                      // [total_vertices] SV_POSITION, then [total_vertices][2] attributes:
                                         // reg1, (reg2.x, 0, 0, 0); with shade_stride kShadeUV,
                                         // [total_vertices] float2 (reg1.w, reg2.x) instead
    TriRaster *raster;                   // [total_tris + overflow_capacity]
    TriShade *shade;                     // records shade_stride float4s apart (see TriShade)
    uint32_t shade_stride;               // kShadeFull, or kShadeUV
    TriGeom *geom;                       // nullptr unless the geometry is kept
    uint16_t *tri_info;                  // [total_tris]: emitted-fan mask | clipped << 8
    uint2 *clip_list;                    // [total_tris]: (input triangle, draw) that k_geometry leaves to k_clip
    uint4 *jobs;                         // [jobs_capacity] bin jobs, one per triangle or fan with bins:
                                         // (key, first bin, nx | ny << 16, view), counted by kCtrJobs
    uint32_t jobs_capacity;              // = raster record slots
    uint32_t *rank;                      // [total_tris]: assembled triangles before g (exclusive)
    uint32_t *bin_count;                 // [total_bins], zero between batches
    uint32_t *bin_start;                 // [total_bins + 1]
    uint32_t *list;                      // [list_capacity] triangle keys, grouped by bin
    uint64_t *info_mask;                 // optional TileInfo capture, parallel to list
    unsigned long long *scan_status;     // decoupled look-back of k_rank: (epoch:30|flag:2) << 32 | value
    unsigned long long *scan_status2;    // decoupled look-back of k_scan
    uint32_t *counters;                  // see Counter
    unsigned long long *stats;           // device statistics, see StatSlot
    uint32_t *error;                     // [0] error bits, [1] first failing batch, [2] warnings,
                                         // [3] bin entries needed, [4] clip-fan slots needed,
                                         // [5] queue entries needed (small-draw path)
    uint32_t debug_flags;                // kDebug* (tests only)
    // small-draw path (one draw, no binning): per-pixel (depth, order) keys of the view, all zero
    // between draws; queued chunks of large triangles' pixel blocks
    unsigned long long *keys;            // [sum of the views' width * height]
    uint4 *queue;                        // [queue_capacity]: key, record slot, first tile, tiles
    uint32_t queue_capacity;
    uint32_t keys_only;                  // 1: the resolve needs no records (depth and ids from the keys)
    // 1 (a small-draw batch whose views fold no clear): the queue kernel lists the tiles the raster
    // kernel marked in `marked`, and the resolve visits only those (an unmarked tile owes nothing)
    uint32_t mark_list;
    uint32_t *marked;                    // [total_tiles]
};

enum Counter : int {
    kCtrRankTicket = 0, kCtrRankDone, kCtrRankEpoch,
    kCtrOverflow, kCtrQueue, kCtrClip, kCtrJobs, kCtrGrid, kCtrClaimGeometry, kCtrClaimTiles,
                                         // per batch (zeroed before each): clip-fan slots used;
                                         // small-draw queue entries used; triangles listed for
                                         // clipping (clip_list); bin jobs listed (jobs); arrivals at
                                         // the persistent launch's grid barriers; its geometry and
                                         // tile blocks claimed
    kCtrScanTicket, kCtrScanDone, kCtrScanEpoch,
    kCtrMarked, kCtrMarkedDone,          // small-draw batches with a marked-tile list: tiles listed (by
                                         // the queue kernel);
                                         // resolve CTAs finished (its last CTA zeroes both)
    kCtrCount = 16
};
constexpr int kCtrPerBatch = kCtrClaimTiles - kCtrOverflow + 1;

// Words of descriptors an eager batch passes in a kernel's parameter block (with the kernel's other
// parameters under the 4 KB limit): a batch of up to 9 draws of one view.
constexpr uint32_t kDescParamWords = 992;


// Statistics are staged per batch (slots kStat*) and added to the totals (kStat* + kStatTotal)
// by the tile kernel, which runs only for batches that completed; a batch that is re-run after
// an overflow is therefore counted once.
enum StatSlot : int {
    kStatAssembled = 0, kStatActiveBins, kStatBinEntries, kStatTotal = 4, kStatCount = 8
};

// ------------------------------------------------------------------ host-side draw set-up
// Shared by mlv_draw_indexed (api.cu) and mlv_draw_indexed_noalloc (noalloc.cu): both must plan a
// draw identically for their results to agree bit for bit.

// screen_from_ndc, main.c:825-830, with the reference's mixed float/double arithmetic.
inline void host_screen_from_ndc(const mlv_viewport &vp, float *m) {
    const float r[16] = {(float)(vp.width * 0.5), 0, 0, (float)(vp.width * 0.5 + vp.top_left_x),
                         0, (float)(-vp.height * 0.5), 0, (float)(vp.height * 0.5 + vp.top_left_y),
                         0, 0, vp.max_depth - vp.min_depth, vp.min_depth,
                         0, 0, 0, 1};
    memcpy(m, r, sizeof(r));
}

// The clipper's plane normals: v4f32_normalize (math.h:267-270) of the six planes of
// main.c:652-657, evaluated with the reference's float/double mix.
inline void host_clip_planes(float planes[6][4]) {
    static const float raw[6][4] = {{1, 0, 0, 1}, {-1, 0, 0, 1}, {0, 1, 0, 1}, {0, -1, 0, 1}, {0, 0, 1, 1}, {0, 0, -1, 1}};
    for (int p = 0; p < 6; ++p) {
        const float dot = raw[p][0] * raw[p][0] + raw[p][1] * raw[p][1] + raw[p][2] * raw[p][2] + raw[p][3] * raw[p][3];
        const float len = (float)std::sqrt((double)dot);
        const float inv = (float)(1.0 / (double)len);
        for (int k = 0; k < 4; ++k) planes[p][k] = raw[p][k] * inv;
    }
}

// Whether a draw's vertices are shaded once each (k_vertex) rather than once per index (the
// reference's way, main.c:673): when it is indexed and references most of its buffer. The outputs
// are identical either way; this only decides where the work goes.
inline bool host_shade_once(const void *index_buffer, uint32_t vertex_count, uint32_t tri_count) {
    return index_buffer != nullptr && vertex_count > 0 && tri_count > 0 &&
           (uint64_t)vertex_count <= 2ull * 3ull * tri_count;
}

}  // namespace mlv
