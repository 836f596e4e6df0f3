// An allocation-free draw entry point (mlv_draw_indexed_noalloc, include/malevich.h).
//
// Some callers cannot call cudaMalloc: a host application that owns all device memory through its
// own allocator and forbids libraries from allocating, a render loop with a no-allocation rule
// after start-up, or code that issues work while another part of the process is capturing a CUDA
// graph, where an allocation would be captured or rejected. This entry point draws with the same
// kernels as mlv_draw_indexed, but its scratch memory (triangle records, bin counts and lists,
// scan state, counters) is one file-scope device array that every GPU loading this library holds
// until the process exits. Inputs and outputs stay caller-owned device memory.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/malevich.h"
#include "internal.h"

namespace mlv {
void set_clip_planes(const float planes[6][4], cudaStream_t stream);
cudaError_t launch_fill_u32(uint32_t *p, size_t n, uint32_t value, const uint32_t *error, cudaStream_t stream);
cudaError_t launch_vertex(const BatchParams &bp, cudaStream_t stream);
cudaError_t launch_geometry(const BatchParams &bp, uint32_t block, int num_sms, cudaStream_t stream);
cudaError_t launch_scan(const BatchParams &bp, cudaStream_t stream);
cudaError_t launch_scatter(const BatchParams &bp, int num_sms, cudaStream_t stream);
cudaError_t launch_tile(const BatchParams &bp, uint32_t warps, uint32_t warps_per_tile, cudaStream_t stream);
void set_last_error(const std::string &msg);
}  // namespace mlv

using namespace mlv;

namespace {

// Limits of the scratch array (see the header).
constexpr uint32_t kMaxTriangles = MLV_NOALLOC_MAX_TRIANGLES;
constexpr uint32_t kMaxVertices = MLV_NOALLOC_MAX_VERTICES;     // shaded once each; more: per index
constexpr uint32_t kMaxTiles = MLV_NOALLOC_MAX_TILES;
constexpr uint32_t kMaxFanSlots = MLV_NOALLOC_MAX_CLIP_FANS;
constexpr uint32_t kMaxBinEntries = MLV_NOALLOC_MAX_BIN_ENTRIES;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Layout of the scratch array, in bytes from its start.
constexpr size_t kOffDraw = 0;
constexpr size_t kOffView = align256(kOffDraw + sizeof(DrawDesc));
constexpr size_t kOffCounters = align256(kOffView + sizeof(ViewDesc));
constexpr size_t kOffStats = align256(kOffCounters + sizeof(uint32_t) * kCtrCount);
constexpr size_t kOffError = align256(kOffStats + sizeof(unsigned long long) * kStatCount);
constexpr size_t kOffStatus = align256(kOffError + sizeof(uint32_t) * 8);
constexpr size_t kStatusWords = kMaxTiles / 4096 + 2;
constexpr size_t kOffBinCount = align256(kOffStatus + sizeof(unsigned long long) * kStatusWords);
constexpr size_t kOffBinStart = align256(kOffBinCount + sizeof(uint32_t) * (kMaxTiles + 1));
constexpr size_t kOffTriInfo = align256(kOffBinStart + sizeof(uint32_t) * (kMaxTiles + 1));
constexpr size_t kOffJobs = align256(kOffTriInfo + sizeof(uint16_t) * (kMaxTriangles + 1));
constexpr size_t kOffRaster = align256(kOffJobs + sizeof(uint4) * (kMaxTriangles + kMaxFanSlots));
constexpr size_t kOffShade = align256(kOffRaster + sizeof(TriRaster) * (kMaxTriangles + kMaxFanSlots));
constexpr size_t kOffVsOut = align256(kOffShade + sizeof(TriShade) * (kMaxTriangles + kMaxFanSlots));
constexpr size_t kOffList = align256(kOffVsOut + sizeof(float4) * 3 * kMaxVertices);
constexpr size_t kScratchBytes = align256(kOffList + sizeof(uint32_t) * kMaxBinEntries);
static_assert(kScratchBytes == MLV_NOALLOC_SCRATCH_BYTES, "header and layout disagree on the scratch size");
static_assert(kMaxBinEntries >= 2 * kMaxTriangles, "the clip list lives in the bin-list region");

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint8_t *g_scratch_ptr[kMaxDevices];   // device address of the scratch array, per device
int g_num_sms[kMaxDevices];

}  // namespace

// The scratch array. In host code this name is only a stand-in for the symbol: its device address
// comes from cudaGetSymbolAddress, once per device, in noalloc_setup below.
static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];

// Writes the draw and view descriptors (passed by value, so no host buffer is involved) and
// resets the scratch state that must start at zero: error words, counters, staged statistics,
// look-back status words and the bin counts.
__global__ void k_noalloc_reset(DrawDesc d, ViewDesc v, uint8_t *base, uint32_t bins) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *(DrawDesc *)(base + kOffDraw) = d;
        *(ViewDesc *)(base + kOffView) = v;
        uint32_t *err = (uint32_t *)(base + kOffError);
        for (int k = 0; k < 8; ++k) err[k] = k == 1 ? 0xFFFFFFFFu : 0u;
        uint32_t *ctr = (uint32_t *)(base + kOffCounters);
        for (int k = 0; k < kCtrCount; ++k) ctr[k] = 0;
        unsigned long long *st = (unsigned long long *)(base + kOffStats);
        for (int k = 0; k < kStatCount; ++k) st[k] = 0;
        unsigned long long *ss = (unsigned long long *)(base + kOffStatus);
        for (size_t k = 0; k < kStatusWords; ++k) ss[k] = 0;
    }
    uint32_t *bc = (uint32_t *)(base + kOffBinCount);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= bins; i += gridDim.x * blockDim.x) bc[i] = 0;
}

namespace {

// First call on a device, with that device current: look up the scratch array's device address
// and load the clipper's plane constants. Synchronous; must run before any stream capture.
mlv_status noalloc_setup(int dev, uint8_t **out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_error("device ordinal out of range for the allocation-free path");
        return MLV_ERROR_INVALID_ARG;
    }
    if (!g_scratch_ptr[dev]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            set_last_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
            return MLV_ERROR_DEVICE;
        }
        float planes[6][4];
        host_clip_planes(planes);
        set_clip_planes(planes, 0);
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            set_last_error(std::string("allocation-free set-up: ") + cudaGetErrorString(e));
            return MLV_ERROR_DEVICE;
        }
        cudaDeviceGetAttribute(&g_num_sms[dev], cudaDevAttrMultiProcessorCount, dev);
        g_scratch_ptr[dev] = (uint8_t *)ptr;
    }
    *out = g_scratch_ptr[dev];
    return MLV_OK;
}

mlv_status fail_na(mlv_status st, const char *msg) {
    set_last_error(msg);
    return st;
}

TexDesc tex_of(const mlv_noalloc_texture &t) {
    TexDesc d = {};
    d.data = t.data;
    d.width = t.width;
    d.height = t.height;
    d.format = t.format == MLV_FORMAT_R8G8B8A8_UNORM ? 1 : t.format == MLV_FORMAT_R16G16B16A16_FLOAT ? 2 : 3;
    return d;
}

bool tex_valid(const mlv_noalloc_texture &t, bool want_float, bool any) {
    if (!t.data || !t.width || !t.height) return false;
    const bool f = t.format == MLV_FORMAT_R32G32B32A32_FLOAT || t.format == MLV_FORMAT_R16G16B16A16_FLOAT;
    const bool u8 = t.format == MLV_FORMAT_R8G8B8A8_UNORM;
    return any ? (f || u8) : (want_float ? f : u8);
}

}  // namespace

#define NA_CUDA(expr)                                                                    \
    do {                                                                                 \
        cudaError_t _e = (expr);                                                         \
        if (_e != cudaSuccess) {                                                         \
            set_last_error(std::string(#expr) + ": " + cudaGetErrorString(_e));          \
            return MLV_ERROR_DEVICE;                                                     \
        }                                                                                \
    } while (0)

extern "C" MLV_API mlv_status mlv_draw_indexed_noalloc(const mlv_noalloc_draw *a, void *cuda_stream) {
    if (!a) return fail_na(MLV_ERROR_INVALID_ARG, "draw is NULL");
    // ---- validation against the scratch limits and the pipeline rules of mlv_draw_indexed
    if (!a->color || !a->depth || !a->tile_min || !a->tile_max || !a->vertex_buffer)
        return fail_na(MLV_ERROR_INVALID_ARG, "color, depth, tile_min, tile_max and vertex_buffer are required");
    if (a->width == 0 || a->height == 0 || a->width > 16384 || a->height > 16384)
        return fail_na(MLV_ERROR_INVALID_ARG, "render target size must be 1..16384");
    const uint32_t tiles_x = (a->width + kTile - 1) / kTile, tiles_y = (a->height + kTile - 1) / kTile;
    if ((uint64_t)tiles_x * tiles_y > kMaxTiles)
        return fail_na(MLV_ERROR_CAPACITY_EXCEEDED, "render target has more 8x8 tiles than MLV_NOALLOC_MAX_TILES");
    const uint32_t tris = a->index_count / 3;
    if (tris > kMaxTriangles)
        return fail_na(MLV_ERROR_CAPACITY_EXCEEDED, "draw has more triangles than MLV_NOALLOC_MAX_TRIANGLES");
    if (a->vertex_stride < 32 || (a->vertex_stride & 3))
        return fail_na(MLV_ERROR_INVALID_ARG, "vertex stride must be >= 32 and a multiple of 4");
    if (a->vs < MLV_VS_BASIC || a->vs > MLV_VS_PASSTHROUGH_UV || a->ps < MLV_PS_BASIC || a->ps > MLV_PS_NONE)
        return fail_na(MLV_ERROR_INVALID_ARG, "unknown shader");
    // the kernels read indices start_index .. start_index + index_count - 1 (as mlv_draw_indexed
    // checks against its bound index buffer)
    if (a->index_buffer && (uint64_t)a->start_index + a->index_count > a->index_buffer_count)
        return fail_na(MLV_ERROR_INVALID_ARG, "draw reads past the index buffer (index_buffer_count)");
    if ((a->vs == MLV_VS_BASIC || a->vs == MLV_VS_VERTEX_LIGHTING || a->vs == MLV_VS_FULLSCREEN) && !a->per_frame_cb)
        return fail_na(MLV_ERROR_INVALID_ARG, "this vertex shader needs per_frame_cb");
    if (a->vs == MLV_VS_VERTEX_LIGHTING && !tex_valid(a->vs_texture, true, false))
        return fail_na(MLV_ERROR_INVALID_ARG, "vertex_lighting_vs needs a float texture");
    if (a->ps == MLV_PS_BASIC && !tex_valid(a->ps_texture, false, false))
        return fail_na(MLV_ERROR_INVALID_ARG, "basic_ps needs an R8G8B8A8 texture");
    if (a->ps == MLV_PS_ENV_LIGHTING && !tex_valid(a->ps_texture, true, false))
        return fail_na(MLV_ERROR_INVALID_ARG, "env_lighting_ps needs a float texture");
    if (a->ps == MLV_PS_COLOR_TIMES_TEXEL && !tex_valid(a->ps_texture, false, true))
        return fail_na(MLV_ERROR_INVALID_ARG, "COLOR_TIMES_TEXEL needs a texture");
    const mlv_viewport &vp = a->viewport;
    if (!(vp.width >= 1.0f && vp.height >= 1.0f) || vp.width > (float)a->width || vp.height > (float)a->height ||
        vp.top_left_x != 0.0f || vp.top_left_y != 0.0f)
        return fail_na(MLV_ERROR_INVALID_ARG, "the viewport must start at (0,0) and fit in the render target");
    int cull;
    switch (a->cull_mode) {
        case MLV_CULL_NONE: cull = 0; break;
        case MLV_CULL_BACK: cull = 1; break;
        case MLV_CULL_FRONT: cull = 2; break;
        default: return fail_na(MLV_ERROR_INVALID_ARG, "unknown cull mode");
    }
    if (a->depth_func != MLV_COMPARISON_LESS && a->depth_func != MLV_COMPARISON_GREATER_EQUAL)
        return fail_na(MLV_ERROR_INVALID_ARG, "depth function must be LESS or GREATER_EQUAL");

    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    uint8_t *base = nullptr;
    mlv_status st = noalloc_setup(dev, &base);
    if (st != MLV_OK) return st;
    cudaStream_t stream = (cudaStream_t)cuda_stream;

    // ---- the draw, as mlv_draw_indexed plans it (one view, one draw)
    DrawDesc d;
    memset(&d, 0, sizeof(d));
    d.vb = (const uint8_t *)a->vertex_buffer;
    d.ib = (const uint32_t *)a->index_buffer;
    d.vb_stride = a->vertex_stride;
    d.vertex_count = a->vertex_count;
    d.start_index = a->start_index;
    d.base_vertex = a->index_buffer ? a->base_vertex : 0;
    d.tri_begin = 0;
    d.tri_count = tris;
    d.vs = a->vs;
    d.ps = a->ps;
    d.cull = cull;
    d.depth_less = a->depth_func == MLV_COMPARISON_LESS ? 1 : 0;
    d.view = 0;
    d.draw_in_view = 0;
    d.draw_seq = 0;
    if (a->per_frame_cb) memcpy(d.cb, a->per_frame_cb, sizeof(d.cb));
    host_screen_from_ndc(vp, d.screen_from_ndc);
    d.vp_w = (int32_t)vp.width;
    d.vp_h = (int32_t)vp.height;
    // shaded once per vertex under the same rule as mlv_draw_indexed, while the vertices fit the
    // scratch array's shaded-vertex area (beyond that, per index: same outputs)
    d.vs_cached = (host_shade_once(d.ib, d.vertex_count, tris) && d.vertex_count <= kMaxVertices) ? 1u : 0u;
    d.vs_base = 0;
    d.vs_count = d.vs_cached ? d.vertex_count : 0;
    d.vs_tex = tex_of(a->vs_texture);
    d.ps_tex = tex_of(a->ps_texture);

    ViewDesc v;
    memset(&v, 0, sizeof(v));
    v.color = (uint32_t *)a->color;
    v.depth = (float *)a->depth;
    v.tile_min = (float *)a->tile_min;
    v.tile_max = (float *)a->tile_max;
    v.width = a->width;
    v.height = a->height;
    v.tiles_x = tiles_x;
    v.tiles_y = tiles_y;
    v.tile_base = 0;
    v.draw_begin = 0;
    v.draw_count = 1;
    v.bin_base = 0;

    BatchParams bp;
    memset(&bp, 0, sizeof(bp));
    bp.draws = (const DrawDesc *)(base + kOffDraw);
    bp.views = (const ViewDesc *)(base + kOffView);
    bp.num_draws = 1;
    bp.num_views = 1;
    bp.total_tris = tris;
    bp.total_tiles = tiles_x * tiles_y;
    bp.total_bins = tiles_x * tiles_y;
    bp.overflow_capacity = kMaxFanSlots;
    bp.list_capacity = kMaxBinEntries;
    bp.big_tiles = 16;
    bp.batch_seq = 1;
    bp.total_vertices = d.vs_count;
    bp.vs_out = (float4 *)(base + kOffVsOut);
    bp.raster = (TriRaster *)(base + kOffRaster);
    bp.shade = (TriShade *)(base + kOffShade);
    bp.shade_stride = kShadeFull;
    bp.tri_info = (uint16_t *)(base + kOffTriInfo);
    bp.jobs = (uint4 *)(base + kOffJobs);
    bp.jobs_capacity = kMaxTriangles + kMaxFanSlots;
    bp.bin_count = (uint32_t *)(base + kOffBinCount);
    bp.bin_start = (uint32_t *)(base + kOffBinStart);
    bp.list = (uint32_t *)(base + kOffList);
    // the list is written only by k_scatter, after k_clip is done with the clip list it holds
    // (MLV_NOALLOC_MAX_BIN_ENTRIES words hold MLV_NOALLOC_MAX_TRIANGLES entries of two)
    bp.clip_list = (uint2 *)(base + kOffList);
    bp.scan_status2 = (unsigned long long *)(base + kOffStatus);
    bp.counters = (uint32_t *)(base + kOffCounters);
    bp.stats = (unsigned long long *)(base + kOffStats);
    bp.error = (uint32_t *)(base + kOffError);

    // ---- the array keeps the last call's contents: reset what must start at zero
    k_noalloc_reset<<<16, 256, 0, stream>>>(d, v, base, bp.total_bins);
    NA_CUDA(cudaGetLastError());
    if (a->flags & MLV_NOALLOC_RESET_HIERARCHICAL_Z) {
        // as clear_depth_stencil_view leaves them: tile minima 0 (main.c:1212-1214), maxima 1
        NA_CUDA(launch_fill_u32((uint32_t *)a->tile_min, bp.total_tiles, 0u, nullptr, stream));
        NA_CUDA(launch_fill_u32((uint32_t *)a->tile_max, bp.total_tiles, 0x3F800000u, nullptr, stream));
    }
    if (tris) {
        NA_CUDA(launch_vertex(bp, stream));
        NA_CUDA(launch_geometry(bp, 128, g_num_sms[dev] ? g_num_sms[dev] : 152, stream));
        NA_CUDA(launch_scan(bp, stream));
        NA_CUDA(launch_scatter(bp, g_num_sms[dev] ? g_num_sms[dev] : 152, stream));
        NA_CUDA(launch_tile(bp, 4, 1, stream));
    }
    // ---- wait, then report what only the device knows
    uint32_t err[8] = {0};
    NA_CUDA(cudaMemcpyAsync(err, base + kOffError, sizeof(err), cudaMemcpyDeviceToHost, stream));
    NA_CUDA(cudaStreamSynchronize(stream));
    if (err[0] & kErrLookbackTimeout) return fail_na(MLV_ERROR_TIMEOUT, "a bounded device-side wait gave up");
    if (err[0] & kErrRecordOverflow)
        return fail_na(MLV_ERROR_CAPACITY_EXCEEDED,
                       "more clip-fan triangles than MLV_NOALLOC_MAX_CLIP_FANS; the render target was not written");
    if (err[0] & kErrListOverflow)
        return fail_na(MLV_ERROR_CAPACITY_EXCEEDED,
                       "more (tile, triangle) pairs than MLV_NOALLOC_MAX_BIN_ENTRIES; the render target was not written");
    if (err[2]) set_last_error("the draw read vertices outside its vertex buffer (zeros were used)");
    return MLV_OK;
}
