// Host runtime behind include/malevich.h: devices, contexts, resources, pipeline state, batch
// planning, workspace management, command lists (CUDA graphs) and error reporting.
//
// The reference keeps its pipeline state in one global struct (source/main.c:109-115,222) and
// mallocs/frees every stage buffer per draw (main.c:675,705,745-746,947,965,986,1253-1259).
// Here a context owns its state and a workspace that only grows; all buffers are sized on the
// host before launch. Capacities that only the device knows (assembled triangles, bin entries)
// are checked by the kernels: on overflow the later kernels of the batch skip their work, the
// render targets stay untouched, and the next synchronisation regrows the workspace and re-runs
// the affected batches.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/malevich.h"
#include "internal.h"

namespace mlv {
void set_clip_planes(const float planes[6][4], cudaStream_t stream);
cudaError_t launch_fill_u32(uint32_t *p, size_t n, uint32_t value, const uint32_t *error, cudaStream_t stream);
cudaError_t launch_fill_many(const FillJob *d_jobs, uint32_t njobs, uint32_t nchunks, const uint32_t *error,
                             cudaStream_t stream);
cudaError_t launch_vertex(const BatchParams &bp, cudaStream_t stream);
cudaError_t launch_geometry(const BatchParams &bp, uint32_t block, int num_sms, cudaStream_t stream);
cudaError_t launch_upload_scatter(const uint8_t *staging, const UploadJobs &jobs, uint32_t njobs, uint64_t max_size,
                                  int num_sms, cudaStream_t stream);
cudaError_t launch_scan(const BatchParams &bp, cudaStream_t stream);
cudaError_t launch_rank(const BatchParams &bp, cudaStream_t stream);
cudaError_t launch_scatter(const BatchParams &bp, int num_sms, cudaStream_t stream);
cudaError_t launch_tile(const BatchParams &bp, uint32_t warps, uint32_t warps_per_tile, cudaStream_t stream);
cudaError_t launch_persistent(const BatchParams &bp, uint32_t warps_per_tile, int num_sms, cudaStream_t stream);
cudaError_t launch_direct_raster(const BatchParams &bp, int num_sms, cudaStream_t stream);
cudaError_t launch_direct_queue(const BatchParams &bp, int num_sms, cudaStream_t stream);
cudaError_t launch_direct_resolve(const BatchParams &bp, int num_sms, cudaStream_t stream);
cudaError_t launch_put_descriptors(const void *a, uint32_t a_bytes, void *dst_a, const void *b, uint32_t b_bytes,
                                   void *dst_b, cudaStream_t stream);
}  // namespace mlv

using namespace mlv;

// ------------------------------------------------------------------ errors

static thread_local std::string g_last_error = "no error";

static mlv_status fail(mlv_status st, const std::string &msg) {
    g_last_error = msg;
    return st;
}

namespace mlv {
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace mlv

#define CUDA_TRY(expr)                                                                               \
    do {                                                                                             \
        cudaError_t _e = (expr);                                                                     \
        if (_e != cudaSuccess)                                                                       \
            return fail(_e == cudaErrorMemoryAllocation ? MLV_ERROR_OUT_OF_MEMORY : MLV_ERROR_DEVICE, \
                        std::string(#expr) + ": " + cudaGetErrorString(_e));                         \
    } while (0)

#define MLV_TRY(expr)                   \
    do {                                \
        mlv_status _s = (expr);         \
        if (_s != MLV_OK) return _s;    \
    } while (0)

// ------------------------------------------------------------------ objects

struct mlv_context_t;

struct mlv_device_t {
    int ordinal = 0;
    int num_sms = 0;
    float clip_planes[6][4];
    mlv_context_t *immediate = nullptr;
    std::vector<mlv_context_t *> deferred;   // live deferred contexts (guarded by mu)
    std::mutex mu;
    // bumped when a resource gets its upload event (first queued upload): captured command lists
    // re-capture, so that their graphs wait for it
    std::atomic<uint64_t> upload_generation{0};
};

struct mlv_buffer_t {
    mlv_device device = nullptr;
    uint8_t *ptr = nullptr;
    uint64_t size = 0;
    uint32_t bind = 0;
    std::vector<uint8_t> shadow;   // host copy of constant buffers (snapshotted at draw time)
    cudaEvent_t ready = nullptr;   // recorded after its last queued upload (copy stream)
};

struct mlv_texture2d_t {
    mlv_device device = nullptr;
    uint8_t *ptr = nullptr;
    uint32_t width = 0, height = 0;
    mlv_format format = MLV_FORMAT_UNKNOWN;
    uint32_t bind = 0;
    uint32_t texel_bytes = 0;
    float *tile_min = nullptr, *tile_max = nullptr;   // hierarchical Z (depth textures)
    uint32_t tiles_x = 0, tiles_y = 0;
    uint32_t draws_since_clear = 0;                    // render targets: numbers draws for visibility
    bool owns_memory = true;                           // false: placed on caller memory
    cudaEvent_t ready = nullptr;                       // recorded after its last queued upload
};

static uint32_t texel_bytes(mlv_format f) {
    switch (f) {
        case MLV_FORMAT_R8G8B8A8_UNORM: return 4;
        case MLV_FORMAT_R16G16B16A16_FLOAT: return 8;
        case MLV_FORMAT_R32G32B32A32_FLOAT: return 16;
        case MLV_FORMAT_D32_FLOAT: return 4;
        case MLV_FORMAT_R32_UINT: return 4;
        case MLV_FORMAT_R32G32_FLOAT: return 8;
        default: return 0;
    }
}

struct PipelineState {
    mlv_buffer ib = nullptr;
    uint32_t ib_offset = 0;
    mlv_buffer vb = nullptr;
    uint32_t vb_stride = 0, vb_offset = 0;
    int vs = 0, ps = 0;
    mlv_buffer vs_cb[MLV_CONSTANT_BUFFER_SLOT_COUNT] = {};
    mlv_texture2d vs_srv[MLV_SHADER_RESOURCE_SLOT_COUNT] = {};
    mlv_texture2d ps_srv[MLV_SHADER_RESOURCE_SLOT_COUNT] = {};
    mlv_viewport viewport = {0, 0, 0, 0, 0, 1};
    bool viewport_set = false;
    int cull = 1;          // internal: 0 none, 1 back, 2 front
    int raster_flags = 0;  // kRasterTopLeft | kRasterCenter
    int depth_less = 0;
    mlv_texture2d rtv = nullptr, dsv = nullptr;
    mlv_texture2d vis_tri = nullptr, vis_draw = nullptr, vis_bary = nullptr, vis_prim = nullptr;
    mlv_primitive_topology topology = MLV_PRIMITIVE_TOPOLOGY_TRIANGLELIST;
};

struct DrawCmd {
    DrawDesc desc;                 // view / draw_in_view / tri_begin filled by the planner
    mlv_texture2d rtv, dsv, vis_tri, vis_draw, vis_bary, vis_prim;
    uint32_t index_count;
    // the inputs, for the waits on their queued uploads (see Plan)
    mlv_buffer vb_res = nullptr, ib_res = nullptr;
    mlv_texture2d vs_res = nullptr, ps_res = nullptr;
};

struct ClearCmd {
    mlv_texture2d target;
    int kind;                      // 0 colour, 1 depth, 2 u32 fill
    uint32_t value;
    float depth;
};

// A segment: clears, then draws that no clear of the segment follows on the same target.
struct Segment {
    std::vector<ClearCmd> clears;
    std::vector<DrawCmd> draws;
    uint64_t input_triangles = 0, vertex_count = 0;
};

struct Workspace {
    TriRaster *raster = nullptr;
    TriShade *shade = nullptr;
    TriGeom *geom = nullptr;
    uint32_t record_cap = 0;          // slots: input triangles + clip-fan overflow
    uint32_t overflow_cap = 0;        // overflow slots the last sizing reserved
    bool keep_geom = false;
    uint16_t *tri_info = nullptr;
    uint4 *jobs = nullptr;
    uint2 *clip_list = nullptr;       // [clip_cap]
    uint32_t clip_cap = 0;
    uint32_t *rank = nullptr;
    uint32_t tri_cap = 0;
    uint32_t *bin_count = nullptr, *bin_start = nullptr;
    uint32_t bin_cap = 0;
    uint32_t *list = nullptr;
    uint64_t *info_mask = nullptr;
    uint32_t list_cap = 0;
    unsigned long long *scan_status = nullptr, *scan_status2 = nullptr;
    uint32_t status_cap = 0, status2_cap = 0;
    uint32_t *counters = nullptr;
    unsigned long long *stats = nullptr;
    uint32_t *error = nullptr;
    DrawDesc *d_draws = nullptr;
    ViewDesc *d_views = nullptr;
    uint32_t desc_draw_cap = 0, desc_view_cap = 0;
    FillJob *d_fills = nullptr;
    uint32_t fill_cap = 0;
    float4 *vs_out = nullptr;
    uint32_t vs_cap = 0;
    // small-draw path: the view's per-pixel keys (zero between draws) and the large-triangle queue
    unsigned long long *keys = nullptr;
    uint32_t keys_cap = 0;
    uint32_t *marked = nullptr;       // [marked_cap]: small-draw path, the tiles a batch marked
    uint32_t marked_cap = 0;
    uint4 *queue = nullptr;
    uint32_t queue_cap = 0;
    uint64_t generation = 0;
};

struct mlv_command_list_t {
    mlv_device device = nullptr;
    std::vector<Segment> segments;
    // graph replay state
    cudaGraphExec_t exec = nullptr;
    uint64_t exec_generation = ~0ull, exec_tuning = ~0ull, exec_uploads = ~0ull;
    mlv_context_t *exec_context = nullptr;
    int executions = 0;
    // what the descriptors in d_draws/d_views/d_fills were planned for: a tuning change can move
    // the list to the other path, whose descriptors differ
    uint64_t desc_tuning = ~0ull;
    mlv_context_t *desc_context = nullptr;
    bool desc_capture = false;
    DrawDesc *d_draws = nullptr;   // per-segment descriptor copies owned by the list
    ViewDesc *d_views = nullptr;
    FillJob *d_fills = nullptr;    // per-segment batched clears
    std::vector<size_t> draw_off, view_off, fill_off;
    size_t draws_total = 0, views_total = 0, fills_total = 0;
    uint64_t launches_per_execution = 0;
};

struct PendingJob {
    const Segment *segment;        // immediate segments are owned by `owned`
    std::shared_ptr<Segment> owned;
    mlv_command_list list;         // or a command list executed as a whole
    uint32_t seq;
};

// Batches of one draw per view take the small-draw path by default whatever their draws' sizes:
// it measured faster than the binned path both on the 20,480-triangle single draw and on the
// 256-view, 51M-triangle visibility pass.
constexpr uint32_t kDefaultSmallDraw = 0xFFFFFFFFu;

struct mlv_context_t {
    mlv_device device = nullptr;
    bool deferred = false;
    cudaStream_t stream = nullptr;
    PipelineState st;
    std::vector<Segment> recorded;     // deferred contexts
    Workspace ws;
    mlv_tuning tuning = {4, 1, 16, 128, 0, 0, kDefaultSmallDraw, 0, 0};   // measured defaults; the autotuner refines them
    uint64_t tuning_generation = 0;    // bumped by mlv_set_tuning: captured graphs re-capture
    uint64_t host_stats[8] = {};       // vertex_count, input triangles, draws, batches, launches
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    size_t ev_next = 0;
    double stage_ms[MLV_STAGE_COUNT] = {};
    uint64_t stage_launches[MLV_STAGE_COUNT] = {};
    bool capture_infos = false;
    bool capturing_graph = false;
    uint32_t batch_seq = 0;
    std::vector<PendingJob> pending;
    uint32_t *h_error = nullptr;       // pinned mirror of the device error words + counters
    // queued uploads run on their own stream, so that a batch's kernels wait only for the inputs
    // they read, when they read them (vertex buffers and VS textures before the vertex stage,
    // index buffers before geometry, PS textures before the tile kernel)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t work_mark = nullptr;   // the context stream's work so far, which uploads follow
    uint8_t *upload_staging = nullptr; // grouped uploads (mlv_update_resources_async) land here first
    uint64_t upload_staging_cap = 0;
    // last single-draw segment, for mlv_get_tile_infos
    bool last_single = false;
    uint32_t last_total_bins = 0, last_tiles_x = 0, last_draw_count = 0;
    uint32_t last_tris = 0;
};

// ------------------------------------------------------------------ small helpers

static mlv_status dev_alloc(void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return fail(MLV_ERROR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return MLV_OK;
}

// Zeroes device memory and waits for it: cudaMemset runs on the legacy default stream, which the
// library's non-blocking streams do not wait for, so work queued next (a graph captured right
// after a workspace grows, a first batch) could otherwise read the old contents.
static cudaError_t zero_now(void *p, size_t bytes) {
    cudaError_t e = cudaMemset(p, 0, bytes);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(cudaStreamLegacy);
}

// The same for a copy from (pageable) host memory: cudaMemcpy may return once the data is staged,
// before it reaches the device.
static cudaError_t copy_to_device_now(void *dst, const void *src, size_t bytes) {
    cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(cudaStreamLegacy);
}

template <class T>
static mlv_status grow(T **p, uint32_t &cap, uint64_t need, uint64_t elem = sizeof(T), bool zero = false) {
    if (need <= cap && *p) return MLV_OK;
    uint64_t n = std::max<uint64_t>(need, 1024);
    n = std::max<uint64_t>(n, (uint64_t)cap + cap / 2);
    if (n > 0xFFFFFFF0ull) n = 0xFFFFFFF0ull;
    if (need > n) return fail(MLV_ERROR_CAPACITY_EXCEEDED, "workspace larger than 2^32 elements");
    if (*p) cudaFree(*p);
    *p = nullptr;
    MLV_TRY(dev_alloc((void **)p, n * elem));
    if (zero) CUDA_TRY(zero_now(*p, n * elem));
    cap = (uint32_t)n;
    return MLV_OK;
}

static mlv_status set_device(mlv_device d) {
    CUDA_TRY(cudaSetDevice(d->ordinal));
    return MLV_OK;
}

static TexDesc tex_desc(mlv_texture2d t) {
    TexDesc d = {};
    if (!t) return d;
    d.data = t->ptr;
    d.width = t->width;
    d.height = t->height;
    d.format = t->format == MLV_FORMAT_R8G8B8A8_UNORM ? 1 : t->format == MLV_FORMAT_R16G16B16A16_FLOAT ? 2 : 3;
    return d;
}

// ------------------------------------------------------------------ workspace

// error words: [0] error bits, [1] first failing batch number (min), [2] warnings, [3] bin
// entries a list overflow needed, [4] clip-fan slots a record overflow needed
static mlv_status reset_error_words(Workspace &w) {
    const uint32_t init[8] = {0, 0xFFFFFFFFu, 0, 0, 0, 0, 0, 0};
    CUDA_TRY(copy_to_device_now(w.error, init, sizeof(init)));
    return MLV_OK;
}

static mlv_status ensure_fixed(mlv_context_t *c) {
    Workspace &w = c->ws;
    if (!w.counters) {
        MLV_TRY(dev_alloc((void **)&w.counters, sizeof(uint32_t) * kCtrCount));
        MLV_TRY(dev_alloc((void **)&w.stats, sizeof(unsigned long long) * kStatCount));
        MLV_TRY(dev_alloc((void **)&w.error, sizeof(uint32_t) * 8));
        CUDA_TRY(zero_now(w.counters, sizeof(uint32_t) * kCtrCount));
        CUDA_TRY(zero_now(w.stats, sizeof(unsigned long long) * kStatCount));
        MLV_TRY(reset_error_words(w));
        CUDA_TRY(cudaMallocHost((void **)&c->h_error, sizeof(uint32_t) * 32));
        memset(c->h_error, 0, sizeof(uint32_t) * 32);
    }
    return MLV_OK;
}

struct BatchSizes {
    uint64_t tris = 0, overflow = 0, bins = 0, tiles = 0, draws = 0, views = 0, vertices = 0;
    uint64_t direct_pixels = 0;   // small-draw path: the view's pixels (one key each)
    bool binned = false;  // some batch takes the binned path: bin jobs and the clip list are needed
    bool shade = false;   // some draw has a pixel shader: the 80-byte shading records are needed
};

static mlv_status reset_scan_state(Workspace &w) {
    // fresh look-back state: every status word "not ready" in epoch 0, counters at epoch 0
    CUDA_TRY(zero_now(w.scan_status, sizeof(unsigned long long) * w.status_cap));
    CUDA_TRY(zero_now(w.scan_status2, sizeof(unsigned long long) * w.status2_cap));
    CUDA_TRY(zero_now(w.counters, sizeof(uint32_t) * kCtrCount));
    return MLV_OK;
}

static mlv_status ensure_workspace(mlv_context_t *c, const BatchSizes &s, bool keep_geom) {
    Workspace &w = c->ws;
    MLV_TRY(ensure_fixed(c));
    bool changed = false;
    const uint64_t slots = s.tris + std::max<uint64_t>(s.overflow, w.overflow_cap);
    // shading records only once a batch has a pixel shader (a depth or visibility pass with the
    // null pixel shader needs none: 80 of its 144 bytes per triangle slot)
    const bool shade = s.shade || w.shade != nullptr;
    const bool binned = s.binned || w.jobs != nullptr;   // (the small-draw path lists no bin jobs)
    if (slots > w.record_cap || !w.raster || (keep_geom && !w.geom) || (shade && !w.shade) || (binned && !w.jobs)) {
        uint64_t n = std::max<uint64_t>(slots, (uint64_t)w.record_cap + w.record_cap / 2);
        if (slots <= w.record_cap && w.raster) n = w.record_cap;   // only the shading records are new
        n = std::max<uint64_t>(n, 4096);
        if (n > 0x7FFFFFFFull) return fail(MLV_ERROR_CAPACITY_EXCEEDED, "more than 2^31 triangle slots");
        cudaFree(w.raster); cudaFree(w.shade); cudaFree(w.geom); cudaFree(w.jobs);
        w.raster = nullptr; w.shade = nullptr; w.geom = nullptr; w.jobs = nullptr;
        MLV_TRY(dev_alloc((void **)&w.raster, n * sizeof(TriRaster)));
        if (binned) MLV_TRY(dev_alloc((void **)&w.jobs, n * sizeof(uint4)));
        if (shade) MLV_TRY(dev_alloc((void **)&w.shade, n * sizeof(TriShade)));
        w.keep_geom = keep_geom || w.keep_geom;
        if (w.keep_geom) MLV_TRY(dev_alloc((void **)&w.geom, n * sizeof(TriGeom)));
        w.record_cap = (uint32_t)n;
        changed = true;
    }
    w.overflow_cap = std::max<uint32_t>(w.overflow_cap, (uint32_t)std::min<uint64_t>(s.overflow, 0x7FFFFFFFull));
    {
        uint16_t *before = w.tri_info;
        uint32_t cap = w.tri_cap;
        MLV_TRY(grow(&w.tri_info, cap, s.tris + 1, sizeof(uint16_t)));
        if (before != w.tri_info) {
            cudaFree(w.rank);
            w.rank = nullptr;
            uint32_t cap2 = 0;
            MLV_TRY(grow(&w.rank, cap2, cap, sizeof(uint32_t)));
            changed = true;
        }
        w.tri_cap = cap;
    }
    if (binned) {
        uint2 *before = w.clip_list;
        MLV_TRY(grow(&w.clip_list, w.clip_cap, s.tris + 1, sizeof(uint2)));
        changed = changed || before != w.clip_list;
    }
    {
        uint32_t *before = w.bin_count;
        uint32_t cap = w.bin_cap;
        MLV_TRY(grow(&w.bin_count, cap, s.bins + 1, sizeof(uint32_t), true));
        if (before != w.bin_count) {
            uint32_t cap2 = 0;
            cudaFree(w.bin_start);
            w.bin_start = nullptr;
            MLV_TRY(grow(&w.bin_start, cap2, cap, sizeof(uint32_t)));
            changed = true;
        }
        w.bin_cap = cap;
    }
    {
        uint64_t want = c->tuning.initial_bin_entries ? c->tuning.initial_bin_entries
                                                      : std::max<uint64_t>(s.tris * 3, 1u << 20);
        uint32_t *before = w.list;
        if (want > w.list_cap || !w.list) {
            uint32_t cap = w.list_cap;
            MLV_TRY(grow(&w.list, cap, want, sizeof(uint32_t)));
            w.list_cap = cap;
        }
        if (before != w.list) {
            changed = true;
            cudaFree(w.info_mask);
            w.info_mask = nullptr;
        }
        if (c->capture_infos && !w.info_mask) MLV_TRY(dev_alloc((void **)&w.info_mask, (size_t)w.list_cap * 8));
    }
    {
        unsigned long long *b1 = w.scan_status, *b2 = w.scan_status2;
        MLV_TRY(grow(&w.scan_status, w.status_cap, s.tris / 2048 + 2, sizeof(unsigned long long)));
        MLV_TRY(grow(&w.scan_status2, w.status2_cap, s.bins / 4096 + 2, sizeof(unsigned long long)));
        if (b1 != w.scan_status || b2 != w.scan_status2) {
            MLV_TRY(reset_scan_state(w));
            changed = true;
        }
    }
    {
        float4 *before = w.vs_out;
        MLV_TRY(grow(&w.vs_out, w.vs_cap, s.vertices * 3, sizeof(float4)));
        if (before != w.vs_out) changed = true;
    }
    if (s.direct_pixels) {
        unsigned long long *before = w.keys;
        MLV_TRY(grow(&w.keys, w.keys_cap, s.direct_pixels, sizeof(unsigned long long), true));
        uint4 *qb = w.queue;
        MLV_TRY(grow(&w.queue, w.queue_cap, std::max<uint64_t>(s.tris, 16384), sizeof(uint4)));
        uint32_t *mb = w.marked;
        MLV_TRY(grow(&w.marked, w.marked_cap, std::max<uint64_t>(s.tiles, 1), sizeof(uint32_t)));
        if (before != w.keys || qb != w.queue || mb != w.marked) changed = true;
    }
    {
        DrawDesc *b1 = w.d_draws;
        ViewDesc *b2 = w.d_views;
        MLV_TRY(grow(&w.d_draws, w.desc_draw_cap, s.draws));
        MLV_TRY(grow(&w.d_views, w.desc_view_cap, s.views));
        if (b1 != w.d_draws || b2 != w.d_views) changed = true;
    }
    if (changed) ++w.generation;
    return MLV_OK;
}

// ------------------------------------------------------------------ batch planning

struct Plan {
    std::vector<DrawDesc> draws;
    std::vector<ViewDesc> views;
    BatchSizes sizes;
    bool direct = false;   // the small-draw path (one draw per view, no binning)
    bool keys_only = false;  // ... whose resolve reads no records
    bool mark_list = false;  // ... whose views fold no clear: the resolve visits the marked tiles only
    std::unordered_set<mlv_texture2d> folded;   // cleared targets the tile kernel clears itself
    // upload events of the batch's inputs, waited for before the stage that first reads them
    std::vector<cudaEvent_t> wait_vertex, wait_index, wait_pixel;
};

static void add_wait(std::vector<cudaEvent_t> &v, cudaEvent_t e) {
    if (e && std::find(v.begin(), v.end(), e) == v.end()) v.push_back(e);
}

// Folds the segment's clears of targets that one view of the plan binds (and that the clear's kind
// fits: colour, depth, u32 fill of a visibility target) into that view. Clears precede every draw
// of a segment and each view covers its whole target, so the tile kernel, starting every tile
// from the clear value and writing all of its pixels, leaves what clear-then-draw leaves.
template <typename Groups>
static void fold_clears(const Segment &seg, const Groups &groups, Plan &p) {
    if (seg.clears.empty()) return;
    std::unordered_map<mlv_texture2d, int> uses;
    for (size_t g = 0; g < groups.size(); ++g) {
        const DrawCmd &first = seg.draws[groups[g].second[0]];
        for (mlv_texture2d t : {first.rtv, first.dsv, first.vis_tri, first.vis_draw, first.vis_bary, first.vis_prim})
            if (t) ++uses[t];
    }
    // the last clear of each target wins
    std::unordered_map<mlv_texture2d, const ClearCmd *> last;
    for (const ClearCmd &cl : seg.clears) last[cl.target] = &cl;
    for (size_t g = 0; g < groups.size(); ++g) {
        const DrawCmd &first = seg.draws[groups[g].second[0]];
        ViewDesc &v = p.views[g];
        auto fold = [&](mlv_texture2d t, int kind, uint32_t flag, uint32_t &value) {
            if (!t || uses[t] != 1) return;
            auto it = last.find(t);
            if (it == last.end() || it->second->kind != kind) return;
            v.clear_flags |= flag;
            value = it->second->value;
            p.folded.insert(t);
        };
        fold(first.rtv, 0, kClearColor, v.clear_color);
        uint32_t depth_bits = 0;
        fold(first.dsv, 1, kClearDepth, depth_bits);
        if (v.clear_flags & kClearDepth) v.clear_depth = last[first.dsv]->depth;
        fold(first.vis_tri, 2, kClearTri, v.clear_tri);
        fold(first.vis_draw, 2, kClearDraw, v.clear_draw);
        fold(first.vis_prim, 2, kClearPrim, v.clear_prim);
        fold(first.vis_bary, 2, kClearBary, v.clear_bary);
    }
}

// Whether a planned batch takes the small-draw path: every view has exactly one draw, each of at
// most `small_draw` input triangles, with no triangle-id target and no TileInfo capture (both need
// the binned path's ranks and lists). The outputs are the same either way.
static bool plan_is_direct(const Plan &p, uint32_t small_draw, bool capture) {
    if (capture || p.draws.empty() || p.draws.size() != p.views.size()) return false;
    uint64_t pixels = 0, tris = 0;
    for (const ViewDesc &v : p.views) {
        if (v.draw_count != 1 || v.vis_tri != nullptr) return false;
        pixels += (uint64_t)v.width * v.height;
    }
    for (const DrawDesc &d : p.draws) {
        if (d.tri_count > small_draw) return false;
        tris += d.tri_count;
    }
    return tris > 0 && pixels < (1ull << 31);
}

// Whether the small-draw path's resolve can take every output from the keys alone: the null pixel
// shader, no barycentric target, and viewports whose min_depth is +0 (a depth of -0, which the
// keys fold onto +0, cannot occur then).
static bool plan_keys_only(const Plan &p) {
    for (const DrawDesc &d : p.draws) {
        uint32_t min_depth_bits;
        memcpy(&min_depth_bits, &d.screen_from_ndc[11], 4);
        if (d.ps != kPsNone || min_depth_bits != 0) return false;
    }
    for (const ViewDesc &v : p.views)
        if (v.vis_bary != nullptr) return false;
    return true;
}

static mlv_status plan_segment(const Segment &seg, Plan &p, uint32_t fan_slots_hint = 0, uint32_t small_draw = 0,
                               bool capture = false) {
    p.draws.clear();
    p.views.clear();
    p.folded.clear();
    p.wait_vertex.clear();
    p.wait_index.clear();
    p.wait_pixel.clear();
    p.sizes = BatchSizes();
    for (const DrawCmd &dc : seg.draws) {
        if (dc.vb_res) add_wait(p.wait_vertex, dc.vb_res->ready);
        if (dc.vs_res) add_wait(p.wait_vertex, dc.vs_res->ready);
        if (dc.ib_res) add_wait(p.wait_index, dc.ib_res->ready);
        if (dc.ps_res) add_wait(p.wait_pixel, dc.ps_res->ready);
    }
    // group draws by (render target, depth) keeping their order inside a view
    std::vector<std::pair<std::pair<mlv_texture2d, mlv_texture2d>, std::vector<size_t>>> groups;
    for (size_t i = 0; i < seg.draws.size(); ++i) {
        auto key = std::make_pair(seg.draws[i].rtv, seg.draws[i].dsv);
        size_t g = 0;
        for (; g < groups.size(); ++g)
            if (groups[g].first == key) break;
        if (g == groups.size()) groups.push_back({key, {}});
        groups[g].second.push_back(i);
    }
    uint32_t tri = 0, tiles = 0;
    uint64_t bins = 0, verts = 0;
    for (size_t g = 0; g < groups.size(); ++g) {
        const DrawCmd &first = seg.draws[groups[g].second[0]];
        ViewDesc v = {};
        mlv_texture2d rt = first.rtv, ds = first.dsv;
        v.color = (uint32_t *)rt->ptr;
        v.depth = (float *)ds->ptr;
        v.tile_min = ds->tile_min;
        v.tile_max = ds->tile_max;
        v.vis_tri = first.vis_tri ? (uint32_t *)first.vis_tri->ptr : nullptr;
        v.vis_draw = first.vis_draw ? (uint32_t *)first.vis_draw->ptr : nullptr;
        v.vis_bary = first.vis_bary ? (float *)first.vis_bary->ptr : nullptr;
        v.vis_prim = first.vis_prim ? (uint32_t *)first.vis_prim->ptr : nullptr;
        v.width = rt->width;
        v.height = rt->height;
        v.tiles_x = ds->tiles_x;
        v.tiles_y = ds->tiles_y;
        v.tile_base = tiles;
        v.draw_begin = (uint32_t)p.draws.size();
        v.draw_count = (uint32_t)groups[g].second.size();
        v.bin_base = (uint32_t)bins;
        for (size_t k = 0; k < groups[g].second.size(); ++k) {
            const DrawCmd &dc = seg.draws[groups[g].second[k]];
            DrawDesc d = dc.desc;
            d.view = (uint32_t)g;
            d.draw_in_view = (uint32_t)k;
            if (groups[g].second.size() > 1) d.raster_flags |= kDrawSharesView;
            d.tri_begin = tri;
            tri += d.tri_count;
            // shade each vertex once when the draw references most of its buffer; a draw that
            // touches a small part of a large buffer keeps per-index shading
            d.vs_cached = host_shade_once(d.ib, d.vertex_count, d.tri_count) ? 1u : 0u;
            d.vs_base = (uint32_t)verts;
            d.vs_count = d.vs_cached ? d.vertex_count : 0u;
            verts += d.vs_count;
            p.draws.push_back(d);
        }
        tiles += v.tiles_x * v.tiles_y;
        bins += (uint64_t)v.tiles_x * v.tiles_y * v.draw_count;
        p.views.push_back(v);
    }
    if (tri > 0) fold_clears(seg, groups, p);   // no triangles: no tile kernel runs
    if (bins > 0x7FFFFFFFull || tiles > 0x7FFFFFFFu || verts > 0x7FFFFFFFull / 3)
        return fail(MLV_ERROR_CAPACITY_EXCEEDED, "batch has too many bins or vertices");
    p.sizes.vertices = verts;
    p.sizes.tris = tri;
    // clip fans beyond the slots of their input triangles; clipping is rare, and an overflow is
    // detected, regrown and re-run
    p.sizes.overflow = std::max<uint64_t>(4096, (uint64_t)tri / 8);
    if (fan_slots_hint) p.sizes.overflow = fan_slots_hint;
    p.sizes.bins = bins;
    p.sizes.tiles = tiles;
    p.sizes.draws = p.draws.size();
    p.sizes.views = p.views.size();
    // shading records: for pixel shaders, and for the draw index of a view with several draws
    for (const DrawDesc &d : p.draws)
        p.sizes.shade = p.sizes.shade || d.ps != kPsNone || (d.raster_flags & kDrawSharesView);
    p.direct = plan_is_direct(p, small_draw, capture);
    p.sizes.binned = !p.direct;
    p.keys_only = false;
    p.mark_list = false;
    if (p.direct) {
        // the vertex shader runs per index inside the raster kernel (main.c:698-734's way)
        for (DrawDesc &d : p.draws) {
            d.vs_cached = 0;
            d.vs_count = 0;
        }
        p.sizes.vertices = 0;
        uint64_t px = 0;
        for (ViewDesc &v : p.views) {
            v.key_base = (uint32_t)px;
            px += (uint64_t)v.width * v.height;
        }
        p.sizes.direct_pixels = px;
        p.keys_only = plan_keys_only(p);
        p.mark_list = true;
        for (const ViewDesc &v : p.views) p.mark_list = p.mark_list && v.clear_flags == 0;
    }
    return MLV_OK;
}

// ------------------------------------------------------------------ execution

static void ev_begin(mlv_context_t *c, int stage, cudaEvent_t *end_out) {
    *end_out = nullptr;
    if (!c->profiling || c->capturing_graph) return;
    if (c->ev_next >= c->ev_pool.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        c->ev_pool.push_back({a, b});
    }
    auto pr = c->ev_pool[c->ev_next++];
    cudaEventRecord(pr.first, c->stream);
    c->ev_pending.push_back({stage, pr});
    *end_out = pr.second;
}

static void ev_end(mlv_context_t *c, cudaEvent_t e) {
    if (e) cudaEventRecord(e, c->stream);
}

static void collect_events(mlv_context_t *c) {
    for (auto &pe : c->ev_pending) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, pe.second.first, pe.second.second) == cudaSuccess) {
            c->stage_ms[pe.first] += ms;
            c->stage_launches[pe.first] += 1;
        }
    }
    cudaGetLastError();
    c->ev_pending.clear();
    c->ev_next = 0;
}

// The fills of a segment's clears, one job per written array (a depth clear also resets the
// target's tile minima to 0, main.c:1212-1214, and the tile maxima that depth LESS uses to 1).
// A target cleared twice keeps its last clear, so the jobs write disjoint memory.
static uint32_t build_fills(const Segment &seg, std::vector<FillJob> &jobs,
                            const std::unordered_set<mlv_texture2d> *folded = nullptr) {
    jobs.clear();
    std::unordered_set<mlv_texture2d> seen;
    for (auto it = seg.clears.rbegin(); it != seg.clears.rend(); ++it) {
        const ClearCmd &cl = *it;
        mlv_texture2d t = cl.target;
        if (!seen.insert(t).second) continue;
        if (folded && folded->count(t)) continue;   // the tile kernel clears it
        uint32_t value = cl.value;
        if (cl.kind == 1) memcpy(&value, &cl.depth, 4);
        jobs.push_back({(uint32_t *)t->ptr, (uint64_t)t->width * t->height * (t->texel_bytes / 4), value, 0});
        if (cl.kind == 1) {
            const uint64_t nt = (uint64_t)t->tiles_x * t->tiles_y;
            jobs.push_back({(uint32_t *)t->tile_min, nt, 0u, 0});
            jobs.push_back({(uint32_t *)t->tile_max, nt, 0x3F800000u, 0});
        }
    }
    uint32_t chunks = 0;
    for (FillJob &j : jobs) {
        j.chunk_begin = chunks;
        chunks += (uint32_t)((j.n + kFillChunk - 1) / kFillChunk);
    }
    return chunks;
}

// Runs a segment's clears: one batched fill from `d_jobs` (device copies of `jobs`) when given,
// else through the workspace's fill buffer, or directly when there is a single array.
static mlv_status run_fills(mlv_context_t *c, const std::vector<FillJob> &jobs, uint32_t chunks,
                            const FillJob *d_jobs) {
    if (jobs.empty()) return MLV_OK;
    cudaEvent_t e;
    ev_begin(c, 0, &e);
    if (!d_jobs && jobs.size() == 1) {
        CUDA_TRY(launch_fill_u32(jobs[0].p, jobs[0].n, jobs[0].value, c->ws.error, c->stream));
    } else {
        if (!d_jobs) {
            Workspace &w = c->ws;
            MLV_TRY(grow(&w.d_fills, w.fill_cap, jobs.size()));
            CUDA_TRY(cudaMemcpyAsync(w.d_fills, jobs.data(), sizeof(FillJob) * jobs.size(), cudaMemcpyHostToDevice,
                                     c->stream));
            d_jobs = w.d_fills;
        }
        CUDA_TRY(launch_fill_many(d_jobs, (uint32_t)jobs.size(), chunks, c->ws.error, c->stream));
    }
    c->host_stats[4] += 1;
    ev_end(c, e);
    return MLV_OK;
}

static mlv_status run_clears(mlv_context_t *c, const Segment &seg) {
    std::vector<FillJob> jobs;
    const uint32_t chunks = build_fills(seg, jobs);
    return run_fills(c, jobs, chunks, nullptr);
}

// Launches the kernels of one segment's draws. `d_draws`/`d_views` hold the plan's descriptors
// on the device (uploaded by the caller).
static mlv_status launch_draws(mlv_context_t *c, const Plan &p, DrawDesc *d_draws, ViewDesc *d_views, uint32_t seq) {
    Workspace &w = c->ws;
    BatchParams bp = {};
    bp.draws = d_draws;
    bp.views = d_views;
    bp.num_draws = (uint32_t)p.draws.size();
    bp.num_views = (uint32_t)p.views.size();
    bp.total_tris = (uint32_t)p.sizes.tris;
    bp.total_tiles = (uint32_t)p.sizes.tiles;
    bp.total_bins = (uint32_t)p.sizes.bins;
    bp.overflow_capacity = w.record_cap - bp.total_tris;
    bp.list_capacity = w.list_cap;
    bp.big_tiles = c->tuning.big_triangle_tiles;
    bp.batch_seq = seq;
    bp.total_vertices = (uint32_t)p.sizes.vertices;
    bp.vs_out = w.vs_out;
    bp.raster = w.raster;
    bp.shade = w.shade;
    // the 48-byte shading record when every pixel shader of the batch reads only U and V
    bool uv_only = true;
    for (const DrawDesc &d : p.draws) uv_only = uv_only && (d.ps == MLV_PS_BASIC || d.ps == kPsNone);
    bp.shade_stride = uv_only ? kShadeUV : kShadeFull;
    bp.geom = w.keep_geom ? w.geom : nullptr;
    bp.tri_info = w.tri_info;
    bp.jobs = w.jobs;
    bp.jobs_capacity = w.record_cap;
    bp.clip_list = w.clip_list;
    bool want_rank = c->capture_infos;
    for (const ViewDesc &v : p.views) want_rank = want_rank || v.vis_tri != nullptr;
    bp.want_rank = want_rank ? 1u : 0u;
    bp.rank = want_rank ? w.rank : nullptr;
    bp.bin_count = w.bin_count;
    bp.bin_start = w.bin_start;
    bp.list = w.list;
    bp.info_mask = c->capture_infos ? w.info_mask : nullptr;
    bp.scan_status = w.scan_status;
    bp.scan_status2 = w.scan_status2;
    bp.counters = w.counters;
    bp.stats = w.stats;
    bp.error = w.error;
    bp.debug_flags = c->tuning.debug_flags;
    bp.keys = w.keys;
    bp.queue = w.queue;
    bp.queue_capacity = w.queue_cap;
    bp.keys_only = p.keys_only ? 1u : 0u;
    bp.mark_list = p.mark_list ? 1u : 0u;
    bp.marked = w.marked;
    c->host_stats[3] += 1;
    if (bp.total_tris == 0) return MLV_OK;   // nothing to assemble: no kernel has work
    // waits on queued uploads (inside a graph capture: external event waits, evaluated at launch)
    auto wait_for = [&](const std::vector<cudaEvent_t> &evs) -> cudaError_t {
        for (cudaEvent_t ev : evs) {
            cudaError_t r = cudaStreamWaitEvent(c->stream, ev, c->capturing_graph ? cudaEventWaitExternal : 0);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    };
    cudaEvent_t e;
    // the per-batch counters (clip-fan slots, queue entries, clip list, bin jobs, the persistent
    // launch's arrivals and claims) are zero here: every batch's last kernel zeroes them for the
    // next one (reset_batch_counters), and a failed batch's recovery zeroes every counter, so the
    // batch's kernels follow one another with no memset in front of them
    if (p.direct) {
        // the small-draw path: raster (vertex shader, setup, small triangles), queued large
        // triangles, resolve; stages 1, 3 and 4 of the stage timers
        CUDA_TRY(wait_for(p.wait_vertex));
        CUDA_TRY(wait_for(p.wait_index));
        ev_begin(c, 1, &e);
        CUDA_TRY(launch_direct_raster(bp, c->device->num_sms, c->stream));
        ev_end(c, e);
        ev_begin(c, 3, &e);
        CUDA_TRY(launch_direct_queue(bp, c->device->num_sms, c->stream));
        ev_end(c, e);
        CUDA_TRY(wait_for(p.wait_pixel));
        ev_begin(c, 4, &e);
        CUDA_TRY(launch_direct_resolve(bp, c->device->num_sms, c->stream));
        ev_end(c, e);
        c->host_stats[4] += 3;
        return MLV_OK;
    }
    if (c->tuning.persistent_launch) {
        // the binned pipeline as one persistent launch (k_batch), timed as the tile stage; it
        // reads every input, so it waits for all of the batch's queued uploads
        CUDA_TRY(wait_for(p.wait_vertex));
        CUDA_TRY(wait_for(p.wait_index));
        CUDA_TRY(wait_for(p.wait_pixel));
        ev_begin(c, 4, &e);
        CUDA_TRY(launch_persistent(bp, c->tuning.warps_per_tile, c->device->num_sms, c->stream));
        ev_end(c, e);
        c->host_stats[4] += 1;
        return MLV_OK;
    }
    CUDA_TRY(wait_for(p.wait_vertex));
    if (bp.total_vertices) {
        ev_begin(c, 5, &e);
        CUDA_TRY(launch_vertex(bp, c->stream));
        ev_end(c, e);
        c->host_stats[4] += 1;
    }
    CUDA_TRY(wait_for(p.wait_index));
    ev_begin(c, 1, &e);
    CUDA_TRY(launch_geometry(bp, c->tuning.geometry_block, c->device->num_sms, c->stream));   // k_geometry, then k_clip
    ev_end(c, e);
    c->host_stats[4] += 1;
    if (bp.want_rank) {
        CUDA_TRY(launch_rank(bp, c->stream));
        c->host_stats[4] += 1;
    }
    ev_begin(c, 2, &e);
    CUDA_TRY(launch_scan(bp, c->stream));
    ev_end(c, e);
    ev_begin(c, 3, &e);
    CUDA_TRY(launch_scatter(bp, c->device->num_sms, c->stream));
    ev_end(c, e);
    CUDA_TRY(wait_for(p.wait_pixel));
    ev_begin(c, 4, &e);
    CUDA_TRY(launch_tile(bp, c->tuning.tile_warps_per_block, c->tuning.warps_per_tile, c->stream));
    ev_end(c, e);
    c->host_stats[4] += 4;
    return MLV_OK;
}

static mlv_status execute_segment_eager(mlv_context_t *c, const Segment &seg, uint32_t seq, bool rerun = false) {
    if (seg.draws.empty()) return run_clears(c, seg);
    Plan p;
    MLV_TRY(plan_segment(seg, p, c->tuning.initial_clip_fan_slots, c->tuning.small_draw_triangles, c->capture_infos));
    {
        std::vector<FillJob> jobs;
        const uint32_t chunks = build_fills(seg, jobs, &p.folded);
        MLV_TRY(run_fills(c, jobs, chunks, nullptr));
    }
    MLV_TRY(ensure_workspace(c, p.sizes, false));
    // the descriptors: in a kernel's parameter block when they fit (a batch of a few draws), so
    // that the batch's kernels follow the previous batch's directly; else two copies
    const size_t draw_bytes = sizeof(DrawDesc) * p.draws.size(), view_bytes = sizeof(ViewDesc) * p.views.size();
    static_assert(sizeof(DrawDesc) % 4 == 0 && sizeof(ViewDesc) % 4 == 0, "descriptors are copied as words");
    if (draw_bytes + view_bytes <= kDescParamWords * 4u) {
        CUDA_TRY(launch_put_descriptors(p.draws.data(), (uint32_t)draw_bytes, c->ws.d_draws, p.views.data(),
                                        (uint32_t)view_bytes, c->ws.d_views, c->stream));
        c->host_stats[4] += 1;
    } else {
        CUDA_TRY(cudaMemcpyAsync(c->ws.d_draws, p.draws.data(), draw_bytes, cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(cudaMemcpyAsync(c->ws.d_views, p.views.data(), view_bytes, cudaMemcpyHostToDevice, c->stream));
    }
    MLV_TRY(launch_draws(c, p, c->ws.d_draws, c->ws.d_views, seq));
    if (!rerun) {
        c->host_stats[0] += seg.vertex_count;
        c->host_stats[1] += seg.input_triangles;
        c->host_stats[2] += seg.draws.size();
    }
    c->last_single = seg.draws.size() == 1;
    if (c->last_single) {
        c->last_total_bins = (uint32_t)p.sizes.bins;
        c->last_tiles_x = p.views[0].tiles_x;
        c->last_draw_count = 1;
        c->last_tris = (uint32_t)p.sizes.tris;
    }
    return MLV_OK;
}

// The error words and counters into the pinned host mirror, queued on the context's stream.
static mlv_status queue_error_fetch(mlv_context_t *c) {
    CUDA_TRY(cudaMemcpyAsync(c->h_error, c->ws.error, sizeof(uint32_t) * 8, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(cudaMemcpyAsync(c->h_error + 8, c->ws.counters, sizeof(uint32_t) * kCtrCount, cudaMemcpyDeviceToHost,
                             c->stream));
    return MLV_OK;
}

// Reads the device error words; on an overflow regrows the workspace and re-runs the pending
// work from the failed batch on. Called with the stream idle. fetched: the mirror already holds
// the words as of the stream's end (queue_error_fetch, then a synchronisation). *reran: set when
// batches were re-run.
static mlv_status check_and_recover(mlv_context_t *c, bool fetched = false, bool *reran = nullptr) {
    if (!c->ws.error) {
        c->pending.clear();
        return MLV_OK;
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        if (!(fetched && attempt == 0)) {
            CUDA_TRY(cudaMemcpy(c->h_error, c->ws.error, sizeof(uint32_t) * 8, cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemcpy(c->h_error + 8, c->ws.counters, sizeof(uint32_t) * kCtrCount, cudaMemcpyDeviceToHost));
        }
        const uint32_t err = c->h_error[0];
        if (c->h_error[2]) {
            // out-of-range indices read zeros, as Direct3D 11 does; report once
            uint32_t z = 0;
            CUDA_TRY(copy_to_device_now(c->ws.error + 2, &z, 4));
            g_last_error = "a draw read vertices outside its vertex buffer (zeros were used)";
        }
        if (err == 0) {
            c->pending.clear();
            return MLV_OK;
        }
        if (err & (kErrLookbackTimeout | kErrGridTimeout)) {
            MLV_TRY(reset_error_words(c->ws));
            CUDA_TRY(zero_now(c->ws.bin_count, sizeof(uint32_t) * c->ws.bin_cap));
            if (c->ws.keys) CUDA_TRY(zero_now(c->ws.keys, sizeof(unsigned long long) * c->ws.keys_cap));
            MLV_TRY(reset_scan_state(c->ws));
            c->pending.clear();
            return fail(MLV_ERROR_TIMEOUT, (err & kErrGridTimeout)
                                               ? "a bounded device-side wait gave up (persistent launch grid barrier)"
                                               : "a bounded device-side wait gave up (decoupled look-back)");
        }
        // regrow: records from the device's assembled count, list from the reported entry count
        const uint32_t need_list = c->h_error[3];
        const uint32_t need_fans = c->h_error[4];
        const uint32_t need_queue = c->h_error[5];
        Workspace &w = c->ws;
        if ((err & kErrQueueOverflow) && need_queue > w.queue_cap) {
            uint32_t cap = w.queue_cap;
            MLV_TRY(grow(&w.queue, cap, (uint64_t)need_queue + need_queue / 4 + 1024, sizeof(uint4)));
            w.queue_cap = cap;
            ++w.generation;
        }
        if (err & kErrRecordOverflow) {
            // the clip-fan region must hold `need_fans` slots beyond the input triangles
            BatchSizes s;
            s.overflow = (uint64_t)need_fans + need_fans / 2 + 4096;
            s.tris = w.tri_cap ? w.tri_cap - 1 : 0;
            MLV_TRY(ensure_workspace(c, s, false));
        }
        if ((err & kErrListOverflow) && need_list > w.list_cap) {
            uint32_t cap = w.list_cap;
            MLV_TRY(grow(&w.list, cap, (uint64_t)need_list + need_list / 4 + 1024, sizeof(uint32_t)));
            w.list_cap = cap;
            cudaFree(w.info_mask);
            w.info_mask = nullptr;
            if (c->capture_infos) MLV_TRY(dev_alloc((void **)&w.info_mask, (size_t)w.list_cap * 8));
            ++w.generation;
        }
        // reset the device state the skipped kernels left behind (and the failed batches' staged
        // statistics, which the re-run stages again)
        CUDA_TRY(zero_now(w.stats, sizeof(unsigned long long) * kStatTotal));
        CUDA_TRY(zero_now(w.bin_count, sizeof(uint32_t) * w.bin_cap));
        if (w.keys) CUDA_TRY(zero_now(w.keys, sizeof(unsigned long long) * w.keys_cap));
        MLV_TRY(reset_scan_state(w));
        MLV_TRY(reset_error_words(w));
        // Jobs before the first failing batch completed; from it on every kernel that writes a
        // render target skipped its work, so those jobs are re-run, in order.
        std::vector<PendingJob> jobs;
        jobs.swap(c->pending);
        const uint32_t failed = c->h_error[1];
        if (reran) *reran = true;
        for (const PendingJob &j : jobs) {
            if (j.seq < failed) continue;
            if (j.segment) {
                MLV_TRY(execute_segment_eager(c, *j.segment, j.seq, true));
            } else {
                for (const Segment &s : j.list->segments) MLV_TRY(execute_segment_eager(c, s, j.seq, true));
            }
            c->pending.push_back(j);
        }
        CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    return fail(MLV_ERROR_CAPACITY_EXCEEDED, "workspace overflow persisted after regrowing");
}

static mlv_status sync_context(mlv_context_t *c) {
    if (c->copy_stream) CUDA_TRY(cudaStreamSynchronize(c->copy_stream));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    collect_events(c);
    return check_and_recover(c);
}

static mlv_status submit_segment(mlv_context_t *c, Segment &&seg) {
    if (c->deferred) {
        c->recorded.push_back(std::move(seg));
        return MLV_OK;
    }
    MLV_TRY(set_device(c->device));
    auto owned = std::make_shared<Segment>(std::move(seg));
    const uint32_t seq = ++c->batch_seq;
    MLV_TRY(execute_segment_eager(c, *owned, seq));
    c->pending.push_back({owned.get(), owned, nullptr, seq});
    if (c->pending.size() > 4096) MLV_TRY(sync_context(c));
    return MLV_OK;
}

// ------------------------------------------------------------------ C ABI

extern "C" {

MLV_API const char *mlv_get_last_error_string(void) { return g_last_error.c_str(); }
MLV_API int mlv_get_abi_version(void) { return MLV_ABI_VERSION; }

MLV_API mlv_status mlv_create_device(int ordinal, mlv_device *out) {
    if (!out) return fail(MLV_ERROR_INVALID_ARG, "out_device is NULL");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || ordinal < 0 || ordinal >= n) {
        cudaGetLastError();
        return fail(MLV_ERROR_DEVICE, "no such CUDA device");
    }
    CUDA_TRY(cudaSetDevice(ordinal));
    auto *d = new mlv_device_t();
    d->ordinal = ordinal;
    cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, ordinal);
    host_clip_planes(d->clip_planes);
    set_clip_planes(d->clip_planes, 0);
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        delete d;
        return fail(MLV_ERROR_DEVICE, std::string("device init: ") + cudaGetErrorString(e));
    }
    auto *c = new mlv_context_t();
    c->device = d;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        delete d;
        return fail(MLV_ERROR_DEVICE, "cudaStreamCreate failed");
    }
    d->immediate = c;
    *out = d;
    return MLV_OK;
}

static void free_workspace(Workspace &w) {
    cudaFree(w.raster); cudaFree(w.shade); cudaFree(w.geom); cudaFree(w.tri_info); cudaFree(w.jobs); cudaFree(w.rank);
    cudaFree(w.clip_list);
    cudaFree(w.bin_count); cudaFree(w.bin_start); cudaFree(w.list); cudaFree(w.info_mask);
    cudaFree(w.scan_status); cudaFree(w.scan_status2); cudaFree(w.counters); cudaFree(w.stats);
    cudaFree(w.error); cudaFree(w.d_draws); cudaFree(w.d_views); cudaFree(w.d_fills); cudaFree(w.vs_out);
    cudaFree(w.keys); cudaFree(w.queue); cudaFree(w.marked);
    w = Workspace();
}

static void destroy_context_internal(mlv_context_t *c) {
    if (!c) return;
    cudaSetDevice(c->device->ordinal);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_workspace(c->ws);
    for (auto &pr : c->ev_pool) {
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    if (c->h_error) cudaFreeHost(c->h_error);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaFree(c->upload_staging);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->work_mark) cudaEventDestroy(c->work_mark);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

MLV_API mlv_status mlv_destroy_device(mlv_device d) {
    if (!d) return fail(MLV_ERROR_INVALID_ARG, "device is NULL");
    destroy_context_internal(d->immediate);
    delete d;
    return MLV_OK;
}

MLV_API mlv_status mlv_get_immediate_context(mlv_device d, mlv_context *out) {
    if (!d || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    *out = d->immediate;
    return MLV_OK;
}

MLV_API mlv_status mlv_create_deferred_context(mlv_device d, mlv_context *out) {
    if (!d || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    auto *c = new mlv_context_t();
    c->device = d;
    c->deferred = true;
    {
        std::lock_guard<std::mutex> lock(d->mu);
        d->deferred.push_back(c);
    }
    *out = c;
    return MLV_OK;
}

MLV_API mlv_status mlv_destroy_context(mlv_context c) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (!c->deferred) return fail(MLV_ERROR_INVALID_ARG, "the immediate context is owned by its device");
    {
        std::lock_guard<std::mutex> lock(c->device->mu);
        auto &v = c->device->deferred;
        v.erase(std::remove(v.begin(), v.end(), c), v.end());
    }
    delete c;
    return MLV_OK;
}

// A destroyed resource is unbound from every context of its device (as Direct3D 11 keeps bound
// views alive, a later state check or draw must not reach freed memory through the binding).
static void unbind_everywhere(mlv_device d, const void *res) {
    auto unbind = [res](PipelineState &st) {
        if (st.ib == res) st.ib = nullptr;
        if (st.vb == res) st.vb = nullptr;
        for (auto &b : st.vs_cb) if (b == res) b = nullptr;
        for (auto &t : st.vs_srv) if (t == res) t = nullptr;
        for (auto &t : st.ps_srv) if (t == res) t = nullptr;
        for (mlv_texture2d *t : {&st.rtv, &st.dsv, &st.vis_tri, &st.vis_draw, &st.vis_bary, &st.vis_prim})
            if (*t == res) *t = nullptr;
    };
    std::lock_guard<std::mutex> lock(d->mu);
    if (d->immediate) unbind(d->immediate->st);
    for (mlv_context_t *c : d->deferred) unbind(c->st);
}

MLV_API mlv_status mlv_create_buffer(mlv_device d, const mlv_buffer_desc *desc, const void *init, mlv_buffer *out) {
    if (!d || !desc || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (desc->byte_width == 0) return fail(MLV_ERROR_INVALID_ARG, "byte_width is 0");
    MLV_TRY(set_device(d));
    auto *b = new mlv_buffer_t();
    b->device = d;
    b->size = desc->byte_width;
    b->bind = desc->bind_flags;
    mlv_status st = dev_alloc((void **)&b->ptr, (desc->byte_width + 15) & ~15ull);
    if (st != MLV_OK) {
        delete b;
        return st;
    }
    if (desc->bind_flags & MLV_BIND_CONSTANT_BUFFER) b->shadow.assign(desc->byte_width, 0);
    if (init) {
        cudaError_t e = copy_to_device_now(b->ptr, init, desc->byte_width);
        if (e != cudaSuccess) {
            cudaFree(b->ptr);
            delete b;
            return fail(MLV_ERROR_DEVICE, cudaGetErrorString(e));
        }
        if (!b->shadow.empty()) memcpy(b->shadow.data(), init, desc->byte_width);
    }
    *out = b;
    return MLV_OK;
}

MLV_API mlv_status mlv_destroy_buffer(mlv_buffer b) {
    if (!b) return fail(MLV_ERROR_INVALID_ARG, "buffer is NULL");
    cudaSetDevice(b->device->ordinal);
    if (b->device->immediate) {
        if (b->device->immediate->copy_stream) cudaStreamSynchronize(b->device->immediate->copy_stream);
        cudaStreamSynchronize(b->device->immediate->stream);
    }
    unbind_everywhere(b->device, b);
    cudaFree(b->ptr);
    if (b->ready) cudaEventDestroy(b->ready);
    delete b;
    return MLV_OK;
}

// A host image's rows are row_pitch bytes apart (0: tightly packed); shorter than a row is an error.
static mlv_status check_pitch(uint64_t row, uint32_t row_pitch) {
    if (row_pitch != 0 && row_pitch < row) return fail(MLV_ERROR_INVALID_ARG, "row_pitch is shorter than a row");
    return MLV_OK;
}

static mlv_status create_texture2d(mlv_device d, const mlv_texture2d_desc *desc, const void *init,
                                   uint32_t row_pitch, void *placed, mlv_texture2d *out) {
    if (!d || !desc || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    uint32_t tb = texel_bytes(desc->format);
    if (!tb) return fail(MLV_ERROR_INVALID_ARG, "unknown texture format");
    if (desc->width == 0 || desc->height == 0 || desc->width > 16384 || desc->height > 16384)
        return fail(MLV_ERROR_INVALID_ARG, "texture size must be 1..16384");
    if (init) MLV_TRY(check_pitch((uint64_t)desc->width * tb, row_pitch));
    MLV_TRY(set_device(d));
    auto *t = new mlv_texture2d_t();
    t->device = d;
    t->width = desc->width;
    t->height = desc->height;
    t->format = desc->format;
    t->bind = desc->bind_flags;
    t->texel_bytes = tb;
    size_t bytes = (size_t)desc->width * desc->height * tb;
    mlv_status st = MLV_OK;
    if (placed) {
        t->ptr = (uint8_t *)placed;
        t->owns_memory = false;
    } else {
        st = dev_alloc((void **)&t->ptr, (bytes + 15) & ~(size_t)15);
    }
    if (st != MLV_OK) {
        delete t;
        return st;
    }
    auto free_own = [&]() {
        if (t->owns_memory) cudaFree(t->ptr);
    };
    if (desc->format == MLV_FORMAT_D32_FLOAT) {
        t->tiles_x = (desc->width + kTile - 1) / kTile;
        t->tiles_y = (desc->height + kTile - 1) / kTile;
        size_t nt = (size_t)t->tiles_x * t->tiles_y;
        st = dev_alloc((void **)&t->tile_min, nt * 4);
        if (st == MLV_OK) st = dev_alloc((void **)&t->tile_max, nt * 4);
        if (st != MLV_OK) {
            free_own();
            cudaFree(t->tile_min);
            delete t;
            return st;
        }
        zero_now(t->tile_min, nt * 4);
        std::vector<float> ones(nt, 1.0f);
        copy_to_device_now(t->tile_max, ones.data(), nt * 4);
    }
    if (init) {
        size_t row = (size_t)desc->width * tb;
        cudaError_t e = cudaMemcpy2D(t->ptr, row, init, row_pitch ? row_pitch : row, row, desc->height,
                                     cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            free_own();
            cudaFree(t->tile_min);
            cudaFree(t->tile_max);
            delete t;
            return fail(MLV_ERROR_DEVICE, cudaGetErrorString(e));
        }
    } else if (!placed) {
        zero_now(t->ptr, bytes);
    }
    *out = t;
    return MLV_OK;
}

MLV_API mlv_status mlv_create_texture2d(mlv_device d, const mlv_texture2d_desc *desc, const void *init,
                                        uint32_t row_pitch, mlv_texture2d *out) {
    return create_texture2d(d, desc, init, row_pitch, nullptr, out);
}

MLV_API mlv_status mlv_create_texture2d_on_memory(mlv_device d, const mlv_texture2d_desc *desc, void *device_memory,
                                                  mlv_texture2d *out) {
    if (!device_memory) return fail(MLV_ERROR_INVALID_ARG, "device_memory is NULL");
    if ((uintptr_t)device_memory & 15u) return fail(MLV_ERROR_INVALID_ARG, "device_memory must be 16-byte aligned");
    return create_texture2d(d, desc, nullptr, 0, device_memory, out);
}

MLV_API mlv_status mlv_destroy_texture2d(mlv_texture2d t) {
    if (!t) return fail(MLV_ERROR_INVALID_ARG, "texture is NULL");
    cudaSetDevice(t->device->ordinal);
    if (t->device->immediate) {
        if (t->device->immediate->copy_stream) cudaStreamSynchronize(t->device->immediate->copy_stream);
        cudaStreamSynchronize(t->device->immediate->stream);
    }
    unbind_everywhere(t->device, t);
    if (t->owns_memory) cudaFree(t->ptr);
    cudaFree(t->tile_min);
    cudaFree(t->tile_max);
    if (t->ready) cudaEventDestroy(t->ready);
    delete t;
    return MLV_OK;
}

MLV_API mlv_status mlv_buffer_device_pointer(mlv_buffer b, void **out) {
    if (!b || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    *out = b->ptr;
    return MLV_OK;
}

MLV_API mlv_status mlv_texture2d_device_pointer(mlv_texture2d t, void **out) {
    if (!t || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    *out = t->ptr;
    return MLV_OK;
}

static mlv_status need_immediate(mlv_context c) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (c->deferred) return fail(MLV_ERROR_INVALID_STATE, "this call needs the immediate context");
    return MLV_OK;
}

MLV_API mlv_status mlv_update_buffer(mlv_context c, mlv_buffer b, uint64_t offset, const void *data, uint64_t size) {
    MLV_TRY(need_immediate(c));
    if (!b || !data) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (offset > b->size || size > b->size - offset) return fail(MLV_ERROR_INVALID_ARG, "update outside the buffer");
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));   // queued draws may still read the old contents
    CUDA_TRY(copy_to_device_now(b->ptr + offset, data, size));
    if (!b->shadow.empty()) memcpy(b->shadow.data() + offset, data, size);
    return MLV_OK;
}

MLV_API mlv_status mlv_update_texture2d(mlv_context c, mlv_texture2d t, const void *data, uint32_t row_pitch) {
    MLV_TRY(need_immediate(c));
    if (!t || !data) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    size_t row = (size_t)t->width * t->texel_bytes;
    MLV_TRY(check_pitch(row, row_pitch));
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));
    CUDA_TRY(cudaMemcpy2D(t->ptr, row, data, row_pitch ? row_pitch : row, row, t->height, cudaMemcpyHostToDevice));
    return MLV_OK;
}

// Queued uploads. A batch still unchecked may be re-run at the next synchronisation (when it
// overflowed its workspace), and a re-run must read the contents it was issued with, so the
// context first synchronises if anything is pending; otherwise the copy is only queued, on the
// context's copy stream behind everything already issued on its stream, and the resource's event
// marks its completion for the batches that read it (Plan::wait_*).
// A resource's first queued upload gives it its ready event, which captured graphs must then wait
// for: that changes the upload generation, so command lists re-capture.
static mlv_status ensure_ready_event(mlv_context_t *c, cudaEvent_t *ready) {
    if (!*ready) {
        CUDA_TRY(cudaEventCreateWithFlags(ready, cudaEventDisableTiming));
        c->device->upload_generation.fetch_add(1);
    }
    return MLV_OK;
}

static mlv_status begin_upload(mlv_context_t *c, cudaEvent_t *ready) {
    if (!c->copy_stream) {
        CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&c->work_mark, cudaEventDisableTiming));
    }
    if (ready) MLV_TRY(ensure_ready_event(c, ready));
    CUDA_TRY(cudaEventRecord(c->work_mark, c->stream));
    CUDA_TRY(cudaStreamWaitEvent(c->copy_stream, c->work_mark, 0));
    return MLV_OK;
}
MLV_API mlv_status mlv_update_buffer_async(mlv_context c, mlv_buffer b, uint64_t offset, const void *data,
                                           uint64_t size) {
    MLV_TRY(need_immediate(c));
    if (!b || !data) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (offset > b->size || size > b->size - offset) return fail(MLV_ERROR_INVALID_ARG, "update outside the buffer");
    MLV_TRY(set_device(c->device));
    if (!c->pending.empty()) MLV_TRY(sync_context(c));
    MLV_TRY(begin_upload(c, &b->ready));
    CUDA_TRY(cudaMemcpyAsync(b->ptr + offset, data, size, cudaMemcpyHostToDevice, c->copy_stream));
    CUDA_TRY(cudaEventRecord(b->ready, c->copy_stream));
    if (!b->shadow.empty()) memcpy(b->shadow.data() + offset, data, size);
    return MLV_OK;
}

MLV_API mlv_status mlv_update_texture2d_async(mlv_context c, mlv_texture2d t, const void *data, uint32_t row_pitch) {
    MLV_TRY(need_immediate(c));
    if (!t || !data) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    size_t row = (size_t)t->width * t->texel_bytes;
    MLV_TRY(check_pitch(row, row_pitch));
    MLV_TRY(set_device(c->device));
    if (!c->pending.empty()) MLV_TRY(sync_context(c));
    MLV_TRY(begin_upload(c, &t->ready));
    CUDA_TRY(cudaMemcpy2DAsync(t->ptr, row, data, row_pitch ? row_pitch : row, row, t->height, cudaMemcpyHostToDevice,
                               c->copy_stream));
    CUDA_TRY(cudaEventRecord(t->ready, c->copy_stream));
    return MLV_OK;
}

// One host-to-device copy of the block into the context's staging area, then k_upload_scatter
// places the ranges (kUploadJobsPerLaunch a launch), all on the copy stream; each resource's ready
// event is recorded after the last placement.
MLV_API mlv_status mlv_update_resources_async(mlv_context c, const void *block, uint64_t block_bytes,
                                              const mlv_upload *ups, uint32_t count) {
    MLV_TRY(need_immediate(c));
    if (count == 0) return MLV_OK;
    if (!block || !ups) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    std::vector<UploadJob> jobs(count);
    for (uint32_t i = 0; i < count; ++i) {
        const mlv_upload &u = ups[i];
        if (!u.resource) return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": NULL resource");
        if (u.src_offset % 16) return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": src_offset must be a multiple of 16");
        if (u.src_offset > block_bytes || u.size > block_bytes - u.src_offset)
            return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": range outside the block");
        uint8_t *dst = nullptr;
        if (u.kind == MLV_UPLOAD_BUFFER) {
            mlv_buffer b = (mlv_buffer)u.resource;
            if (b->device != c->device) return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": another device's buffer");
            if (u.dst_offset > b->size || u.size > b->size - u.dst_offset)
                return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": update outside the buffer");
            dst = b->ptr + u.dst_offset;
        } else if (u.kind == MLV_UPLOAD_TEXTURE2D) {
            mlv_texture2d t = (mlv_texture2d)u.resource;
            if (t->device != c->device) return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": another device's texture");
            if (u.dst_offset != 0 || u.size != (uint64_t)t->width * t->height * t->texel_bytes)
                return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": a texture takes its whole size at offset 0");
            dst = t->ptr;
        } else {
            return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": unknown kind");
        }
        if ((uintptr_t)dst % 16) return fail(MLV_ERROR_INVALID_ARG, "upload " + std::to_string(i) + ": destination not 16-byte aligned");
        jobs[i] = UploadJob{dst, u.src_offset, u.size};
    }
    MLV_TRY(set_device(c->device));
    if (!c->pending.empty()) MLV_TRY(sync_context(c));
    MLV_TRY(begin_upload(c, nullptr));
    if (block_bytes > c->upload_staging_cap) {
        CUDA_TRY(cudaStreamSynchronize(c->copy_stream));   // earlier grouped uploads still read it
        cudaFree(c->upload_staging);
        c->upload_staging = nullptr;
        c->upload_staging_cap = 0;
        MLV_TRY(dev_alloc((void **)&c->upload_staging, block_bytes));
        c->upload_staging_cap = block_bytes;
    }
    CUDA_TRY(cudaMemcpyAsync(c->upload_staging, block, block_bytes, cudaMemcpyHostToDevice, c->copy_stream));
    for (uint32_t first = 0; first < count; first += kUploadJobsPerLaunch) {
        UploadJobs part = {};
        const uint32_t n = std::min<uint32_t>(kUploadJobsPerLaunch, count - first);
        uint64_t largest = 0;
        for (uint32_t k = 0; k < n; ++k) {
            part.job[k] = jobs[first + k];
            largest = std::max<uint64_t>(largest, jobs[first + k].size);
        }
        CUDA_TRY(launch_upload_scatter(c->upload_staging, part, n, largest, c->device->num_sms, c->copy_stream));
    }
    for (uint32_t i = 0; i < count; ++i) {
        const mlv_upload &u = ups[i];
        cudaEvent_t *ready = u.kind == MLV_UPLOAD_BUFFER ? &((mlv_buffer)u.resource)->ready : &((mlv_texture2d)u.resource)->ready;
        MLV_TRY(ensure_ready_event(c, ready));
        CUDA_TRY(cudaEventRecord(*ready, c->copy_stream));
        if (u.kind == MLV_UPLOAD_BUFFER) {
            mlv_buffer b = (mlv_buffer)u.resource;
            if (!b->shadow.empty()) memcpy(b->shadow.data() + u.dst_offset, (const uint8_t *)block + u.src_offset, u.size);
        }
    }
    return MLV_OK;
}

// The copy is queued behind the context's work together with the error words, so one
// synchronisation covers both; when that shows a batch must be re-run, the copy is made again.
MLV_API mlv_status mlv_read_texture2d(mlv_context c, mlv_texture2d t, void *dst, uint32_t row_pitch) {
    MLV_TRY(need_immediate(c));
    if (!t || !dst) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    const size_t row = (size_t)t->width * t->texel_bytes, pitch = row_pitch ? row_pitch : row;
    MLV_TRY(check_pitch(row, row_pitch));
    MLV_TRY(set_device(c->device));
    if (c->copy_stream) CUDA_TRY(cudaStreamSynchronize(c->copy_stream));   // queued uploads land first
    CUDA_TRY(cudaMemcpy2DAsync(dst, pitch, t->ptr, row, row, t->height, cudaMemcpyDeviceToHost, c->stream));
    const bool fetched = c->ws.error != nullptr;
    if (fetched) MLV_TRY(queue_error_fetch(c));
    CUDA_TRY(cudaStreamSynchronize(c->stream));
    collect_events(c);
    bool reran = false;
    MLV_TRY(check_and_recover(c, fetched, &reran));
    if (reran) CUDA_TRY(cudaMemcpy2D(dst, pitch, t->ptr, row, row, t->height, cudaMemcpyDeviceToHost));
    return MLV_OK;
}

MLV_API mlv_status mlv_ia_set_primitive_topology(mlv_context c, mlv_primitive_topology topo) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (topo != MLV_PRIMITIVE_TOPOLOGY_TRIANGLELIST) return fail(MLV_ERROR_UNSUPPORTED, "only triangle lists");
    c->st.topology = topo;
    return MLV_OK;
}

MLV_API mlv_status mlv_ia_set_index_buffer(mlv_context c, mlv_buffer b, mlv_format fmt, uint32_t offset) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (b && fmt != MLV_FORMAT_R32_UINT) return fail(MLV_ERROR_UNSUPPORTED, "index buffers are 32-bit");
    if (offset & 3) return fail(MLV_ERROR_INVALID_ARG, "index buffer offset must be a multiple of 4");
    c->st.ib = b;
    c->st.ib_offset = offset;
    return MLV_OK;
}

MLV_API mlv_status mlv_ia_set_vertex_buffers(mlv_context c, uint32_t start, uint32_t n, const mlv_buffer *bufs,
                                             const uint32_t *strides, const uint32_t *offsets) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (start != 0 || n > 1) return fail(MLV_ERROR_UNSUPPORTED, "one vertex buffer slot");
    if (n == 0) return MLV_OK;
    if (!bufs || !strides) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (bufs[0] && (strides[0] < 32 || (strides[0] & 3)))
        return fail(MLV_ERROR_INVALID_ARG, "vertex stride must be >= 32 and a multiple of 4");
    const uint32_t offset = offsets ? offsets[0] : 0;
    if (offset & 3) return fail(MLV_ERROR_INVALID_ARG, "vertex buffer offset must be a multiple of 4");
    c->st.vb = bufs[0];   // a refused call leaves the bound state as it was
    c->st.vb_stride = strides[0];
    c->st.vb_offset = offset;
    return MLV_OK;
}

MLV_API mlv_status mlv_vs_set_shader(mlv_context c, mlv_vertex_shader_id s) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (s < MLV_VS_BASIC || s > MLV_VS_PASSTHROUGH_UV) return fail(MLV_ERROR_INVALID_ARG, "unknown vertex shader");
    c->st.vs = s;
    return MLV_OK;
}

MLV_API mlv_status mlv_ps_set_shader(mlv_context c, mlv_pixel_shader_id s) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (s < MLV_PS_BASIC || s > MLV_PS_NONE) return fail(MLV_ERROR_INVALID_ARG, "unknown pixel shader");
    c->st.ps = s;
    return MLV_OK;
}

MLV_API mlv_status mlv_vs_set_constant_buffers(mlv_context c, uint32_t start, uint32_t n, const mlv_buffer *bufs) {
    if (!c || (n && !bufs)) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (start > MLV_CONSTANT_BUFFER_SLOT_COUNT || n > MLV_CONSTANT_BUFFER_SLOT_COUNT - start)
        return fail(MLV_ERROR_INVALID_ARG, "slot out of range");
    for (uint32_t i = 0; i < n; ++i) c->st.vs_cb[start + i] = bufs[i];
    return MLV_OK;
}

MLV_API mlv_status mlv_vs_set_shader_resources(mlv_context c, uint32_t start, uint32_t n, const mlv_texture2d *t) {
    if (!c || (n && !t)) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (start > MLV_SHADER_RESOURCE_SLOT_COUNT || n > MLV_SHADER_RESOURCE_SLOT_COUNT - start)
        return fail(MLV_ERROR_INVALID_ARG, "slot out of range");
    for (uint32_t i = 0; i < n; ++i) c->st.vs_srv[start + i] = t[i];
    return MLV_OK;
}

MLV_API mlv_status mlv_ps_set_shader_resources(mlv_context c, uint32_t start, uint32_t n, const mlv_texture2d *t) {
    if (!c || (n && !t)) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (start > MLV_SHADER_RESOURCE_SLOT_COUNT || n > MLV_SHADER_RESOURCE_SLOT_COUNT - start)
        return fail(MLV_ERROR_INVALID_ARG, "slot out of range");
    for (uint32_t i = 0; i < n; ++i) c->st.ps_srv[start + i] = t[i];
    return MLV_OK;
}

MLV_API mlv_status mlv_rs_set_viewports(mlv_context c, uint32_t n, const mlv_viewport *vp) {
    if (!c || (n && !vp)) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (n != 1) return fail(MLV_ERROR_UNSUPPORTED, "one viewport");
    c->st.viewport = vp[0];
    c->st.viewport_set = true;
    return MLV_OK;
}

MLV_API mlv_status mlv_rs_set_state(mlv_context c, const mlv_rasterizer_desc *d) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (!d) { c->st.cull = 1; c->st.raster_flags = 0; return MLV_OK; }
    int cull;
    switch (d->cull_mode) {
        case MLV_CULL_NONE: cull = 0; break;
        case MLV_CULL_BACK: cull = 1; break;
        case MLV_CULL_FRONT: cull = 2; break;
        default: return fail(MLV_ERROR_INVALID_ARG, "unknown cull mode");
    }
    if (d->fill_rule != MLV_FILL_INCLUSIVE && d->fill_rule != MLV_FILL_TOP_LEFT)
        return fail(MLV_ERROR_INVALID_ARG, "unknown fill rule");
    if (d->sample_position != MLV_SAMPLE_PIXEL_CORNER && d->sample_position != MLV_SAMPLE_PIXEL_CENTER)
        return fail(MLV_ERROR_INVALID_ARG, "unknown sample position");
    c->st.cull = cull;
    c->st.raster_flags = (d->fill_rule == MLV_FILL_TOP_LEFT ? kRasterTopLeft : 0) |
                         (d->sample_position == MLV_SAMPLE_PIXEL_CENTER ? kRasterCenter : 0);
    return MLV_OK;
}

MLV_API mlv_status mlv_om_set_depth_stencil_state(mlv_context c, const mlv_depth_stencil_desc *d) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (!d) { c->st.depth_less = 0; return MLV_OK; }
    if (!d->depth_enable) return fail(MLV_ERROR_UNSUPPORTED, "depth testing cannot be disabled");
    if (d->depth_func == MLV_COMPARISON_GREATER_EQUAL) c->st.depth_less = 0;
    else if (d->depth_func == MLV_COMPARISON_LESS) c->st.depth_less = 1;
    else return fail(MLV_ERROR_UNSUPPORTED, "depth function must be LESS or GREATER_EQUAL");
    return MLV_OK;
}

MLV_API mlv_status mlv_om_set_render_targets(mlv_context c, mlv_texture2d rt, mlv_texture2d ds) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (rt && rt->format != MLV_FORMAT_R8G8B8A8_UNORM)
        return fail(MLV_ERROR_INVALID_ARG, "render target must be R8G8B8A8_UNORM");
    if (ds && ds->format != MLV_FORMAT_D32_FLOAT) return fail(MLV_ERROR_INVALID_ARG, "depth target must be D32_FLOAT");
    if (rt && ds && (rt->width != ds->width || rt->height != ds->height))
        return fail(MLV_ERROR_INVALID_ARG, "render target and depth target differ in size");
    c->st.rtv = rt;
    c->st.dsv = ds;
    return MLV_OK;
}

MLV_API mlv_status mlv_om_set_primitive_id_target(mlv_context c, mlv_texture2d prim) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (prim && prim->format != MLV_FORMAT_R32_UINT)
        return fail(MLV_ERROR_INVALID_ARG, "primitive-id target must be R32_UINT");
    c->st.vis_prim = prim;
    return MLV_OK;
}

MLV_API mlv_status mlv_om_set_visibility_targets(mlv_context c, mlv_texture2d tri, mlv_texture2d draw,
                                                 mlv_texture2d bary) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    if (tri && tri->format != MLV_FORMAT_R32_UINT) return fail(MLV_ERROR_INVALID_ARG, "triangle-id target must be R32_UINT");
    if (draw && draw->format != MLV_FORMAT_R32_UINT) return fail(MLV_ERROR_INVALID_ARG, "draw-id target must be R32_UINT");
    if (bary && bary->format != MLV_FORMAT_R32G32_FLOAT)
        return fail(MLV_ERROR_INVALID_ARG, "barycentric target must be R32G32_FLOAT");
    c->st.vis_tri = tri;
    c->st.vis_draw = draw;
    c->st.vis_bary = bary;
    return MLV_OK;
}

static uint32_t encode_clear(const float *c) {
    auto tr = [](float x) -> uint32_t {
        if (!(x > -9.2e18f && x < 9.2e18f)) return 0u;
        return (uint32_t)(long long)x;
    };
    return (tr(c[3] * 255.f) << 24) + (tr(c[2] * 255.f) << 16) + (tr(c[1] * 255.f) << 8) + tr(c[0] * 255.f);
}

static bool draw_touches(const DrawCmd &d, mlv_texture2d t) {
    if (d.rtv == t || d.dsv == t || d.vis_tri == t || d.vis_draw == t || d.vis_bary == t || d.vis_prim == t)
        return true;
    return d.desc.vs_tex.data == t->ptr || d.desc.ps_tex.data == t->ptr;
}

static mlv_status submit_clear(mlv_context c, const ClearCmd &cl) {
    if (c->deferred) {
        // A clear joins the last segment (it runs before the segment's draws) unless one of those
        // draws reads or writes the cleared texture; then it opens a new segment.
        if (!c->recorded.empty()) {
            Segment &last = c->recorded.back();
            bool conflict = false;
            for (const DrawCmd &d : last.draws) conflict = conflict || draw_touches(d, cl.target);
            if (!conflict) {
                last.clears.push_back(cl);
                return MLV_OK;
            }
        }
        Segment seg;
        seg.clears.push_back(cl);
        c->recorded.push_back(std::move(seg));
        return MLV_OK;
    }
    Segment seg;
    seg.clears.push_back(cl);
    return submit_segment(c, std::move(seg));
}

MLV_API mlv_status mlv_clear_render_target_view(mlv_context c, mlv_texture2d rt, const float rgba[4]) {
    if (!c || !rt || !rgba) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (rt->format != MLV_FORMAT_R8G8B8A8_UNORM) return fail(MLV_ERROR_INVALID_ARG, "not a colour target");
    ClearCmd cl = {rt, 0, encode_clear(rgba), 0.f};
    rt->draws_since_clear = 0;
    return submit_clear(c, cl);
}

MLV_API mlv_status mlv_clear_depth_stencil_view(mlv_context c, mlv_texture2d ds, float depth) {
    if (!c || !ds) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (ds->format != MLV_FORMAT_D32_FLOAT) return fail(MLV_ERROR_INVALID_ARG, "not a depth target");
    ClearCmd cl = {ds, 1, 0u, depth};
    return submit_clear(c, cl);
}

MLV_API mlv_status mlv_clear_texture_u32(mlv_context c, mlv_texture2d t, uint32_t value) {
    if (!c || !t) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    ClearCmd cl = {t, 2, value, 0.f};
    return submit_clear(c, cl);
}

static mlv_status build_draw(mlv_context c, uint32_t count, uint32_t start, int32_t base_vertex, bool indexed,
                             DrawCmd &out) {
    const PipelineState &s = c->st;
    if (!s.rtv || !s.dsv) return fail(MLV_ERROR_INVALID_STATE, "render target and depth target must be bound");
    if (!s.vb) return fail(MLV_ERROR_INVALID_STATE, "no vertex buffer bound");
    if (indexed && !s.ib) return fail(MLV_ERROR_INVALID_STATE, "no index buffer bound");
    if (!s.vs || !s.ps) return fail(MLV_ERROR_INVALID_STATE, "shaders not set");
    if (!s.viewport_set) return fail(MLV_ERROR_INVALID_STATE, "no viewport set");
    const mlv_viewport &vp = s.viewport;
    if (!(vp.width >= 1.0f && vp.height >= 1.0f) || vp.width > (float)s.rtv->width ||
        vp.height > (float)s.rtv->height || vp.top_left_x != 0.0f || vp.top_left_y != 0.0f)
        return fail(MLV_ERROR_INVALID_STATE, "the viewport must start at (0,0) and fit in the render target");
    DrawDesc &d = out.desc;
    memset(&d, 0, sizeof(d));
    d.vb = s.vb->ptr + s.vb_offset;
    d.vb_stride = s.vb_stride;
    uint64_t avail = s.vb->size > s.vb_offset ? s.vb->size - s.vb_offset : 0;
    d.vertex_count = avail >= 32 ? (uint32_t)std::min<uint64_t>((avail - 32) / s.vb_stride + 1, 0xFFFFFFFFu) : 0;
    if (indexed) {
        const uint64_t nidx = s.ib->size > s.ib_offset ? (s.ib->size - s.ib_offset) / 4 : 0;
        if ((uint64_t)start + count > nidx) return fail(MLV_ERROR_INVALID_ARG, "draw reads past the index buffer");
        d.ib = (const uint32_t *)(s.ib->ptr + s.ib_offset);
    } else {
        d.ib = nullptr;
        base_vertex = 0;
    }
    d.start_index = start;
    d.base_vertex = base_vertex;
    d.tri_count = count / 3;
    d.vs = s.vs;
    d.ps = s.ps;
    d.cull = s.cull;
    d.raster_flags = s.raster_flags;
    d.depth_less = s.depth_less;
    mlv_buffer cb = s.vs_cb[0];
    if (s.vs == MLV_VS_BASIC || s.vs == MLV_VS_VERTEX_LIGHTING || s.vs == MLV_VS_FULLSCREEN) {
        if (!cb || cb->shadow.size() < sizeof(d.cb))
            return fail(MLV_ERROR_INVALID_STATE, "VS constant buffer 0 must hold a 192-byte PerFrameCB");
    }
    if (cb && !cb->shadow.empty()) memcpy(d.cb, cb->shadow.data(), std::min(sizeof(d.cb), cb->shadow.size()));
    host_screen_from_ndc(vp, d.screen_from_ndc);
    d.vp_w = (int32_t)vp.width;
    d.vp_h = (int32_t)vp.height;
    mlv_texture2d vt = s.vs_srv[0], pt = s.ps_srv[0];
    auto is_float = [](mlv_texture2d t) {
        return t && (t->format == MLV_FORMAT_R32G32B32A32_FLOAT || t->format == MLV_FORMAT_R16G16B16A16_FLOAT);
    };
    if (s.vs == MLV_VS_VERTEX_LIGHTING && !is_float(vt))
        return fail(MLV_ERROR_INVALID_STATE, "vertex_lighting_vs needs a float texture in VS slot 0");
    if (s.ps == MLV_PS_BASIC && !(pt && pt->format == MLV_FORMAT_R8G8B8A8_UNORM))
        return fail(MLV_ERROR_INVALID_STATE, "basic_ps needs an R8G8B8A8 texture in PS slot 0");
    if (s.ps == MLV_PS_ENV_LIGHTING && !is_float(pt))
        return fail(MLV_ERROR_INVALID_STATE, "env_lighting_ps needs a float texture in PS slot 0");
    if (s.ps == MLV_PS_COLOR_TIMES_TEXEL && !(pt && (is_float(pt) || pt->format == MLV_FORMAT_R8G8B8A8_UNORM)))
        return fail(MLV_ERROR_INVALID_STATE, "COLOR_TIMES_TEXEL needs a texture in PS slot 0");
    d.vs_tex = tex_desc(vt);
    d.ps_tex = tex_desc(pt);
    auto vis_ok = [&](mlv_texture2d t) { return !t || (t->width == s.rtv->width && t->height == s.rtv->height); };
    if (!vis_ok(s.vis_tri) || !vis_ok(s.vis_draw) || !vis_ok(s.vis_bary) || !vis_ok(s.vis_prim))
        return fail(MLV_ERROR_INVALID_STATE, "visibility targets must match the render target size");
    d.draw_seq = s.rtv->draws_since_clear++;
    out.rtv = s.rtv;
    out.dsv = s.dsv;
    out.vis_tri = s.vis_tri;
    out.vis_draw = s.vis_draw;
    out.vis_bary = s.vis_bary;
    out.vis_prim = s.vis_prim;
    out.index_count = count;
    out.vb_res = s.vb;
    out.ib_res = indexed ? s.ib : nullptr;
    out.vs_res = vt;
    out.ps_res = pt;
    return MLV_OK;
}

static mlv_status submit_draw(mlv_context c, DrawCmd &&dc) {
    if (c->deferred) {
        // a draw that samples a texture an earlier draw of the segment renders to (or renders to
        // one an earlier draw samples) starts a new segment: a batch reads all inputs first
        bool conflict = c->recorded.empty();
        if (!conflict) {
            for (const DrawCmd &d : c->recorded.back().draws) {
                auto ptr_of = [](mlv_texture2d t) { return t ? (const void *)t->ptr : (const void *)1; };
                if (d.desc.vs_tex.data == ptr_of(dc.rtv) || d.desc.ps_tex.data == ptr_of(dc.rtv) ||
                    dc.desc.vs_tex.data == ptr_of(d.rtv) || dc.desc.ps_tex.data == ptr_of(d.rtv) ||
                    dc.desc.vs_tex.data == ptr_of(d.dsv) || dc.desc.ps_tex.data == ptr_of(d.dsv))
                    conflict = true;
            }
        }
        if (conflict) c->recorded.emplace_back();
        Segment &last = c->recorded.back();
        last.draws.push_back(std::move(dc));
        last.input_triangles += last.draws.back().desc.tri_count;
        last.vertex_count += last.draws.back().index_count;
        return MLV_OK;
    }
    Segment seg;
    seg.input_triangles = dc.desc.tri_count;
    seg.vertex_count = dc.index_count;
    seg.draws.push_back(std::move(dc));
    return submit_segment(c, std::move(seg));
}

MLV_API mlv_status mlv_draw_indexed(mlv_context c, uint32_t count, uint32_t start, int32_t base_vertex) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    DrawCmd dc;
    MLV_TRY(build_draw(c, count, start, base_vertex, true, dc));
    return submit_draw(c, std::move(dc));
}

MLV_API mlv_status mlv_draw(mlv_context c, uint32_t count, uint32_t start) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    DrawCmd dc;
    MLV_TRY(build_draw(c, count, start, 0, false, dc));
    return submit_draw(c, std::move(dc));
}

MLV_API mlv_status mlv_flush(mlv_context c) {
    if (!c) return fail(MLV_ERROR_INVALID_ARG, "context is NULL");
    return MLV_OK;
}

MLV_API mlv_status mlv_finish(mlv_context c) {
    MLV_TRY(need_immediate(c));
    MLV_TRY(set_device(c->device));
    return sync_context(c);
}

MLV_API mlv_status mlv_get_stream(mlv_context c, void **out) {
    if (!c || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    *out = c->deferred ? nullptr : (void *)c->stream;
    return MLV_OK;
}

MLV_API mlv_status mlv_finish_command_list(mlv_context c, mlv_command_list *out) {
    if (!c || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (!c->deferred) return fail(MLV_ERROR_INVALID_STATE, "command lists come from deferred contexts");
    auto *l = new mlv_command_list_t();
    l->device = c->device;
    l->segments.swap(c->recorded);
    *out = l;
    return MLV_OK;
}

MLV_API mlv_status mlv_destroy_command_list(mlv_command_list l) {
    if (!l) return fail(MLV_ERROR_INVALID_ARG, "list is NULL");
    cudaSetDevice(l->device->ordinal);
    if (l->device->immediate) cudaStreamSynchronize(l->device->immediate->stream);
    if (l->exec) cudaGraphExecDestroy(l->exec);
    cudaFree(l->d_draws);
    cudaFree(l->d_views);
    cudaFree(l->d_fills);
    delete l;
    return MLV_OK;
}

// Plans every segment of the list with the context's tuning; maxs: the largest of their sizes.
static mlv_status plan_list(mlv_context_t *c, mlv_command_list l, std::vector<Plan> &plans, BatchSizes &maxs,
                            size_t &nd, size_t &nv) {
    plans.assign(l->segments.size(), Plan());
    maxs = BatchSizes();
    nd = nv = 0;
    for (size_t i = 0; i < l->segments.size(); ++i) {
        MLV_TRY(plan_segment(l->segments[i], plans[i], c->tuning.initial_clip_fan_slots,
                             c->tuning.small_draw_triangles, c->capture_infos));
        const BatchSizes &s = plans[i].sizes;
        maxs.direct_pixels = std::max(maxs.direct_pixels, s.direct_pixels);
        maxs.tris = std::max(maxs.tris, s.tris);
        maxs.overflow = std::max(maxs.overflow, s.overflow);
        maxs.bins = std::max(maxs.bins, s.bins);
        maxs.tiles = std::max(maxs.tiles, s.tiles);
        maxs.draws = std::max(maxs.draws, s.draws);
        maxs.views = std::max(maxs.views, s.views);
        maxs.vertices = std::max(maxs.vertices, s.vertices);
        maxs.shade = maxs.shade || s.shade;
        maxs.binned = maxs.binned || s.binned;
        nd += plans[i].draws.size();
        nv += plans[i].views.size();
    }
    return MLV_OK;
}

// Sizes the workspace for the list as the context's tuning plans it, and uploads its descriptors
// if they were planned otherwise. Run before a graph capture: the captured kernels keep the
// workspace's pointers, and a tuning change can move the list to another path with buffers and
// descriptors of its own (the small-draw path's keys, the binned path's job list; whether the
// vertices are shaded once or per index).
static mlv_status upload_list(mlv_context_t *c, mlv_command_list l, const std::vector<Plan> &plans,
                              const std::vector<std::vector<FillJob>> &fills, size_t nd, size_t nv);
static bool list_descriptors_current(const mlv_context_t *c, mlv_command_list l);
static void build_list_fills(mlv_command_list l, const std::vector<Plan> &plans,
                             std::vector<std::vector<FillJob>> &fills, std::vector<uint32_t> &chunks);

static mlv_status size_list(mlv_context_t *c, mlv_command_list l) {
    std::vector<Plan> plans;
    BatchSizes maxs;
    size_t nd = 0, nv = 0;
    MLV_TRY(plan_list(c, l, plans, maxs, nd, nv));
    MLV_TRY(ensure_workspace(c, maxs, false));
    // the descriptors too: planned for another tuning, they may describe the other path
    if (!list_descriptors_current(c, l)) {
        std::vector<std::vector<FillJob>> fills;
        std::vector<uint32_t> chunks;
        build_list_fills(l, plans, fills, chunks);
        MLV_TRY(upload_list(c, l, plans, fills, nd, nv));
    }
    return MLV_OK;
}

// Builds the list's device descriptors, sizes the workspace for its largest segment and
// records all of its kernels on the context stream (eagerly, or into a graph being captured,
// after size_list).
// Uploads the list's fill jobs and draw and view descriptors as planned (before any capture: the
// copies are synchronous).
static mlv_status upload_list(mlv_context_t *c, mlv_command_list l, const std::vector<Plan> &plans,
                              const std::vector<std::vector<FillJob>> &fills, size_t nd, size_t nv) {
    size_t nf = 0;
    for (auto &f : fills) nf += f.size();
    if (nf > l->fills_total || !l->d_fills) {
        cudaFree(l->d_fills);
        l->d_fills = nullptr;
        MLV_TRY(dev_alloc((void **)&l->d_fills, std::max<size_t>(nf, 1) * sizeof(FillJob)));
        l->fills_total = nf;
    }
    l->fill_off.clear();
    size_t of = 0;
    for (auto &f : fills) {
        l->fill_off.push_back(of);
        if (!f.empty()) CUDA_TRY(copy_to_device_now(l->d_fills + of, f.data(), sizeof(FillJob) * f.size()));
        of += f.size();
    }
    if (nd > l->draws_total || !l->d_draws) {
        cudaFree(l->d_draws);
        l->d_draws = nullptr;
        MLV_TRY(dev_alloc((void **)&l->d_draws, std::max<size_t>(nd, 1) * sizeof(DrawDesc)));
        l->draws_total = nd;
    }
    if (nv > l->views_total || !l->d_views) {
        cudaFree(l->d_views);
        l->d_views = nullptr;
        MLV_TRY(dev_alloc((void **)&l->d_views, std::max<size_t>(nv, 1) * sizeof(ViewDesc)));
        l->views_total = nv;
    }
    l->draw_off.clear();
    l->view_off.clear();
    size_t od = 0, ov = 0;
    for (auto &p : plans) {
        l->draw_off.push_back(od);
        l->view_off.push_back(ov);
        if (!p.draws.empty())
            CUDA_TRY(copy_to_device_now(l->d_draws + od, p.draws.data(), sizeof(DrawDesc) * p.draws.size()));
        if (!p.views.empty())
            CUDA_TRY(copy_to_device_now(l->d_views + ov, p.views.data(), sizeof(ViewDesc) * p.views.size()));
        od += p.draws.size();
        ov += p.views.size();
    }
    l->desc_tuning = c->tuning_generation;
    l->desc_context = c;
    l->desc_capture = c->capture_infos;
    return MLV_OK;
}

// Whether the list's uploaded descriptors were planned with the context's current tuning.
static bool list_descriptors_current(const mlv_context_t *c, mlv_command_list l) {
    return l->d_draws && l->d_fills && l->desc_tuning == c->tuning_generation && l->desc_context == c &&
           l->desc_capture == c->capture_infos;
}

static void build_list_fills(mlv_command_list l, const std::vector<Plan> &plans,
                             std::vector<std::vector<FillJob>> &fills, std::vector<uint32_t> &chunks) {
    fills.assign(l->segments.size(), {});
    chunks.assign(l->segments.size(), 0);
    for (size_t i = 0; i < l->segments.size(); ++i) chunks[i] = build_fills(l->segments[i], fills[i], &plans[i].folded);
}

static mlv_status run_list(mlv_context_t *c, mlv_command_list l, uint32_t seq, bool upload) {
    std::vector<Plan> plans;
    BatchSizes maxs;
    size_t nd = 0, nv = 0;
    MLV_TRY(plan_list(c, l, plans, maxs, nd, nv));
    if (!c->capturing_graph) MLV_TRY(ensure_workspace(c, maxs, false));
    std::vector<std::vector<FillJob>> fills;
    std::vector<uint32_t> fill_chunks;
    build_list_fills(l, plans, fills, fill_chunks);
    if (upload || !list_descriptors_current(c, l)) {
        if (c->capturing_graph) return fail(MLV_ERROR_INVALID_STATE, "command list descriptors not uploaded before a capture");
        MLV_TRY(upload_list(c, l, plans, fills, nd, nv));
    }
    for (size_t i = 0; i < l->segments.size(); ++i) {
        MLV_TRY(run_fills(c, fills[i], fill_chunks[i], l->d_fills + l->fill_off[i]));
        if (!plans[i].draws.empty())
            MLV_TRY(launch_draws(c, plans[i], l->d_draws + l->draw_off[i], l->d_views + l->view_off[i], seq));
        c->host_stats[0] += l->segments[i].vertex_count;
        c->host_stats[1] += l->segments[i].input_triangles;
        c->host_stats[2] += l->segments[i].draws.size();
    }
    return MLV_OK;
}

MLV_API mlv_status mlv_execute_command_list(mlv_context c, mlv_command_list l) {
    MLV_TRY(need_immediate(c));
    if (!l) return fail(MLV_ERROR_INVALID_ARG, "list is NULL");
    if (l->device != c->device) return fail(MLV_ERROR_INVALID_ARG, "the list was recorded for another device");
    MLV_TRY(set_device(c->device));
    const uint32_t seq = ++c->batch_seq;
    c->last_single = false;
    if (l->executions == 0 || c->profiling) {
        // first execution runs eagerly and synchronises, so that the workspace is sized before
        // the list is captured into a graph
        MLV_TRY(run_list(c, l, seq, l->executions == 0));
        c->pending.push_back({nullptr, nullptr, l, seq});
        ++l->executions;
        if (l->executions == 1) MLV_TRY(sync_context(c));
        return MLV_OK;
    }
    const uint64_t uploads = c->device->upload_generation.load();
    if (!l->exec || l->exec_generation != c->ws.generation || l->exec_context != c ||
        l->exec_tuning != c->tuning_generation || l->exec_uploads != uploads) {
        if (l->exec) cudaGraphExecDestroy(l->exec);
        l->exec = nullptr;
        MLV_TRY(size_list(c, l));
        cudaGraph_t g = nullptr;
        uint64_t saved[8];
        memcpy(saved, c->host_stats, sizeof(saved));
        CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        c->capturing_graph = true;
        mlv_status st = run_list(c, l, seq, false);
        c->capturing_graph = false;
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        l->launches_per_execution = c->host_stats[4] - saved[4];
        memcpy(c->host_stats, saved, sizeof(saved));
        if (st != MLV_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return fail(MLV_ERROR_DEVICE, std::string("graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&l->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(MLV_ERROR_DEVICE, std::string("graph instantiate: ") + cudaGetErrorString(e));
        l->exec_generation = c->ws.generation;
        l->exec_tuning = c->tuning_generation;
        l->exec_uploads = uploads;
        l->exec_context = c;
    }
    CUDA_TRY(cudaGraphLaunch(l->exec, c->stream));
    for (const Segment &s : l->segments) {
        c->host_stats[0] += s.vertex_count;
        c->host_stats[1] += s.input_triangles;
        c->host_stats[2] += s.draws.size();
        c->host_stats[3] += s.draws.empty() ? 0 : 1;
    }
    c->host_stats[4] += l->launches_per_execution;
    c->pending.push_back({nullptr, nullptr, l, seq});
    if (c->pending.size() > 4096) MLV_TRY(sync_context(c));
    ++l->executions;
    return MLV_OK;
}

MLV_API mlv_status mlv_get_stats(mlv_context c, mlv_stats *out) {
    MLV_TRY(need_immediate(c));
    if (!out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));
    MLV_TRY(ensure_fixed(c));
    unsigned long long dev[kStatCount];
    CUDA_TRY(cudaMemcpy(dev, c->ws.stats, sizeof(dev), cudaMemcpyDeviceToHost));
    out->vertex_count = c->host_stats[0];
    out->input_triangle_count = c->host_stats[1];
    out->assembled_triangle_count = dev[kStatTotal + kStatAssembled];
    out->active_bin_count = dev[kStatTotal + kStatActiveBins];
    out->total_triangle_count_in_bins = dev[kStatTotal + kStatBinEntries];
    out->draw_count = c->host_stats[2];
    out->batch_count = c->host_stats[3];
    out->kernel_launches = c->host_stats[4];
    return MLV_OK;
}

MLV_API mlv_status mlv_reset_stats(mlv_context c) {
    MLV_TRY(need_immediate(c));
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));
    MLV_TRY(ensure_fixed(c));
    CUDA_TRY(zero_now(c->ws.stats, sizeof(unsigned long long) * kStatCount));
    memset(c->host_stats, 0, sizeof(c->host_stats));
    memset(c->stage_ms, 0, sizeof(c->stage_ms));
    memset(c->stage_launches, 0, sizeof(c->stage_launches));
    return MLV_OK;
}

MLV_API mlv_status mlv_get_tuning(mlv_context c, mlv_tuning *out) {
    if (!c || !out) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    *out = c->tuning;
    return MLV_OK;
}

MLV_API mlv_status mlv_set_tuning(mlv_context c, const mlv_tuning *t) {
    if (!c || !t) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    if (t->tile_warps_per_block != 2 && t->tile_warps_per_block != 4 && t->tile_warps_per_block != 8)
        return fail(MLV_ERROR_INVALID_ARG, "tile_warps_per_block must be 2, 4 or 8");
    if (t->warps_per_tile != 1 && t->warps_per_tile != 2 && t->warps_per_tile != 4 && t->warps_per_tile != 8)
        return fail(MLV_ERROR_INVALID_ARG, "warps_per_tile must be 1, 2, 4 or 8");
    if (t->geometry_block != 128 && t->geometry_block != 256 && t->geometry_block != 512)
        return fail(MLV_ERROR_INVALID_ARG, "geometry_block must be 128, 256 or 512");
    if (t->big_triangle_tiles < 1) return fail(MLV_ERROR_INVALID_ARG, "big_triangle_tiles must be >= 1");
    if (t->persistent_launch > 1) return fail(MLV_ERROR_INVALID_ARG, "persistent_launch must be 0 or 1");
    if (t->debug_flags & ~(uint32_t)(MLV_DEBUG_STALL_LOOKBACK | MLV_DEBUG_STALL_GRID))
        return fail(MLV_ERROR_INVALID_ARG, "unknown debug flag");
    if (memcmp(&c->tuning, t, sizeof(*t)) != 0) ++c->tuning_generation;
    c->tuning = *t;
    return MLV_OK;
}

MLV_API mlv_status mlv_set_profiling(mlv_context c, int enable) {
    MLV_TRY(need_immediate(c));
    c->profiling = enable != 0;
    return MLV_OK;
}

MLV_API mlv_status mlv_get_stage_times(mlv_context c, double *ms, uint64_t *launches) {
    MLV_TRY(need_immediate(c));
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));
    for (int i = 0; i < MLV_STAGE_COUNT; ++i) {
        if (ms) ms[i] = c->stage_ms[i];
        if (launches) launches[i] = c->stage_launches[i];
    }
    return MLV_OK;
}

MLV_API mlv_status mlv_set_debug_capture(mlv_context c, int enable) {
    MLV_TRY(need_immediate(c));
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));
    c->capture_infos = enable != 0;
    if (c->capture_infos && c->ws.list && !c->ws.info_mask)
        MLV_TRY(dev_alloc((void **)&c->ws.info_mask, (size_t)c->ws.list_cap * 8));
    ++c->ws.generation;
    return MLV_OK;
}

MLV_API mlv_status mlv_get_tile_infos(mlv_context c, uint32_t *tile_index, uint32_t *tri_id, uint64_t *mask,
                                      uint64_t capacity, uint64_t *out_count) {
    MLV_TRY(need_immediate(c));
    if (!out_count) return fail(MLV_ERROR_INVALID_ARG, "NULL argument");
    MLV_TRY(set_device(c->device));
    MLV_TRY(sync_context(c));
    if (!c->capture_infos || !c->last_single || !c->ws.info_mask)
        return fail(MLV_ERROR_INVALID_STATE, "capture was off or the last batch was not a single draw");
    const uint32_t nb = c->last_total_bins;
    std::vector<uint32_t> start(nb + 1);
    CUDA_TRY(cudaMemcpy(start.data(), c->ws.bin_start, sizeof(uint32_t) * (nb + 1), cudaMemcpyDeviceToHost));
    const uint32_t total = start[nb];
    *out_count = total;
    if (!tile_index || !tri_id || !mask) return MLV_OK;
    if (capacity < total) return fail(MLV_ERROR_INVALID_ARG, "capacity too small");
    std::vector<uint32_t> list(total);
    std::vector<uint64_t> m(total);
    const uint32_t nt = c->last_tris;
    std::vector<uint16_t> info(nt + 1);
    std::vector<uint32_t> rank(nt + 1);
    if (total) {
        CUDA_TRY(cudaMemcpy(list.data(), c->ws.list, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(m.data(), c->ws.info_mask, sizeof(uint64_t) * total, cudaMemcpyDeviceToHost));
    }
    if (nt) {
        CUDA_TRY(cudaMemcpy(info.data(), c->ws.tri_info, sizeof(uint16_t) * nt, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(rank.data(), c->ws.rank, sizeof(uint32_t) * nt, cudaMemcpyDeviceToHost));
    }
    // key (g << 3 | c) -> the reference's triangle id: assembled triangles before g, plus the
    // emitted fans of g before fan c - 1
    auto tri_of = [&](uint32_t key) {
        const uint32_t g = key >> 3, cf = key & 7u;
        const uint32_t fm = info[g] & 0xFFu;
        return rank[g] + (cf ? (uint32_t)__builtin_popcount(fm & ((1u << (cf - 1)) - 1u)) : 0u);
    };
    uint64_t k = 0;
    for (uint32_t b = 0; b < nb; ++b) {
        std::vector<std::pair<uint32_t, uint64_t>> e;
        for (uint32_t i = start[b]; i < start[b + 1]; ++i) e.push_back({tri_of(list[i]), m[i]});
        std::sort(e.begin(), e.end());
        for (auto &pr : e) {
            tile_index[k] = b;
            tri_id[k] = pr.first;
            mask[k] = pr.second;
            ++k;
        }
    }
    return MLV_OK;
}

}  // extern "C"
