// Draw-path kernels for sm_103a.
//
// One batch (any number of draws over any number of render targets) runs as:
//   k_vertex    the vertex shader, once per vertex of each draw's buffer (main.c:698-734 shades
//               once per index; the shader is pure, so the outputs are identical).
//   k_geometry  IA + primitive assembly/clip/setup + per-(tile, draw) bin counts
//               (main.c:662-913 and the counting half of the binner, 924-936). One thread per input
//               triangle; records go to slots indexed by input triangle (see BatchParams), so the
//               reference's serial order is the slot order and no compaction is needed. Triangles
//               that need clipping are listed instead, for
//   k_clip      one warp per listed triangle: clipping (main.c:649-661) and its fans' setup.
//   k_rank      only when visibility or TileInfo outputs are requested: the reference's compact
//               triangle index (its `out_triangle_index`, main.c:873-875), by an exclusive scan of
//               the per-input-triangle output counts.
//   k_scan      exclusive scan of the bin counts (main.c:937-946); k_scan_small for batches of
//               up to 16,384 bins (one CTA).
//   k_scatter   bin lists (main.c:950-962); the order inside a bin does not matter (see k_tile).
//   k_tile      one warp per 8x8 tile: hierarchical Z, coverage, depth, pixel shader, output
//               merger, write-back (main.c:983-1189, 577-603), for every draw of the batch that
//               touches the tile, in draw order, with colour and depth held on-chip until one
//               write-back; the segment's clears of the batch's targets are folded in.
//               k_tile_coop: the same with 2, 4 or 8 warps sharing each tile's triangles.
//   k_fill_many the clears that are not folded (one launch per segment).
//   k_put_descriptors  an eager batch's draw and view descriptors, from the launch's parameters.
//   k_batch     the six stages above as one persistent launch (mlv_tuning::persistent_launch).
// The kernels are launched with programmatic stream serialisation (see pdl_wait).
//
// Why the order inside a bin does not matter: there is no blending (main.c:1180-1181) and pixel
// shaders have no side effects, so after a draw a pixel holds the output of the *last* fragment
// (in assembled order) whose depth is the maximum among the fragments that passed coverage, the
// hierarchical-Z test and `z >= depth at draw start` (GREATER_EQUAL; for LESS, the *first*
// fragment with the minimum depth). That is a max (min) over the 64-bit key (depth, order), which
// the tile kernel computes with shared-memory atomics, then shades only the winner.
#include <cuda_runtime.h>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <utility>

#include "internal.h"
#include "shade.cuh"

namespace mlv {

__constant__ float c_clip_planes[6][4];

// ------------------------------------------------------------------ memory-order helpers

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_volatile_u32(const uint32_t *p) {
    return *(const volatile uint32_t *)p;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// A load of what an earlier stage of the same batch wrote (shaded vertices, clip-fan bases, bin
// starts). The separate kernels read it through the read-only path: its writer was an earlier
// kernel. In the persistent launch (k_batch) the writer is the same kernel, and the read-only path
// is only for data that no thread writes while the kernel runs, so its copies of the stage bodies
// (COHERENT) use an ordinary load with the cache-all-levels hint, which the grid barrier's fences
// make see the other CTAs' writes.
template <bool COHERENT, typename T>
__device__ __forceinline__ T ld_stage(const T *p) {
    if constexpr (COHERENT) return __ldca(p);
    else return __ldg(p);
}

// Programmatic dependent launch: the pipeline's kernels are launched so that the next one may be
// scheduled while the previous one finishes. Each waits for its predecessor's completion (and the
// visibility of its writes) before touching any of its outputs, and lets its dependents launch
// once its own work is done.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

constexpr uint32_t kFlagAggregate = 1, kFlagInclusive = 2;
constexpr uint32_t kSpinLimit = 1u << 22;   // bounded wait: about half a second with the backoff

// Decoupled look-back, run by one full warp. Publishes this block's aggregate, then inspects the
// 32 closest predecessors at once: if every one up to the nearest inclusive prefix is ready, their
// values are summed with one warp reduction; otherwise the window is re-read. Without an
// inclusive prefix in the window, the 32 aggregates are added and the window moves back. Every
// wait is bounded: on timeout the error bit is set and the block still publishes, so no successor
// waits on it. Returns the exclusive prefix in every lane.
__device__ uint32_t lookback_warp(unsigned long long *status, uint32_t bid, uint32_t epoch, uint32_t aggregate,
                                  uint32_t *error) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t ep = epoch & 0x3FFFFFFFu;
    const unsigned long long tag = (unsigned long long)ep << 34;
    if (bid == 0) {
        if (lane == 0) st_release_u64(status, tag | ((unsigned long long)kFlagInclusive << 32) | aggregate);
        return 0;
    }
    if (lane == 0) st_release_u64(status + bid, tag | ((unsigned long long)kFlagAggregate << 32) | aggregate);
    uint32_t prefix = 0;
    int32_t top = (int32_t)bid - 1;
    uint32_t spins = 0;
    while (true) {
        const int32_t j = top - (int32_t)lane;
        uint32_t flag = kFlagInclusive, val = 0;   // before block 0: an inclusive zero ends the walk
        if (j >= 0) {
            const unsigned long long sv = ld_acquire_u64(status + j);
            const uint32_t hi = (uint32_t)(sv >> 32);
            flag = ((hi >> 2) == ep) ? (hi & 3u) : 0u;
            val = (uint32_t)sv;
        }
        const uint32_t incl = __ballot_sync(0xFFFFFFFFu, flag == kFlagInclusive);
        const uint32_t waiting = __ballot_sync(0xFFFFFFFFu, flag == 0);
        const int first = incl ? __ffs(incl) - 1 : 32;
        const uint32_t need = first >= 31 ? 0xFFFFFFFFu : ((2u << first) - 1u);
        if (waiting & need) {
            if (++spins > kSpinLimit) {
                if (lane == 0) atomicOr(error, kErrLookbackTimeout);
                break;
            }
            __nanosleep(32);
            continue;
        }
        uint32_t c = ((int)lane <= first) ? val : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xFFFFFFFFu, c, o);
        prefix += c;
        if (first < 32) break;
        top -= 32;
    }
    if (lane == 0) st_release_u64(status + bid, tag | ((unsigned long long)kFlagInclusive << 32) | (prefix + aggregate));
    return prefix;
}

template <int BLOCK>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *s_warp, uint32_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < BLOCK / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < BLOCK / 32) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[BLOCK / 32 - 1];
    uint32_t warp_prefix = warp ? s_warp[warp - 1] : 0;
    return warp_prefix + x - v;
}

// ------------------------------------------------------------------ primitive setup

// One clip-space vertex as the rest of the pipeline sees it: SV_POSITION + reg1.xyz + U + V.
struct Vtx {
    float v[9];
};

struct Setup {
    int32_t e[9];           // edge0 a,b,c  edge1 a,b,c  edge2 a,b,c
    float inv_area, zbound;
    float ss[3][4];         // screen-space reg0 of the three vertices
    float rw[3];
    int32_t minx, miny, maxx, maxy;      // the reference's pixel box: binning
    int32_t tminx, tminy, tmaxx, tmaxy;  // the same box shrunk to the samples it can cover: tile kernel
};

// set_edge_function, main.c:563-575 (wrapping int32)
__device__ __forceinline__ void set_edge(int32_t *e, int32_t area, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
    uint32_t a = (uint32_t)y0 - (uint32_t)y1;
    uint32_t b = (uint32_t)x1 - (uint32_t)x0;
    if (area < 0) { a = 0u - a; b = 0u - b; }
    uint32_t c = (0u - a) * (uint32_t)x0 - b * (uint32_t)y0;
    e[0] = (int32_t)a; e[1] = (int32_t)b; e[2] = (int32_t)c;
}

// The viewport transform of main.c:823-839, out[r] = ((m[4r]p0 + m[4r+1]p1) + m[4r+2]p2) + m[4r+3]p3,
// for the matrix the host builds (main.c:825-830): its entries 1, 2, 4, 6, 8, 9, 12, 13, 14 are 0
// and entry 15 is 1. With finite inputs, the products by those zeros are signed zeros, which can
// change a row's sum only when the sum is itself zero; so a row is its two other products unless
// that gives zero (or an input is not finite), when the whole product is taken as written.
__device__ __forceinline__ void viewport_transform(const float *m, float p0, float p1, float p2, float p3,
                                                   float *out) {
    const float x = m[0] * p0 + m[3] * p3;
    const float y = m[5] * p1 + m[7] * p3;
    const float z = m[10] * p2 + m[11] * p3;
    const bool finite = fabsf(p0) < INFINITY && fabsf(p1) < INFINITY && fabsf(p2) < INFINITY && fabsf(p3) < INFINITY;
    if (finite && x != 0.0f && y != 0.0f && z != 0.0f && p3 != 0.0f) {
        out[0] = x; out[1] = y; out[2] = z; out[3] = p3;
        return;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) out[r] = dot4_lr(m + 4 * r, p0, p1, p2, p3);
}

// Projection, viewport, 28.4 snap, signed area, cull, edge functions, 1/w, depth bound and pixel
// bounds for one (possibly clip-generated) triangle: main.c:798-904. Returns false when culled.
__device__ __forceinline__ bool setup_triangle(const DrawDesc &d, const Vtx &v0, const Vtx &v1, const Vtx &v2,
                                               Setup &s) {
    const Vtx *tv[3] = {&v0, &v1, &v2};
    const float *m = d.screen_from_ndc;
    int32_t x[3], y[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float rw = 1.0f / tv[k]->v[3];
        float p0 = tv[k]->v[0] * rw, p1 = tv[k]->v[1] * rw, p2 = tv[k]->v[2] * rw, p3 = tv[k]->v[3] * rw;
        s.rw[k] = rw;
        viewport_transform(m, p0, p1, p2, p3, s.ss[k]);
        x[k] = snap28_4(s.ss[k][0]);
        y[k] = snap28_4(s.ss[k][1]);
    }
    int32_t area = (int32_t)(((uint32_t)x[1] - (uint32_t)x[0]) * ((uint32_t)y[2] - (uint32_t)y[0]) -
                             ((uint32_t)x[2] - (uint32_t)x[0]) * ((uint32_t)y[1] - (uint32_t)y[0]));
    if (d.cull == 1 && area > 0) return false;
    if (d.cull == 2 && area < 0) return false;
    set_edge(s.e + 6, area, x[0], y[0], x[1], y[1]);
    set_edge(s.e + 0, area, x[1], y[1], x[2], y[2]);
    set_edge(s.e + 3, area, x[2], y[2], x[0], y[0]);
    if (d.raster_flags & kRasterCenter) {
        // E at (x + 1/2, y + 1/2): ((a x) << 4) + 8 a + ((b y) << 4) + 8 b + c
#pragma unroll
        for (int k = 0; k < 9; k += 3) s.e[k + 2] = (int32_t)((uint32_t)s.e[k + 2] + (((uint32_t)s.e[k] + (uint32_t)s.e[k + 1]) << 3));
    }
    float af = (float)(area >> (kSubpix * 2));
    if (af == 0.0f) af = 1.0f;
    s.inv_area = fabsf(1.f / af);
    if (d.depth_less)
        s.zbound = fmin_ref(s.ss[0][2], fmin_ref(s.ss[1][2], s.ss[2][2]));
    else
        s.zbound = fmax_ref(s.ss[0][2], fmax_ref(s.ss[1][2], s.ss[2][2]));
    int32_t mnx = min(x[0], min(x[1], x[2])) >> kSubpix, mny = min(y[0], min(y[1], y[2])) >> kSubpix;
    int32_t mxx = max(x[0], max(x[1], x[2])) >> kSubpix, mxy = max(y[0], max(y[1], y[2])) >> kSubpix;
    mnx = min(max(mnx, 0), d.vp_w - 1);
    mny = min(max(mny, 0), d.vp_h - 1);
    mxx = min(mxx + 1, d.vp_w - 1);
    mxy = min(mxy + 1, d.vp_h - 1);
    // Every maximum <= -8 bins nowhere and covers no pixel (C division truncates -1..-7 to tile 0,
    // main.c:928), so clamping it there changes nothing and keeps the bounds exact in the 16-bit
    // fields of TriRaster, where the tile kernels read the box.
    mxx = max(mxx, -8);
    mxy = max(mxy, -8);
    s.minx = mnx; s.miny = mny; s.maxx = mxx; s.maxy = mxy;
    // A covered sample lies in the closed triangle, so inside its snapped vertex bounds: x * 16 (+ 8
    // at pixel centres) in [xmin, xmax]. (A degenerate triangle covers none: its edge values are of
    // mixed sign off its line and all 0 on it.) That holds while the edge values are exact, which
    // they are for vertex extents up to 1024 pixels: |E| stays below 2^31 over the box, so the
    // wrapping sums equal the true values. The box shrinks by at most 1 at the minimum and 3 at the
    // maximum.
    const int32_t xlo = min(x[0], min(x[1], x[2])), xhi = max(x[0], max(x[1], x[2]));
    const int32_t ylo = min(y[0], min(y[1], y[2])), yhi = max(y[0], max(y[1], y[2]));
    int32_t dlx = 0, dly = 0, dhx = 0, dhy = 0;
    if ((uint32_t)xhi - (uint32_t)xlo <= 16384u && (uint32_t)yhi - (uint32_t)ylo <= 16384u) {
        const int32_t off = (d.raster_flags & kRasterCenter) ? 8 : 0;
        dlx = min(max(((xlo - off + 15) >> kSubpix) - mnx, 0), 1);
        dly = min(max(((ylo - off + 15) >> kSubpix) - mny, 0), 1);
        dhx = min(max(mxx - ((xhi - off) >> kSubpix), 0), 3);
        dhy = min(max(mxy - ((yhi - off) >> kSubpix), 0), 3);
    }
    s.tminx = mnx + dlx; s.tminy = mny + dly; s.tmaxx = mxx - dhx; s.tmaxy = mxy - dhy;
    return true;
}

// The raster record's four words (TriRaster) of a set-up triangle.
__device__ __forceinline__ void raster_words(const Setup &s, int4 *r) {
    r[0] = make_int4(s.e[0], s.e[1], s.e[2], s.e[3]);
    r[1] = make_int4(s.e[4], s.e[5], s.e[6], s.e[7]);
    r[2] = make_int4(s.e[8], __float_as_int(s.inv_area), __float_as_int(s.zbound), __float_as_int(s.ss[0][2]));
    r[3] = make_int4(__float_as_int(s.ss[1][2]), __float_as_int(s.ss[2][2]),
                     (s.tminx & 0xFFFF) | (s.tminy << 16), (s.tmaxx & 0xFFFF) | (s.tmaxy << 16));
}

__device__ __forceinline__ void write_record(const BatchParams &bp, uint32_t rec, uint32_t draw, int ps,
                                             bool sole_draw, const Setup &s, const Vtx &v0, const Vtx &v1,
                                             const Vtx &v2) {
    int4 w[4];
    raster_words(s, w);
    int4 *r = bp.raster[rec].w;
    r[0] = w[0];
    r[1] = w[1];
    r[2] = w[2];
    r[3] = w[3];
    if (bp.geom) {
        TriGeom &g = bp.geom[rec];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            g.x[k] = s.ss[k][0]; g.y[k] = s.ss[k][1]; g.z[k] = s.ss[k][2]; g.w[k] = s.ss[k][3];
        }
    }
    // A null pixel shader reads no 1/w and no attributes; the tile kernel still takes the draw
    // index from the record when the view has several draws (sole_draw: it has one)
    if (ps == kPsNone && sole_draw) return;
    float4 *h = reinterpret_cast<float4 *>(bp.shade) + (size_t)rec * bp.shade_stride;
    h[0] = make_float4(s.rw[0], s.rw[1], s.rw[2], __uint_as_float(draw));
    if (bp.shade_stride == kShadeUV) {   // the batch's pixel shaders read U (reg1.w) and V (reg2.x) only
        h[1] = make_float4(v0.v[7], v1.v[7], v2.v[7], v0.v[8]);
        h[2] = make_float4(v1.v[8], v2.v[8], 0.0f, 0.0f);
        return;
    }
    h[1] = make_float4(v0.v[4], v0.v[5], v0.v[6], v0.v[7]);
    h[2] = make_float4(v1.v[4], v1.v[5], v1.v[6], v1.v[7]);
    h[3] = make_float4(v2.v[4], v2.v[5], v2.v[6], v2.v[7]);
    h[4] = make_float4(v0.v[8], v1.v[8], v2.v[8], 0.0f);
}

// clip_by_plane, main.c:609-647 (Sutherland-Hodgman on one normalised plane, plane_d = 0), run by a
// whole warp on a polygon in shared memory (poly: count vertices, at most kMaxClipVertices), into
// out. Lane i takes vertex i and the edge from it to the next: the reference's distance, t and
// lerps, each output written where the reference's serial loop puts it (an exclusive warp scan of
// the lanes' emission counts); outputs past kMaxClipVertices are dropped. Returns false, out
// untouched, when every vertex is inside (distance > -0): the reference's pass then gives the
// polygon back unchanged. Every lane calls it with the same count and plane.
__device__ bool clip_by_plane_warp(const Vtx *poly, Vtx *out, int &count, const float *n, int lane) {
    const int nv = count;
    if (nv <= 0) return false;
    const bool mine = lane < nv;
    const float dist = mine ? dot4_lr(n, poly[lane].v[0], poly[lane].v[1], poly[lane].v[2], poly[lane].v[3]) : 0.0f;
    const bool in = mine && dist > -0.0f;
    const uint32_t inm = __ballot_sync(0xFFFFFFFFu, in);
    if (inm == (nv >= 32 ? 0xFFFFFFFFu : (1u << nv) - 1u)) return false;
    const int next = lane + 1 >= nv ? 0 : lane + 1;
    const float dnext = __shfl_sync(0xFFFFFFFFu, dist, next);
    const bool cross = mine && in != (((inm >> next) & 1u) != 0);
    const uint32_t emits = (in ? 1u : 0u) + (cross ? 1u : 0u);
    uint32_t incl = emits;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    uint32_t at = incl - emits;
    if (in && at < (uint32_t)kMaxClipVertices) out[at] = poly[lane];
    if (in) ++at;
    if (cross && at < (uint32_t)kMaxClipVertices) {
        const float t = (0.0f + dist) / (dist - dnext);
        const float omt = 1.f - t;
#pragma unroll
        for (int c = 0; c < 9; ++c) out[at].v[c] = poly[lane].v[c] * omt + poly[next].v[c] * t;
    }
    count = (int)min(total, (uint32_t)kMaxClipVertices);
    __syncwarp();
    return true;
}

__device__ __forceinline__ uint32_t find_draw(const BatchParams &bp, uint32_t tri) {
    uint32_t lo = 0, hi = bp.num_draws;   // last draw with tri_begin <= tri
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&bp.draws[mid].tri_begin) <= tri) lo = mid; else hi = mid;
    }
    return lo;
}

// A CTA's triangles almost always share one draw, found once for all of them (k_direct_raster);
// kNoDraw when they do not.
constexpr uint32_t kNoDraw = 0xFFFFFFFFu;

// The last draw whose begin(d) <= key, for a key uniform over the warp, by the whole warp: each
// round every lane probes one draw of the remaining range (a draw descriptor is a cache line of its
// own, so a halving search waits on one load per step: 10 for 623 draws), and the ballot of the
// probes that are <= key narrows the range 32-fold: two rounds of loads for up to 1,024 draws.
// begin(0) is 0 <= key, so lane 0's probe always holds.
template <typename Begin>
__device__ __forceinline__ uint32_t warp_find_last_le(uint32_t n, uint32_t key, Begin begin, int lane) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t idx = lo + (uint32_t)lane * step;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, idx < hi && begin(idx) <= key);
        lo += (uint32_t)(31 - __clz(m)) * step;
        hi = min(hi, lo + step);
    }
    return lo;
}

// The draw of input triangle g of each lane (consecutive over the warp; a lane at or past the
// batch's end gets 0). Up to 32 draws the warp searches for its first triangle's draw in one round
// of probes, then each lane steps past the draws that begin at or before its own triangle (rarely
// any). With more draws the lanes' halving searches, which follow one path over consecutive
// triangles and so load one descriptor line per step, touch fewer lines than the warp's rounds
// (a 623-draw batch measured 4.07 against 4.16 ms). Every lane calls it.
__device__ __forceinline__ uint32_t warp_find_draw(const BatchParams &bp, uint32_t g, int lane) {
    if (bp.num_draws > 32) return g < bp.total_tris ? find_draw(bp, g) : 0u;   // uniform
    const uint32_t g0 = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g0 >= bp.total_tris) return 0;   // uniform: the whole warp is past the end
    uint32_t d = warp_find_last_le(bp.num_draws, g0, [&](uint32_t i) { return __ldg(&bp.draws[i].tri_begin); },
                                   lane);
    if (g < bp.total_tris)
        while (d + 1 < bp.num_draws && __ldg(&bp.draws[d + 1].tri_begin) <= g) ++d;
    return d;
}

__device__ __forceinline__ void fetch_vertex(const DrawDesc &d, uint32_t idx_pos, float *in, uint32_t *warn) {
    int64_t idx = d.ib ? (int64_t)__ldg(d.ib + idx_pos) : (int64_t)idx_pos;
    idx += d.base_vertex;
    if (idx < 0 || idx >= (int64_t)d.vertex_count) {
        atomicOr(warn, kErrBadIndex);
#pragma unroll
        for (int k = 0; k < 8; ++k) in[k] = 0.0f;   // D3D11: out-of-range vertex fetch reads zeros
        return;
    }
    const uint8_t *p = d.vb + (size_t)idx * d.vb_stride;
    if ((((uintptr_t)p) & 15) == 0) {
        float4 a = __ldg((const float4 *)p), b = __ldg((const float4 *)p + 1);
        in[0] = a.x; in[1] = a.y; in[2] = a.z; in[3] = a.w; in[4] = b.x; in[5] = b.y; in[6] = b.z; in[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) in[k] = __ldg((const float *)p + k);
    }
}

__device__ __forceinline__ void tile_range(const ViewDesc &v, int32_t minx, int32_t miny, int32_t maxx, int32_t maxy,
                                           int32_t &tx0, int32_t &ty0, int32_t &tx1, int32_t &ty1) {
    // binner, main.c:927-928 (C division truncates toward zero)
    tx0 = max(minx / kTile, 0);
    ty0 = max(miny / kTile, 0);
    tx1 = min(maxx / kTile, (int32_t)v.tiles_x - 1);
    ty1 = min(maxy / kTile, (int32_t)v.tiles_y - 1);
}

// ------------------------------------------------------------------ unique-vertex shading

// The reference shades one vertex per index (main.c:673, "no post-transform cache"). A vertex
// shader is a pure function of its input, so shading every vertex of the buffer once gives
// bit-identical outputs; k_geometry then gathers them by index.
constexpr int kVertexBlock = 256;

// The vertex shading of block blk (kVertexBlock vertices); k_vertex and the persistent launch run it.
__device__ __forceinline__ void vertex_body(const BatchParams &bp, uint32_t blk) {
    const uint32_t v = blk * kVertexBlock + threadIdx.x;
    // the draw of each lane's vertex: the last draw whose range in vs_out begins at or before it,
    // by warp_find_draw's scheme (vertices are consecutive over the warp)
    uint32_t di;
    if (bp.num_draws > 32) {   // uniform
        if (v >= bp.total_vertices) return;
        uint32_t lo = 0, hi = bp.num_draws;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(&bp.draws[mid].vs_base) <= v) lo = mid; else hi = mid;
        }
        di = lo;
    } else {
        const uint32_t v0 = __shfl_sync(0xFFFFFFFFu, v, 0);
        if (v0 >= bp.total_vertices) return;   // uniform
        di = warp_find_last_le(bp.num_draws, v0, [&](uint32_t i) { return __ldg(&bp.draws[i].vs_base); },
                               (int)(threadIdx.x & 31));
        if (v >= bp.total_vertices) return;
        while (di + 1 < bp.num_draws && __ldg(&bp.draws[di + 1].vs_base) <= v) ++di;
    }
    const DrawDesc &d = bp.draws[di];
    const uint32_t local = v - d.vs_base;
    const uint8_t *p = d.vb + (size_t)local * d.vb_stride;
    float in[8];
    if ((((uintptr_t)p) & 15) == 0) {
        float4 a = __ldg((const float4 *)p), b = __ldg((const float4 *)p + 1);
        in[0] = a.x; in[1] = a.y; in[2] = a.z; in[3] = a.w; in[4] = b.x; in[5] = b.y; in[6] = b.z; in[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) in[k] = __ldg((const float *)p + k);
    }
    float o[9];
    run_vs(d.vs, in, d.cb, d.vs_tex, o);
    // positions densely first (the gathers of the clip tests and setup read nothing else, and
    // neighbouring vertices share cache sectors), the attributes after all positions; a null pixel
    // shader reads no attributes
    bp.vs_out[v] = make_float4(o[0], o[1], o[2], o[3]);
    if (d.ps != kPsNone) {
        if (bp.shade_stride == kShadeUV) {   // the batch's pixel shaders read U and V only
            reinterpret_cast<float2 *>(bp.vs_out + bp.total_vertices)[v] = make_float2(o[7], o[8]);
        } else {
            float4 *attr = bp.vs_out + bp.total_vertices + 2 * (size_t)v;
            attr[0] = make_float4(o[4], o[5], o[6], o[7]);
            attr[1] = make_float4(o[8], 0.0f, 0.0f, 0.0f);
        }
    }
}

__global__ void __launch_bounds__(kVertexBlock) k_vertex(BatchParams bp) {
    pdl_wait();
    vertex_body(bp, blockIdx.x);
    pdl_trigger();
}

// The attributes of shaded vertex `slot` (o[4..8]: reg1.xyzw, reg2.x) from the shaded-vertex
// buffer: two float4s a vertex, or in a batch whose pixel shaders read only U and V, (U, V), with
// reg1.xyz, which no such shader reads, left zero.
template <bool COHERENT = false>
__device__ __forceinline__ void load_attributes(const BatchParams &bp, size_t slot, float *o) {
    if (bp.shade_stride == kShadeUV) {
        const float2 uv = ld_stage<COHERENT>(reinterpret_cast<const float2 *>(bp.vs_out + bp.total_vertices) + slot);
        o[4] = o[5] = o[6] = 0.0f;
        o[7] = uv.x;
        o[8] = uv.y;
        return;
    }
    const float4 *attr = bp.vs_out + bp.total_vertices + 2 * slot;
    const float4 b = ld_stage<COHERENT>(attr), c = ld_stage<COHERENT>(attr + 1);
    o[4] = b.x; o[5] = b.y; o[6] = b.z; o[7] = b.w; o[8] = c.x;
}

// Vertex k of a triangle: from the shaded-vertex buffer, or shaded here (per-index path, and for
// out-of-range indices, which read zeros as in Direct3D 11).
template <bool COHERENT = false>
__device__ __forceinline__ void triangle_vertex(const BatchParams &bp, const DrawDesc &d, uint32_t idx_pos, float *o) {
    if (d.vs_cached) {
        int64_t idx = d.ib ? (int64_t)__ldg(d.ib + idx_pos) : (int64_t)idx_pos;
        idx += d.base_vertex;
        if (idx >= 0 && idx < (int64_t)d.vertex_count) {
            const size_t slot = (size_t)d.vs_base + (size_t)idx;
            const float4 a = ld_stage<COHERENT>(bp.vs_out + slot);
            o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
            if (d.ps == kPsNone) {   // positions only (see k_vertex)
                o[4] = o[5] = o[6] = o[7] = o[8] = 0.0f;
                return;
            }
            load_attributes<COHERENT>(bp, slot, o);
            return;
        }
    }
    float in[8];
    fetch_vertex(d, idx_pos, in, bp.error + 2);
    run_vs(d.vs, in, d.cb, d.vs_tex, o);
}

// The position of vertex k of a triangle, for the clip tests and setup; its attributes are read
// only once the triangle survives them (triangle_attributes), as most triangles of a large scene
// do not. Returns the vertex's slot in the shaded-vertex buffer, or kNoSlot when o already holds
// the whole vertex (shaded here, or a null pixel shader, which reads no attributes).
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;

template <bool COHERENT = false>
__device__ __forceinline__ uint32_t triangle_position(const BatchParams &bp, const DrawDesc &d, uint32_t idx_pos,
                                                      float *o) {
    if (d.vs_cached && d.ps != kPsNone) {
        int64_t idx = d.ib ? (int64_t)__ldg(d.ib + idx_pos) : (int64_t)idx_pos;
        idx += d.base_vertex;
        if (idx >= 0 && idx < (int64_t)d.vertex_count) {
            const uint32_t slot = d.vs_base + (uint32_t)idx;
            const float4 a = ld_stage<COHERENT>(bp.vs_out + slot);
            o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
            return slot;
        }
    }
    triangle_vertex<COHERENT>(bp, d, idx_pos, o);
    return kNoSlot;
}

template <bool COHERENT = false>
__device__ __forceinline__ void triangle_attributes(const BatchParams &bp, uint32_t slot, float *o) {
    if (slot == kNoSlot) return;
    load_attributes<COHERENT>(bp, slot, o);
}

// Slot of the record a triangle key names (see BatchParams).
template <bool COHERENT = false>
__device__ __forceinline__ uint32_t record_of(const BatchParams &bp, uint32_t key) {
    const uint32_t g = key >> 3, c = key & 7u;
    if (c == 0) return g;
    return bp.total_tris + (uint32_t)ld_stage<COHERENT>(&bp.raster[g].w[0].x) + (c - 1);
}

// The tiles (bins) of one emitted triangle from its clamped pixel bounds: the binner's tile range
// (main.c:924-936). k_geometry counts them and k_scatter fills them; both call this on the same
// bounds (k_scatter re-reads them from the raster record), so they agree on every bin.
__device__ __forceinline__ bool bin_job(const ViewDesc &vw, uint32_t draw_in_view, int32_t minx, int32_t miny,
                                        int32_t maxx, int32_t maxy, uint32_t key, BinJob &job) {
    int32_t tx0, ty0, tx1, ty1;
    tile_range(vw, minx, miny, maxx, maxy, tx0, ty0, tx1, ty1);
    job.key = key;
    job.nx = tx1 >= tx0 ? (uint32_t)(tx1 - tx0 + 1) : 0u;
    job.ny = ty1 >= ty0 ? (uint32_t)(ty1 - ty0 + 1) : 0u;
    job.col_stride = vw.draw_count;
    job.row_stride = vw.tiles_x * vw.draw_count;
    job.first_bin = vw.bin_base + ((uint32_t)max(ty0, 0) * vw.tiles_x + (uint32_t)max(tx0, 0)) * vw.draw_count +
                    draw_in_view;
    job.pad0 = job.pad1 = 0;
    return job.nx != 0 && job.ny != 0;
}

__device__ __forceinline__ uint32_t job_bin(const BinJob &j, uint32_t t) {
    const uint32_t y = t / j.nx, x = t - y * j.nx;
    return j.first_bin + y * j.row_stride + x * j.col_stride;
}


// Appends the bin job of every lane with one (has) to the batch's job list, one atomic per warp:
// its key, first bin, tile counts and view, which k_scatter fills from. Lanes of a warp hold
// neighbouring triangles, which stay neighbours in the list. Every lane of the warp calls it.
__device__ __forceinline__ void push_jobs(const BatchParams &bp, bool has, const BinJob &job, uint32_t view, int lane) {
    const uint32_t lanes = __ballot_sync(0xFFFFFFFFu, has);
    if (!lanes) return;
    uint32_t at = 0;
    if (lane == 0) at = atomicAdd(bp.counters + kCtrJobs, (uint32_t)__popc(lanes));
    at = __shfl_sync(0xFFFFFFFFu, at, 0) + (uint32_t)__popc(lanes & ((1u << lane) - 1u));
    if (!has) return;
    if (at < bp.jobs_capacity) bp.jobs[at] = make_uint4(job.key, job.first_bin, job.nx | (job.ny << 16), view);
    else atomicOr(bp.error, kErrRecordOverflow);   // cannot happen: a job per record slot at most
}

// Resident threads per SM the geometry kernel's register budget is sized for (1024: 64 registers).
#ifndef MLV_GEOMETRY_THREADS_PER_SM
#define MLV_GEOMETRY_THREADS_PER_SM 1024
#endif

// Input triangle g of each lane (32 consecutive ones), by one whole warp; k_geometry and the
// persistent launch run it.
template <bool COHERENT = false>
__device__ __forceinline__ void geometry_warp(const BatchParams &bp, uint32_t g) {
    const int lane = threadIdx.x & 31;
    uint32_t draw = 0, view = 0;
    bool clipped = false;       // left to k_clip
    uint32_t mask = 0;
    BinJob own;                 // the bins of an unclipped triangle, counted warp-wide below
    bool have_own = false;
    uint32_t ghost_entries = 0; // bins of a triangle that covers no sample (statistics only)
    uint32_t ghost_bin = 0xFFFFFFFFu;   // its bin when it has one, marked warp-wide below
    const uint32_t lane_draw = warp_find_draw(bp, g, lane);
    if (g < bp.total_tris) {
        draw = lane_draw;
        const DrawDesc &d = bp.draws[draw];
        view = d.view;
        const ViewDesc &vw = bp.views[view];
        const uint32_t local = g - d.tri_begin;
        Vtx v[3];
        uint32_t slot[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) slot[k] = triangle_position<COHERENT>(bp, d, d.start_index + 3 * local + k, v[k].v);
        const float *p0 = v[0].v, *p1 = v[1].v, *p2 = v[2].v;
        // main.c:759-781
        bool reject = p0[3] == 0 || p1[3] == 0 || p2[3] == 0;
        reject = reject || (p0[0] < -p0[3] && p1[0] < -p1[3] && p2[0] < -p2[3]) ||
                 (p0[0] > +p0[3] && p1[0] > +p1[3] && p2[0] > +p2[3]) ||
                 (p0[1] < -p0[3] && p1[1] < -p1[3] && p2[1] < -p2[3]) ||
                 (p0[1] > +p0[3] && p1[1] > +p1[3] && p2[1] > +p2[3]) ||
                 (p0[2] < 0.f && p1[2] < 0.f && p2[2] < 0.f) ||
                 (p0[2] > +p0[3] && p1[2] > +p1[3] && p2[2] > +p2[3]);
        if (!reject) {
            clipped = !((p0[0] >= -p0[3] && p1[0] >= -p1[3] && p2[0] >= -p2[3]) &&
                        (p0[0] <= +p0[3] && p1[0] <= +p1[3] && p2[0] <= +p2[3]) &&
                        (p0[1] >= -p0[3] && p1[1] >= -p1[3] && p2[1] >= -p2[3]) &&
                        (p0[1] <= +p0[3] && p1[1] <= +p1[3] && p2[1] <= +p2[3]) &&
                        (p0[2] >= 0.f && p1[2] >= 0.f && p2[2] >= 0.f) &&
                        (p0[2] <= +p0[3] && p1[2] <= +p1[3] && p2[2] <= +p2[3]));
            if (!clipped) {
                Setup su;
                if (setup_triangle(d, v[0], v[1], v[2], su)) {
                    // A triangle whose sample box is empty covers no sample: the reference bins it
                    // (its statistics count it) but it can write nothing, so it gets no record and
                    // no list entries, only its bins' activity (see the counting below). Kept
                    // whole when TileInfo masks are captured (the reference's list them, empty).
                    const bool ghost = bp.info_mask == nullptr && (su.tminx > su.tmaxx || su.tminy > su.tmaxy);
                    mask = 1;
                    if (!ghost) {
#pragma unroll
                        for (int k = 0; k < 3; ++k) triangle_attributes<COHERENT>(bp, slot[k], v[k].v);
                        write_record(bp, g, draw, d.ps, !(d.raster_flags & kDrawSharesView), su, v[0], v[1], v[2]);
                        have_own = bin_job(vw, d.draw_in_view, su.minx, su.miny, su.maxx, su.maxy, g << 3, own);
                    } else {
                        // its bins are only marked active (bit 31 of the count, which k_scan counts
                        // as activity and clears); the entry statistic is added below
                        BinJob job;
                        if (bin_job(vw, d.draw_in_view, su.minx, su.miny, su.maxx, su.maxy, 0u, job)) {
                            ghost_entries = job.nx * job.ny;
                            if (ghost_entries == 1) ghost_bin = job.first_bin;
                            else
                                for (uint32_t t = 0; t < ghost_entries; ++t)
                                    atomicOr(bp.bin_count + job_bin(job, t), kBinGhost);
                        }
                    }
                }
            }
            // a triangle that needs clipping is listed for k_clip, which writes its fans, their
            // bin jobs and its tri_info after this kernel
        }
        if (!clipped) bp.tri_info[g] = (uint16_t)mask;
    }
    push_jobs(bp, have_own, own, view, lane);
    const uint32_t clip_lanes = __ballot_sync(0xFFFFFFFFu, clipped);
    if (clip_lanes) {   // one position per warp in the clip list
        uint32_t at = 0;
        if (lane == 0) at = atomicAdd(bp.counters + kCtrClip, (uint32_t)__popc(clip_lanes));
        at = __shfl_sync(0xFFFFFFFFu, at, 0);
        const uint32_t slot = at + __popc(clip_lanes & ((1u << lane) - 1u));
        // below total_tris (the list's size) while the per-batch counters start at zero, as they
        // do except behind a failed batch (error word set; such batches are re-run)
        if (clipped && slot < bp.total_tris) bp.clip_list[slot] = make_uint2(g, draw);
    }
    if (!__any_sync(0xFFFFFFFFu, mask != 0u)) return;   // the warp assembled nothing: nothing to count
    // assembled-triangle statistic (main.c:1238)
    uint32_t n = __popc(mask);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xFFFFFFFFu, n, o);
    if (lane == 0 && n) atomicAdd(bp.stats + kStatAssembled, (unsigned long long)n);
    // triangles without samples: their bins for the entry statistic (main.c:937-944), and the
    // one-tile ones' activity marks, one per distinct bin per warp
    if (__any_sync(0xFFFFFFFFu, ghost_entries != 0)) {
        uint32_t ge = ghost_entries;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ge += __shfl_xor_sync(0xFFFFFFFFu, ge, o);
        if (lane == 0) atomicAdd(bp.stats + kStatBinEntries, (unsigned long long)ge);
        const uint32_t gpeers = __match_any_sync(0xFFFFFFFFu, ghost_bin);
        if (ghost_bin != 0xFFFFFFFFu && lane == __ffs(gpeers) - 1) atomicOr(bp.bin_count + ghost_bin, kBinGhost);
    }
    // neighbouring triangles of a mesh mostly share their tile: one update per distinct bin
    const uint32_t nt_own = have_own ? own.nx * own.ny : 0u;
    const uint32_t single_bin = nt_own == 1 ? own.first_bin : 0xFFFFFFFFu;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, single_bin);
    if (single_bin != 0xFFFFFFFFu && lane == __ffs(peers) - 1)
        atomicAdd(bp.bin_count + single_bin, (uint32_t)__popc(peers));
    if (nt_own > 1 && nt_own <= bp.big_tiles)
        for (uint32_t t = 0; t < nt_own; ++t) atomicAdd(bp.bin_count + job_bin(own, t), 1u);
    // triangles spanning many tiles: the warp counts their tiles together
    uint32_t big = __ballot_sync(0xFFFFFFFFu, nt_own > bp.big_tiles);
    while (big) {
        const int src = __ffs(big) - 1;
        big &= big - 1;
        BinJob j;
        j.first_bin = __shfl_sync(0xFFFFFFFFu, own.first_bin, src);
        j.nx = __shfl_sync(0xFFFFFFFFu, own.nx, src);
        j.ny = __shfl_sync(0xFFFFFFFFu, own.ny, src);
        j.col_stride = __shfl_sync(0xFFFFFFFFu, own.col_stride, src);
        j.row_stride = __shfl_sync(0xFFFFFFFFu, own.row_stride, src);
        for (uint32_t t = lane; t < j.nx * j.ny; t += 32) atomicAdd(bp.bin_count + job_bin(j, t), 1u);
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, MLV_GEOMETRY_THREADS_PER_SM / BLOCK) k_geometry(BatchParams bp) {
    pdl_wait();
    geometry_warp(bp, blockIdx.x * BLOCK + threadIdx.x);
    pdl_trigger();
}

// Clipping (main.c:649-661) of the triangles k_geometry listed, one warp per triangle: lanes 0-2
// fetch its vertices again, the warp clips them plane by plane (clip_by_plane_warp), and lane f sets
// up fan f (main.c:662-913): its record in slot total_tris + base + f, its bins counted (by the warp
// together when it spans more than big_tiles). Then the triangle's fan mask, clipped bit and box
// deltas are written where k_geometry writes an unclipped triangle's. Spread over the whole GPU,
// the clipped triangles' serial work no longer lengthens the warps of k_geometry that hold them.
constexpr int kClipBlock = 128;

template <int WARPS>
struct ClipSmem {
    Vtx poly[WARPS][2][kMaxClipVertices];   // each warp's polygon and its clipped copy
};

// The listed triangles of CTA blk of nblk, a warp per triangle (WARPS warps a CTA); k_clip and the
// persistent launch run it.
template <int WARPS, bool COHERENT = false>
__device__ __forceinline__ void clip_body(const BatchParams &bp, uint32_t blk, uint32_t nblk, ClipSmem<WARPS> &sm) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // behind a failed batch (error word set) the counters need not have started at zero, and the
    // batch is re-run anyway: nothing to clip. Decided per warp (another warp's clip may set the
    // word meanwhile, and the warp's lanes clip together)
    if (__any_sync(0xFFFFFFFFu, ld_volatile_u32(bp.error) != 0u)) return;
    const uint32_t n = min(ld_volatile_u32(bp.counters + kCtrClip), bp.total_tris);
    uint32_t assembled = 0;
    for (uint32_t i = blk * WARPS + warp; i < n; i += nblk * WARPS) {
        const uint2 entry = bp.clip_list[i];
        const uint32_t g = entry.x, draw = entry.y;
        const DrawDesc &d = bp.draws[draw];
        Vtx *poly = sm.poly[warp][0], *other = sm.poly[warp][1];
        if (lane < 3) triangle_vertex<COHERENT>(bp, d, d.start_index + 3 * (g - d.tri_begin) + (uint32_t)lane, poly[lane].v);
        __syncwarp();
        int count = 3;
        for (int p = 0; p < 6; ++p)
            if (clip_by_plane_warp(poly, other, count, c_clip_planes[p], lane)) {
                Vtx *t = poly;
                poly = other;
                other = t;
            }
        const int nf = count - 2;
        uint32_t fans = 0;
        if (nf > 0) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(bp.counters + kCtrOverflow, (uint32_t)nf);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + (uint32_t)nf > bp.overflow_capacity) {
                if (lane == 0) {
                    atomicOr(bp.error, kErrRecordOverflow);
                    atomicMin(bp.error + 1, bp.batch_seq);
                    atomicMax(bp.error + 4, base + (uint32_t)nf);
                }
            } else {
                Setup su;
                bool ok = false;
                BinJob job;
                uint32_t nt = 0;
                if (lane < min(nf, 7)) {
                    ok = setup_triangle(d, poly[0], poly[lane + 1], poly[lane + 2], su);
                    if (ok) {
                        write_record(bp, bp.total_tris + base + (uint32_t)lane, draw, d.ps,
                                     !(d.raster_flags & kDrawSharesView), su, poly[0], poly[lane + 1], poly[lane + 2]);
                        if (bin_job(bp.views[d.view], d.draw_in_view, su.minx, su.miny, su.maxx, su.maxy,
                                    (g << 3) | (uint32_t)(lane + 1), job))
                            nt = job.nx * job.ny;
                        if (nt <= bp.big_tiles)
                            for (uint32_t t = 0; t < nt; ++t) atomicAdd(bp.bin_count + job_bin(job, t), 1u);
                    }
                }
                fans = __ballot_sync(0xFFFFFFFFu, ok);
                // fans over many tiles: their bins counted by the whole warp
                uint32_t big = __ballot_sync(0xFFFFFFFFu, nt > bp.big_tiles);
                while (big) {
                    const int src = __ffs(big) - 1;
                    big &= big - 1;
                    BinJob j;
                    j.first_bin = __shfl_sync(0xFFFFFFFFu, job.first_bin, src);
                    j.nx = __shfl_sync(0xFFFFFFFFu, job.nx, src);
                    j.ny = __shfl_sync(0xFFFFFFFFu, job.ny, src);
                    j.col_stride = __shfl_sync(0xFFFFFFFFu, job.col_stride, src);
                    j.row_stride = __shfl_sync(0xFFFFFFFFu, job.row_stride, src);
                    for (uint32_t t = lane; t < j.nx * j.ny; t += 32) atomicAdd(bp.bin_count + job_bin(j, t), 1u);
                }
                push_jobs(bp, nt != 0, job, d.view, lane);
                // slot g (no record of its own) holds the fans' base
                if (lane == 0) bp.raster[g].w[0] = make_int4((int)base, 0, 0, 0);
            }
        }
        if (lane == 0) bp.tri_info[g] = (uint16_t)(fans | 0x100u);
        assembled += (uint32_t)__popc(fans);
        __syncwarp();
    }
    if (lane == 0 && assembled) atomicAdd(bp.stats + kStatAssembled, (unsigned long long)assembled);   // main.c:1238
}

__global__ void __launch_bounds__(kClipBlock) k_clip(BatchParams bp) {
    __shared__ ClipSmem<kClipBlock / 32> sm;
    pdl_wait();
    clip_body<kClipBlock / 32>(bp, blockIdx.x, gridDim.x, sm);
    pdl_trigger();
}

// ------------------------------------------------------------------ assembled-triangle ranks

constexpr int kRankBlock = 256, kRankItems = 8;

// Shared state of one block of a decoupled look-back scan (k_rank, k_scan).
struct ScanSmem {
    uint32_t bid, epoch, prefix;
    uint32_t warp[8];
};

// The scans' block order: a separate kernel takes it from a ticket, in the order its blocks start,
// so that a block only ever waits on blocks that already run. The persistent launch gives block
// b = CTA + k * CTAs to its CTAs in increasing k: all of them are resident and each finishes its
// blocks in order, so every block a block waits on is done or running.
constexpr uint32_t kTicket = 0xFFFFFFFFu;

// rank[g] = number of triangles input triangles 0..g-1 of the batch assembled (exclusive scan of
// the popcount of tri_info's fan masks), same decoupled look-back as k_scan. Block `block` of
// nblk (kTicket: from the ticket counter).
__device__ __forceinline__ void rank_body(const BatchParams &bp, uint32_t block, uint32_t nblk, ScanSmem &sm) {
    uint32_t &s_bid = sm.bid, &s_epoch = sm.epoch, &s_prefix = sm.prefix;
    uint32_t *s_warp = sm.warp;
    static_assert(kRankBlock / 32 <= 8, "ScanSmem::warp");
    if (threadIdx.x == 0) {
        s_bid = block == kTicket ? atomicAdd(bp.counters + kCtrRankTicket, 1u) : block;
        s_epoch = ld_volatile_u32(bp.counters + kCtrRankEpoch);
    }
    __syncthreads();
    const uint32_t bid = s_bid;
    const uint32_t n = bp.total_tris;
    const uint32_t base = bid * kRankBlock * kRankItems + threadIdx.x * kRankItems;
    uint32_t vals[kRankItems];
    uint32_t sum = 0;
#pragma unroll
    for (int i = 0; i < kRankItems; ++i) {
        uint32_t idx = base + i;
        vals[i] = idx < n ? (uint32_t)__popc(bp.tri_info[idx] & 0xFFu) : 0u;
        sum += vals[i];
    }
    uint32_t total;
    uint32_t excl = block_exclusive_scan<kRankBlock>(sum, s_warp, total);
    if (threadIdx.x < 32) {
        const uint32_t p = lookback_warp(bp.scan_status, bid, s_epoch, total, bp.error);
        if (threadIdx.x == 0) s_prefix = p;
    }
    __syncthreads();
    uint32_t run = s_prefix + excl;
#pragma unroll
    for (int i = 0; i < kRankItems; ++i) {
        uint32_t idx = base + i;
        if (idx < n) bp.rank[idx] = run;
        run += vals[i];
    }
    if (threadIdx.x == 0) {
        __threadfence();
        uint32_t done = atomicAdd(bp.counters + kCtrRankDone, 1u);
        if (done == nblk - 1) {
            bp.counters[kCtrRankTicket] = 0;
            bp.counters[kCtrRankDone] = 0;
            bp.counters[kCtrRankEpoch] = s_epoch + 1;
            __threadfence();
        }
    }
}

__global__ void __launch_bounds__(kRankBlock) k_rank(BatchParams bp) {
    __shared__ ScanSmem sm;
    pdl_wait();
    rank_body(bp, kTicket, gridDim.x, sm);
    pdl_trigger();
}

// ------------------------------------------------------------------ bin scan

constexpr int kScanBlock = 256, kScanItems = 16;   // 4096 bins per block, read as 4 x uint4 per thread

// Block `block` of nblk of the bin scan (kTicket: from the ticket counter).
__device__ __forceinline__ void scan_body(const BatchParams &bp, uint32_t block, uint32_t nblk, ScanSmem &sm) {
    uint32_t &s_bid = sm.bid, &s_epoch = sm.epoch, &s_prefix = sm.prefix;
    uint32_t *s_warp = sm.warp;
    static_assert(kScanBlock / 32 <= 8, "ScanSmem::warp");
    if (threadIdx.x == 0) {
        s_bid = block == kTicket ? atomicAdd(bp.counters + kCtrScanTicket, 1u) : block;
        s_epoch = ld_volatile_u32(bp.counters + kCtrScanEpoch);
    }
    __syncthreads();
    const uint32_t bid = s_bid;
    const uint32_t n = bp.total_bins;
    const uint32_t base = bid * kScanBlock * kScanItems + threadIdx.x * kScanItems;
    uint32_t vals[kScanItems];
    uint32_t sum = 0, active = 0;
    if (base + kScanItems <= n) {
        // bin_count is 16-byte aligned (cudaMalloc) and base is a multiple of 16
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 v4 = reinterpret_cast<const uint4 *>(bp.bin_count + base)[q];
            vals[4 * q] = v4.x; vals[4 * q + 1] = v4.y; vals[4 * q + 2] = v4.z; vals[4 * q + 3] = v4.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) vals[i] = base + i < n ? bp.bin_count[base + i] : 0u;
    }
    // bit 31: only triangles without samples (k_geometry) were binned here; active, no entries
    uint32_t ghosts = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        active += vals[i] ? 1u : 0u;
        ghosts |= (vals[i] >> 31) << i;
        vals[i] &= ~kBinGhost;
        sum += vals[i];
    }
    uint32_t total;
    uint32_t excl = block_exclusive_scan<kScanBlock>(sum, s_warp, total);
    if (threadIdx.x < 32) {
        // failure-detection tests (kDebugStallLookback): block 0 never publishes its prefix, so the
        // bounded waits of the blocks after it run out (error bit set, they publish and go on)
        const bool stall = bid == 0 && (bp.debug_flags & kDebugStallLookback);
        const uint32_t p = stall ? 0u : lookback_warp(bp.scan_status2, bid, s_epoch, total, bp.error);
        if (threadIdx.x == 0) s_prefix = p;
    }
    __syncthreads();
    uint32_t run = s_prefix + excl;
    uint32_t outv[kScanItems];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        outv[i] = run;
        run += vals[i];
    }
    if (ghosts) {   // the count is k_scatter's cursor and must end at 0: clear the mark
#pragma unroll
        for (int i = 0; i < kScanItems; ++i)
            if (ghosts >> i & 1u) bp.bin_count[base + i] = vals[i];
    }
    if (base + kScanItems <= n) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q)
            reinterpret_cast<uint4 *>(bp.bin_start + base)[q] =
                make_uint4(outv[4 * q], outv[4 * q + 1], outv[4 * q + 2], outv[4 * q + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i)
            if (base + i < n) bp.bin_start[base + i] = outv[i];
    }
    // active-bin statistic (main.c:937-944)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) active += __shfl_xor_sync(0xFFFFFFFFu, active, o);
    if ((threadIdx.x & 31) == 0 && active) atomicAdd(bp.stats + kStatActiveBins, (unsigned long long)active);
    if (threadIdx.x == 0) {
        if (bid == nblk - 1) {
            bp.bin_start[n] = s_prefix + total;
            atomicAdd(bp.stats + kStatBinEntries, (unsigned long long)(s_prefix + total));
        }
        __threadfence();
        uint32_t done = atomicAdd(bp.counters + kCtrScanDone, 1u);
        if (done == nblk - 1) {
            bp.counters[kCtrScanTicket] = 0;
            bp.counters[kCtrScanDone] = 0;
            bp.counters[kCtrScanEpoch] = s_epoch + 1;
            __threadfence();
        }
    }
}

__global__ void __launch_bounds__(kScanBlock) k_scan(BatchParams bp) {
    __shared__ ScanSmem sm;
    pdl_wait();
    if (ld_volatile_u32(bp.error)) return;   // uniform: set only by earlier kernels
    scan_body(bp, kTicket, gridDim.x, sm);
    pdl_trigger();
}

// The same scan for batches of up to kSmallScanBins bins, in one CTA: no look-back, no tickets,
// so a small frame (one draw at 1280x720: 14,400 bins) does not wait on a chain of CTAs.
constexpr int kSmallScanBlock = 1024;
constexpr uint32_t kSmallScanBins = kSmallScanBlock * kScanItems;

__global__ void __launch_bounds__(kSmallScanBlock) k_scan_small(BatchParams bp) {
    __shared__ uint32_t s_warp[kSmallScanBlock / 32];
    pdl_wait();
    if (ld_volatile_u32(bp.error)) return;   // uniform: set only by earlier kernels
    const uint32_t n = bp.total_bins;
    const uint32_t base = threadIdx.x * kScanItems;
    uint32_t vals[kScanItems];
    if (base + kScanItems <= n) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 v4 = reinterpret_cast<const uint4 *>(bp.bin_count + base)[q];
            vals[4 * q] = v4.x; vals[4 * q + 1] = v4.y; vals[4 * q + 2] = v4.z; vals[4 * q + 3] = v4.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) vals[i] = base + i < n ? bp.bin_count[base + i] : 0u;
    }
    uint32_t sum = 0, active = 0, ghosts = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {   // bit 31: a bin of triangles without samples only
        active += vals[i] ? 1u : 0u;
        ghosts |= (vals[i] >> 31) << i;
        vals[i] &= ~kBinGhost;
        sum += vals[i];
    }
    uint32_t total;
    uint32_t run = block_exclusive_scan<kSmallScanBlock>(sum, s_warp, total);
    if (ghosts) {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i)
            if (ghosts >> i & 1u) bp.bin_count[base + i] = vals[i];
    }
    uint32_t outv[kScanItems];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        outv[i] = run;
        run += vals[i];
    }
    if (base + kScanItems <= n) {
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q)
            reinterpret_cast<uint4 *>(bp.bin_start + base)[q] =
                make_uint4(outv[4 * q], outv[4 * q + 1], outv[4 * q + 2], outv[4 * q + 3]);
    } else {
#pragma unroll
        for (int i = 0; i < kScanItems; ++i)
            if (base + i < n) bp.bin_start[base + i] = outv[i];
    }
    // active-bin statistic (main.c:937-944)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) active += __shfl_xor_sync(0xFFFFFFFFu, active, o);
    if ((threadIdx.x & 31) == 0 && active) atomicAdd(bp.stats + kStatActiveBins, (unsigned long long)active);
    if (threadIdx.x == 0) {
        bp.bin_start[n] = total;
        atomicAdd(bp.stats + kStatBinEntries, (unsigned long long)total);
    }
    pdl_trigger();
}

// ------------------------------------------------------------------ bin scatter

constexpr int kScatterBlock = 256;

// Puts key[k] into bin[k] for the k (of 4) whose bit is set in m: the list positions (atomics on
// the bin counters) and the bins' starts are all requested before any is used, so one thread's
// fills take one round trip instead of one each.
template <bool COHERENT = false>
__device__ __forceinline__ void put4(const BatchParams &bp, const uint32_t *bin, const uint32_t *key, uint32_t m) {
    uint32_t pos[4], st[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (m >> k & 1u) {
            pos[k] = atomicSub(bp.bin_count + bin[k], 1u) - 1u;
            st[k] = ld_stage<COHERENT>(bp.bin_start + bin[k]);
        }
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (m >> k & 1u) bp.list[st[k] + pos[k]] = key[k];
}

// The bins t, t + step, ... (below nt) of one job, four at a time.
template <bool COHERENT = false>
__device__ __forceinline__ void put_job(const BatchParams &bp, const BinJob &j, uint32_t t, uint32_t step) {
    const uint32_t nt = j.nx * j.ny;
    const uint32_t key[4] = {j.key, j.key, j.key, j.key};
    for (; t < nt; t += 4 * step) {
        uint32_t bin[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) bin[k] = job_bin(j, min(t + (uint32_t)k * step, nt - 1));
        put4<COHERENT>(bp, bin, key, (1u << min(4u, (nt - t + step - 1) / step)) - 1u);
    }
}

// Fills the bin lists (main.c:950-962) from the bin jobs k_geometry and k_clip listed (one per
// triangle or fan with bins: its key, first bin, tile counts and view), one thread per job: the key
// goes to the list of every bin of its range (the order inside a bin does not matter, see k_tile).
// One-tile jobs of a warp that share a bin take their list positions with one atomic; jobs over
// more than big_tiles bins are filled by the whole warp.
struct ScatterSmem {
    BinJob big[kScatterBlock / 32][32];       // the warp's jobs over many bins
    uint32_t bigpref[kScatterBlock / 32][32]; // inclusive prefix of their bin counts
};

// CTA blk of nblk (kScatterBlock threads); k_scatter and the persistent launch run it (which
// reads the error word at its grid barrier instead, where no CTA can be setting it).
template <bool CHECK_ERROR = true, bool COHERENT = false>
__device__ __forceinline__ void scatter_body(const BatchParams &bp, uint32_t blk, uint32_t nblk, ScatterSmem &sm) {
    auto &s_big = sm.big;
    auto &s_bigpref = sm.bigpref;
    if (CHECK_ERROR && ld_volatile_u32(bp.error)) return;
    const uint32_t total = bp.bin_start[bp.total_bins];
    if (total > bp.list_capacity) {
        if (blk == 0 && threadIdx.x == 0) {
            atomicOr(bp.error, kErrListOverflow);
            atomicMin(bp.error + 1, bp.batch_seq);
            atomicMax(bp.error + 3, total);
        }
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t njobs = ld_volatile_u32(bp.counters + kCtrJobs);
    const uint32_t stride = nblk * kScatterBlock;
    const uint32_t j_first = blk * kScatterBlock + threadIdx.x;
    uint4 e_next = j_first < njobs ? bp.jobs[j_first] : make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t base = blk * kScatterBlock; base < njobs; base += stride) {
        const uint32_t j = base + threadIdx.x;
        const uint4 e = e_next;
        // the next iteration's job is in flight while this one's bins are filled
        e_next = j + stride < njobs ? bp.jobs[j + stride] : make_uint4(0u, 0u, 0u, 0u);
        BinJob own;
        own.key = e.x;
        own.first_bin = e.y;
        own.nx = e.z & 0xFFFFu;
        own.ny = e.z >> 16;
        const uint32_t nt_own = j < njobs ? own.nx * own.ny : 0u;
        if (nt_own > 1) {   // the bin strides of its view (a one-tile job needs none)
            const ViewDesc &vw = bp.views[e.w];
            own.col_stride = vw.draw_count;
            own.row_stride = vw.tiles_x * vw.draw_count;
        }
        const uint32_t single = nt_own == 1 ? own.first_bin : 0xFFFFFFFFu;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, single);
        if (single != 0xFFFFFFFFu) {
            const int leader = __ffs(peers) - 1;
            const uint32_t st = ld_stage<COHERENT>(bp.bin_start + single);
            uint32_t top = 0;
            if (lane == leader) top = atomicSub(bp.bin_count + single, (uint32_t)__popc(peers));
            top = __shfl_sync(peers, top, leader);
            const uint32_t r = (uint32_t)__popc(peers & ((1u << lane) - 1u));
            bp.list[st + top - 1u - r] = own.key;
        } else if (nt_own > 1 && nt_own <= bp.big_tiles) {
            put_job<COHERENT>(bp, own, 0, 1);
        }
        // triangles over more than big_tiles bins are filled by the whole warp, 32 (triangle, bin)
        // pairs per round. Each big triangle normally starts a new round (its pair count is padded
        // to a multiple of 32 and the padding skipped); when that leaves many rounds part-empty
        // (triangles of a few dozen bins), the pairs of all of them are packed into as few rounds
        // as they need instead.
        const uint32_t nbig = nt_own > bp.big_tiles ? nt_own : 0u;
        const uint32_t bigmask = __ballot_sync(0xFFFFFFFFu, nbig != 0u);
        if (bigmask) {
            const uint32_t rounds_each = __reduce_add_sync(0xFFFFFFFFu, (nbig + 31u) >> 5);
            const uint32_t rounds_packed = (__reduce_add_sync(0xFFFFFFFFu, nbig) + 31u) >> 5;
            uint32_t incl = rounds_packed < rounds_each ? nbig : (nbig + 31u) & ~31u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t total_big = __shfl_sync(0xFFFFFFFFu, incl, 31);
            if (nbig) {   // compacted: the k-th big triangle and the end of its pairs
                const uint32_t k = __popc(bigmask & ((1u << lane) - 1u));
                s_big[warp][k] = own;
                s_bigpref[warp][k] = incl;
            }
            __syncwarp();
            // each lane's pairs are item = lane, lane + 32, ...: its triangle only moves forward,
            // so the job stays in registers until the lane crosses the end of a triangle; four
            // pairs are filled together
            uint32_t jb = 0, first = 0, end = s_bigpref[warp][0];
            BinJob job = s_big[warp][0];
            for (uint32_t item0 = lane; item0 < total_big; item0 += 128) {
                uint32_t bin[4], key[4], m = 0;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const uint32_t item = item0 + 32u * (uint32_t)k;
                    bin[k] = 0;
                    key[k] = 0;
                    if (item >= total_big) continue;
                    if (item >= end) {
                        do {
                            ++jb;
                            first = end;
                            end = s_bigpref[warp][jb];
                        } while (item >= end);
                        job = s_big[warp][jb];
                    }
                    if (item - first < job.nx * job.ny) {   // not padding
                        bin[k] = job_bin(job, item - first);
                        key[k] = job.key;
                        m |= 1u << k;
                    }
                }
                put4<COHERENT>(bp, bin, key, m);
            }
        }
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kScatterBlock) k_scatter(BatchParams bp) {
    __shared__ ScatterSmem sm;
    pdl_wait();
    scatter_body(bp, blockIdx.x, gridDim.x, sm);
    pdl_trigger();
}

// ------------------------------------------------------------------ tile kernel

// Monotone map of a float depth to u32 (after folding -0 onto +0, which compares equal).
__device__ __forceinline__ uint32_t depth_key(float z) {
    uint32_t u = __float_as_uint(z);
    if (u == 0x80000000u) u = 0;
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float depth_from_key(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

__device__ __forceinline__ uint32_t find_view(const BatchParams &bp, uint32_t tile) {
    uint32_t lo = 0, hi = bp.num_views;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&bp.views[mid].tile_base) <= tile) lo = mid; else hi = mid;
    }
    return lo;
}

// Position of the k-th (0-based) set bit of m, k < popc(m).
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t k) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t step = 16; step; step >>= 1) {
        const uint32_t c = __popc(m & ((1u << step) - 1u));
        if (k >= c) {
            k -= c;
            m >>= step;
            pos += step;
        }
    }
    return pos;
}

// Per-triangle parameters staged in shared memory for the work-expansion loop (17 words per
// triangle, an odd stride, so lanes reading different triangles hit different banks).
// Per-triangle parameters staged in shared memory for the work-expansion loop: 20 words (five
// 16-byte groups, read with vector loads) per triangle:
//   q0 = E0, A0, B0, E1     edge values at the box's first pixel (E), x steps A = a << 4,
//   q1 = A1, B1, E2, A2     y steps B = b << 4
//   q2 = B2, width, pad, origin
//   q3 = 1/area, z0, z1 - z0, z2 - z0
//   q4 = key, -, -, -
// width: box width | reciprocal << 8 (row = local * recip >> 16); pad: the top-left rule's bias
// bits (edge k needs E >= 1) | box height << 8; origin: box origin in the tile, x | y << 8.
// Eight lanes storing their triangles (80-byte stride) hit distinct banks.
constexpr int kStage = 20;

// Writes the folded clears (ViewDesc::clear_flags) of a pixel that no draw of the batch wrote;
// depth is the running value, which for such a pixel is the clear value.
__device__ __forceinline__ void write_cleared(const ViewDesc &V, size_t o, float depth) {
    const uint32_t f = V.clear_flags;
    if (f & kClearColor) V.color[o] = V.clear_color;
    if (f & kClearDepth) V.depth[o] = depth;
    if (f & kClearTri) V.vis_tri[o] = V.clear_tri;
    if (f & kClearDraw) V.vis_draw[o] = V.clear_draw;
    if (f & kClearPrim) V.vis_prim[o] = V.clear_prim;
    if (f & kClearBary)
        reinterpret_cast<uint2 *>(V.vis_bary)[o] = make_uint2(V.clear_bary, V.clear_bary);
}

// Triangles with more (triangle, pixel) work items in the tile than this are tested at every pixel
// of the tile by the whole warp, two pixels a lane, instead of through the work-item list: the
// list costs a few instructions per item per lane (finding the item's triangle and decoding it),
// the whole-tile test a fixed amount per triangle.
constexpr uint32_t kWholeTileItems = 24;

// Keeps the better of two (depth, key) pairs: the larger for GREATER_EQUAL, the smaller for LESS.
__device__ __forceinline__ unsigned long long better_key(bool less, unsigned long long a, unsigned long long b) {
    return less ? (a < b ? a : b) : (a > b ? a : b);
}

// One chunk of up to 32 entries [chunk, min(chunk + 32, e)) of a tile's bin for one draw. Each lane
// stages one triangle (hierarchical-Z test, main.c:1005-1010; its box clipped to the tile), then
// the warp walks the (triangle, pixel) work items of the small ones, 32 at a time, and tests the
// large ones at every pixel of the tile, and folds every covered fragment (main.c:1015-1028) whose
// depth (main.c:1092-1102, 1131-1132) passes the test against the depth at draw start
// (main.c:1164-1168) into the pixel's best (depth, key): for work items an atomic max (min for
// LESS) on best[pixel], for whole-tile tests the lane's own fa (pixel lane) and fb (pixel lane + 32),
// which the caller folds into best after the draw. best and depth are the tile's 64 pixels,
// row-major; stage, pref and mask are the warp's own.
template <bool COHERENT = false>
__device__ __forceinline__ void tile_chunk(const BatchParams &bp, uint32_t chunk, uint32_t e, int32_t x0, int32_t y0,
                                           bool less, bool top_left, float hiz, uint32_t *stage, uint32_t *pref,
                                           unsigned long long *mask, unsigned long long *best, const float *depth,
                                           bool capture, int lane, unsigned long long &fa, unsigned long long &fb) {
    const uint32_t i = chunk + lane;
    uint32_t cnt = 0;   // work items of this lane's triangle in the tile
    if (i < e) {
        const uint32_t key = bp.list[i];
        const uint32_t rec = record_of<COHERENT>(bp, key);
        const int4 *R = bp.raster[rec].w;
        const int4 w2 = R[2], w3 = R[3];
        const float zb = __int_as_float(w2.z);
        const bool rejected = less ? (zb > hiz) : (zb < hiz);   // main.c:1005-1010 (mirrored for LESS)
        int32_t bx0 = (int16_t)(w3.z & 0xFFFF), by0 = w3.z >> 16;
        int32_t bx1 = (int16_t)(w3.w & 0xFFFF), by1 = w3.w >> 16;
        bx0 = max(bx0, x0); by0 = max(by0, y0);
        bx1 = min(bx1, x0 + kTile - 1); by1 = min(by1, y0 + kTile - 1);
        if (!rejected && bx1 >= bx0 && by1 >= by0) {
            const int4 w0 = R[0], w1 = R[1];
            const uint32_t a0 = w0.x, b0 = w0.y, c0 = w0.z, a1 = w0.w, b1 = w1.x, c1 = w1.y, a2 = w1.z, b2 = w1.w,
                           c2 = w2.x;
            const uint32_t w = (uint32_t)(bx1 - bx0 + 1), h = (uint32_t)(by1 - by0 + 1);
            cnt = w * h;
            uint4 *sq = reinterpret_cast<uint4 *>(stage + lane * kStage);
            // main.c:1015-1025: ((a*x)<<4) + ((b*y)<<4) + c, wrapping int32
            const uint32_t e0 = ((a0 * (uint32_t)bx0) << kSubpix) + ((b0 * (uint32_t)by0) << kSubpix) + c0;
            const uint32_t e1 = ((a1 * (uint32_t)bx0) << kSubpix) + ((b1 * (uint32_t)by0) << kSubpix) + c1;
            const uint32_t e2 = ((a2 * (uint32_t)bx0) << kSubpix) + ((b2 * (uint32_t)by0) << kSubpix) + c2;
            // top-left rule: an edge value of 0 covers only on a left edge (a > 0) or a top edge
            // (a == 0, b > 0); the others need E >= 1 (bit k set: edge k needs it)
            const uint32_t pad = ((int32_t)a0 > 0 || (a0 == 0 && (int32_t)b0 > 0) ? 0u : 1u) |
                                 ((int32_t)a1 > 0 || (a1 == 0 && (int32_t)b1 > 0) ? 0u : 2u) |
                                 ((int32_t)a2 > 0 || (a2 == 0 && (int32_t)b2 > 0) ? 0u : 4u) | (h << 8);
            const float z0 = __int_as_float(w2.w);
            sq[0] = make_uint4(e0, a0 << kSubpix, b0 << kSubpix, e1);
            sq[1] = make_uint4(a1 << kSubpix, b1 << kSubpix, e2, a2 << kSubpix);
            sq[2] = make_uint4(b2 << kSubpix, w | (((65536u + w - 1) / w) << 8), pad,
                               (uint32_t)(bx0 - x0) | ((uint32_t)(by0 - y0) << 8));
            sq[3] = make_uint4((uint32_t)w2.y, (uint32_t)w2.w, __float_as_uint(__int_as_float(w3.x) - z0),
                               __float_as_uint(__int_as_float(w3.y) - z0));
            sq[4] = make_uint4(key, 0u, 0u, 0u);
        }
    }
    if (capture) mask[lane] = 0;
    const bool whole = cnt > kWholeTileItems;
    // exclusive offsets of the (triangle, pixel) work items of the small triangles
    uint32_t incl = whole ? 0u : cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    pref[lane] = incl;
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    __syncwarp();
    for (uint32_t item = lane; item < total; item += 32) {
        uint32_t j = 0;   // triangle of this item: number of prefixes <= item
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1)
            if (pref[j + step - 1] <= item) j += step;
        const uint4 *sq = reinterpret_cast<const uint4 *>(stage + j * kStage);
        const uint32_t local = item - (j ? pref[j - 1] : 0u);
        const uint4 q0 = sq[0], q1 = sq[1], q2 = sq[2];
        const uint32_t wr = q2.y;
        const uint32_t row = (local * (wr >> 8)) >> 16;
        const uint32_t col = local - row * (wr & 0xFFu);
        const uint32_t E0 = q0.x + col * q0.y + row * q0.z;
        const uint32_t E1 = q0.w + col * q1.x + row * q1.y;
        const uint32_t E2 = q1.z + col * q1.w + row * q2.x;
        const uint32_t nb = q2.z;
        const bool covered = top_left ? (int32_t)((E0 - (nb & 1u)) | (E1 - ((nb >> 1) & 1u)) | (E2 - ((nb >> 2) & 1u))) >= 0
                                      : (int32_t)(E0 | E1 | E2) > 0;   // main.c:1028
        if (covered) {
            const uint32_t org = q2.w;
            const int p = (int)(((org >> 8) + row) * 8 + (org & 0xFFu) + col);
            if (capture) atomicOr(&mask[j], 1ull << p);
            // main.c:1092-1102 and 1131-1132 for reg0.z
            const uint4 q3 = sq[3];
            const float inv_area = __uint_as_float(q3.x);
            const float bb1 = (float)((int32_t)E1 >> (kSubpix * 2)) * inv_area;
            const float bb2 = (float)((int32_t)E2 >> (kSubpix * 2)) * inv_area;
            float z = __uint_as_float(q3.y) + __uint_as_float(q3.z) * bb1;
            z = z + __uint_as_float(q3.w) * bb2;
            const float dstart = depth[p];
            const bool cand = less ? (z < dstart) : (z >= dstart);   // main.c:1164-1168
            if (cand) {
                const unsigned long long k = ((unsigned long long)depth_key(z) << 32) | sq[4].x;
                if (less) atomicMin(&best[p], k);
                else atomicMax(&best[p], k);
            }
        }
    }
    // the large triangles: every lane tests its two pixels, (lane & 7, lane >> 3) and 4 rows below
    uint32_t big = __ballot_sync(0xFFFFFFFFu, whole);
    if (big) {
        const float da = depth[lane], db = depth[lane + 32];
        const int32_t cx = lane & 7, cy = lane >> 3;
        do {
            const int j = __ffs(big) - 1;
            big &= big - 1;
            const uint4 *sq = reinterpret_cast<const uint4 *>(stage + j * kStage);
            const uint4 q0 = sq[0], q1 = sq[1], q2 = sq[2];
            const uint32_t org = q2.w, nb = q2.z;
            // offsets from the box origin; outside the box nothing is tested (main.c:1015-1025)
            const uint32_t dx = (uint32_t)(cx - (int32_t)(org & 0xFFu)), dy = (uint32_t)(cy - (int32_t)(org >> 8));
            const uint32_t w = q2.y & 0xFFu, h = nb >> 8;
            const bool in_x = dx < w;
            const bool in_a = in_x && dy < h, in_b = in_x && dy + 4u < h;
            const uint32_t sb0 = q0.z, sb1 = q1.y, sb2 = q2.x;
            const uint32_t E0a = q0.x + dx * q0.y + dy * sb0, E0b = E0a + (sb0 << 2);
            const uint32_t E1a = q0.w + dx * q1.x + dy * sb1, E1b = E1a + (sb1 << 2);
            const uint32_t E2a = q1.z + dx * q1.w + dy * sb2, E2b = E2a + (sb2 << 2);
            bool ca, cb;
            if (top_left) {
                ca = (int32_t)((E0a - (nb & 1u)) | (E1a - ((nb >> 1) & 1u)) | (E2a - ((nb >> 2) & 1u))) >= 0;
                cb = (int32_t)((E0b - (nb & 1u)) | (E1b - ((nb >> 1) & 1u)) | (E2b - ((nb >> 2) & 1u))) >= 0;
            } else {
                ca = (int32_t)(E0a | E1a | E2a) > 0;   // main.c:1028
                cb = (int32_t)(E0b | E1b | E2b) > 0;
            }
            ca = ca && in_a;
            cb = cb && in_b;
            if (capture) {
                const uint32_t ma = __ballot_sync(0xFFFFFFFFu, ca), mb = __ballot_sync(0xFFFFFFFFu, cb);
                if (lane == 0) mask[j] = (unsigned long long)ma | ((unsigned long long)mb << 32);
            }
            const uint4 q3 = sq[3];
            const float inv_area = __uint_as_float(q3.x);
            const float z0 = __uint_as_float(q3.y), dz1 = __uint_as_float(q3.z), dz2 = __uint_as_float(q3.w);
            const unsigned long long key = sq[4].x;
            if (ca) {
                const float bb1 = (float)((int32_t)E1a >> (kSubpix * 2)) * inv_area;
                const float bb2 = (float)((int32_t)E2a >> (kSubpix * 2)) * inv_area;
                float z = z0 + dz1 * bb1;
                z = z + dz2 * bb2;
                if (less ? (z < da) : (z >= da)) fa = better_key(less, fa, ((unsigned long long)depth_key(z) << 32) | key);
            }
            if (cb) {
                const float bb1 = (float)((int32_t)E1b >> (kSubpix * 2)) * inv_area;
                const float bb2 = (float)((int32_t)E2b >> (kSubpix * 2)) * inv_area;
                float z = z0 + dz1 * bb1;
                z = z + dz2 * bb2;
                if (less ? (z < db) : (z >= db)) fb = better_key(less, fb, ((unsigned long long)depth_key(z) << 32) | key);
            }
        } while (big);
    }
    __syncwarp();
    if (capture && i < e) bp.info_mask[i] = cnt ? mask[lane] : 0ull;
    __syncwarp();
}

// The pixel shader and output merger for the fragment that won pixel (x, y): interpolation with
// the reference's quantised barycentrics and perspective correction (main.c:1089-1160), the
// shader (main.c:1172), packing (main.c:1176-1178), the colour and depth write (main.c:1180-1181)
// and the visibility outputs.
template <bool COHERENT = false>
__device__ __forceinline__ void shade_pixel(const BatchParams &bp, const ViewDesc &V, uint32_t key, int32_t x,
                                            int32_t y) {
    const size_t o = (size_t)y * V.width + x;
    const uint32_t rec = record_of<COHERENT>(bp, key);
    const int4 *R = bp.raster[rec].w;
    const int4 w0 = R[0], w1 = R[1], w2 = R[2], w3 = R[3];
    // the winner's draw: the view's only one, or the index its shading record keeps
    const bool sole = V.draw_count == 1;
    const float4 *S = reinterpret_cast<const float4 *>(bp.shade) + (size_t)rec * bp.shade_stride;
    float4 s0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!sole) s0 = S[0];
    const DrawDesc &D = bp.draws[sole ? V.draw_begin : __float_as_uint(s0.w)];
    const uint32_t E1 = (((uint32_t)w0.w * (uint32_t)x) << kSubpix) + (((uint32_t)w1.x * (uint32_t)y) << kSubpix) + (uint32_t)w1.y;
    const uint32_t E2 = (((uint32_t)w1.z * (uint32_t)x) << kSubpix) + (((uint32_t)w1.w * (uint32_t)y) << kSubpix) + (uint32_t)w2.x;
    const float inv_area = __int_as_float(w2.y);
    const float b1 = (float)((int32_t)E1 >> (kSubpix * 2)) * inv_area;
    const float b2 = (float)((int32_t)E2 >> (kSubpix * 2)) * inv_area;
    const float z0 = __int_as_float(w2.w), z1 = __int_as_float(w3.x), z2 = __int_as_float(w3.y);
    float z = z0 + (z1 - z0) * b1;
    z = z + (z2 - z0) * b2;
    if (D.ps != kPsNone) {
        if (sole) s0 = S[0];
        // perspective correction, main.c:1106-1115
        float den = (1.0f - (b1 + b2)) * s0.x;
        den = den + b1 * s0.y;
        den = den + b2 * s0.z;
        den = 1.0f / den;
        const float pb1 = (b1 * s0.y) * den;
        const float pb2 = (b2 * s0.z) * den;
        auto interp = [&](float v0, float v1, float v2) {
            float tmp = v0 + (v1 - v0) * pb1;
            return tmp + (v2 - v0) * pb2;
        };
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, u, v;
        if (bp.shade_stride == kShadeUV) {   // U and V only (basic_ps reads nothing else)
            const float4 q1 = S[1], q2 = S[2];
            u = interp(q1.x, q1.y, q1.z);
            v = interp(q1.w, q2.x, q2.y);
        } else {
            const float4 r0 = S[1], r1 = S[2], r2 = S[3], uv2 = S[4];
            a0 = interp(r0.x, r1.x, r2.x);
            a1 = interp(r0.y, r1.y, r2.y);
            a2 = interp(r0.z, r1.z, r2.z);
            u = interp(r0.w, r1.w, r2.w);
            v = interp(uv2.x, uv2.y, uv2.z);
        }
        const float3 c = run_ps(D.ps, a0, a1, a2, u, v, D.ps_tex);
        V.color[o] = pack_color(c.x, c.y, c.z);
    } else if (V.clear_flags & kClearColor) {
        V.color[o] = V.clear_color;   // a null pixel shader leaves the (folded) clear colour
    }
    V.depth[o] = z;
    if (V.vis_tri && bp.rank) {
        // the reference's triangle id: its index among the draw's assembled triangles
        const uint32_t g = key >> 3, cf = key & 7u;
        const uint32_t fmask = bp.tri_info[g] & 0xFFu;
        const uint32_t below = cf ? (uint32_t)__popc(fmask & ((1u << (cf - 1)) - 1u)) : 0u;
        V.vis_tri[o] = bp.rank[g] - bp.rank[D.tri_begin] + below;
    }
    if (V.vis_draw) V.vis_draw[o] = D.draw_seq;
    if (V.vis_prim) V.vis_prim[o] = (key >> 3) - D.tri_begin;
    if (V.vis_bary) reinterpret_cast<float2 *>(V.vis_bary)[o] = make_float2(b1, b2);
}

// Zeroes the per-batch counters (kCtrOverflow ... kCtrClaimTiles) for the next batch. The batch's
// last kernel does it once its predecessors are done with them, so that a batch needs no memset of
// its own in front of its first kernel (in a graph, a memset node there keeps the first kernel
// from being launched early). The counters are zero on allocation and after a failed batch's
// recovery, which zeroes every counter.
__device__ __forceinline__ void reset_batch_counters(const BatchParams &bp) {
#pragma unroll
    for (int k = 0; k < kCtrPerBatch; ++k) bp.counters[kCtrOverflow + k] = 0u;
}

// Commits the batch's staged statistics (k_geometry and k_scan finished before the tile kernel).
__device__ __forceinline__ void commit_stats(const BatchParams &bp, uint32_t blk) {
    if (blk == 0 && threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            bp.stats[kStatTotal + k] += bp.stats[k];
            bp.stats[k] = 0;
        }
    }
}

template <int WARPS>
struct TileSmem {
    __align__(16) uint32_t stage[WARPS][32 * kStage];
    unsigned long long best[WARPS][64];
    float depth[WARPS][64];
    uint32_t pref[WARPS][32];
    unsigned long long mask[WARPS][32];
};

// Tile gtile of the batch by one warp, with the warp's slices of sm; k_tile (WARPS tiles per CTA)
// and the persistent launch run it.
template <int WARPS, bool COHERENT = false>
__device__ __forceinline__ void tile_warp(const BatchParams &bp, uint32_t gtile, TileSmem<WARPS> &sm) {
    auto &s_best = sm.best;
    auto &s_depth = sm.depth;
    auto &s_stage = sm.stage;
    auto &s_pref = sm.pref;
    auto &s_mask = sm.mask;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (gtile >= bp.total_tiles) return;
    const uint32_t vi = find_view(bp, gtile);
    const ViewDesc &V = bp.views[vi];
    const uint32_t t = gtile - V.tile_base;
    const uint32_t tx = t % V.tiles_x, ty = t / V.tiles_x;
    const uint32_t bin0 = V.bin_base + t * V.draw_count;
    const uint32_t dc = V.draw_count;
    // the bin boundaries of this tile's draws, one per lane (lane d holds bin_start[bin0 + d])
    const uint32_t my_start = lane <= dc ? ld_stage<COHERENT>(bp.bin_start + bin0 + lane) : 0u;
    const uint32_t last = dc < 32 ? __shfl_sync(0xFFFFFFFFu, my_start, dc) : ld_stage<COHERENT>(bp.bin_start + bin0 + dc);

    const int32_t x0 = (int32_t)tx * kTile, y0 = (int32_t)ty * kTile;
    // lane owns pixels p0 = lane (rows 0-3) and p1 = lane + 32 (rows 4-7)
    const int32_t px = x0 + (lane & 7), py0 = y0 + (lane >> 3), py1 = py0 + 4;
    const bool valid0 = px < (int32_t)V.width && py0 < (int32_t)V.height;
    const bool valid1 = px < (int32_t)V.width && py1 < (int32_t)V.height;
    const size_t o0 = (size_t)py0 * V.width + px, o1 = (size_t)py1 * V.width + px;
    const bool depth_cleared = (V.clear_flags & kClearDepth) != 0;
    if (__shfl_sync(0xFFFFFFFFu, my_start, 0) == last) {   // no draw binned a triangle here
        if (V.clear_flags) {
            if (valid0) write_cleared(V, o0, V.clear_depth);
            if (valid1) write_cleared(V, o1, V.clear_depth);
            if (lane == 0 && depth_cleared) {   // clear_depth_stencil_view's tile bounds (main.c:1212-1214)
                V.tile_min[t] = 0.0f;
                V.tile_max[t] = 1.0f;
            }
        }
        return;
    }
    float dcur0 = valid0 ? (depth_cleared ? V.clear_depth : V.depth[o0]) : 0.0f;
    float dcur1 = valid1 ? (depth_cleared ? V.clear_depth : V.depth[o1]) : 0.0f;
    uint32_t win0 = 0xFFFFFFFFu, win1 = 0xFFFFFFFFu;
    s_depth[warp][lane] = dcur0;
    s_depth[warp][lane + 32] = dcur1;
    float hiz_min = depth_cleared ? 0.0f : V.tile_min[t], hiz_max = depth_cleared ? 1.0f : V.tile_max[t];
    const bool capture = bp.info_mask != nullptr;

    for (uint32_t dd = 0; dd < dc; ++dd) {
        if (dc < 32) {   // skip to the next draw with entries here (lane d: draw d has some)
            const uint32_t next = __shfl_down_sync(0xFFFFFFFFu, my_start, 1);   // every lane takes part
            const uint32_t rest = __ballot_sync(0xFFFFFFFFu, (uint32_t)lane >= dd && (uint32_t)lane < dc &&
                                                                 my_start != next);
            if (!rest) break;
            dd = (uint32_t)__ffs(rest) - 1u;
        }
        uint32_t s, e;
        if (dd + 1 < 32) {
            s = __shfl_sync(0xFFFFFFFFu, my_start, dd);
            e = __shfl_sync(0xFFFFFFFFu, my_start, dd + 1);
        } else {
            s = ld_stage<COHERENT>(bp.bin_start + bin0 + dd);
            e = ld_stage<COHERENT>(bp.bin_start + bin0 + dd + 1);
        }
        if (s == e) continue;
        const DrawDesc &D = bp.draws[V.draw_begin + dd];
        const bool less = D.depth_less != 0;
        const bool top_left = (D.raster_flags & kRasterTopLeft) != 0;
        const unsigned long long sentinel = less ? ~0ull : 0ull;
        s_best[warp][lane] = sentinel;
        s_best[warp][lane + 32] = sentinel;
        const float hiz = less ? hiz_max : hiz_min;
        unsigned long long fa = sentinel, fb = sentinel;
        for (uint32_t chunk = s; chunk < e; chunk += 32)
            tile_chunk<COHERENT>(bp, chunk, e, x0, y0, less, top_left, hiz, s_stage[warp], s_pref[warp], s_mask[warp],
                       s_best[warp], s_depth[warp], capture, lane, fa, fb);
        // fold this draw's winners into the running state; hierarchical Z update (write_tile, main.c:589-603)
        const unsigned long long k0 = better_key(less, s_best[warp][lane], fa);
        const unsigned long long k1 = better_key(less, s_best[warp][lane + 32], fb);
        if (k0 != sentinel) { dcur0 = depth_from_key((uint32_t)(k0 >> 32)); win0 = (uint32_t)k0; }
        if (k1 != sentinel) { dcur1 = depth_from_key((uint32_t)(k1 >> 32)); win1 = (uint32_t)k1; }
        s_depth[warp][lane] = dcur0;
        s_depth[warp][lane + 32] = dcur1;
        float mn = 1.0f, mx = 0.0f;
        if (valid0) { mn = fmin_ref(mn, dcur0); mx = fmax_ref(mx, dcur0); }
        if (valid1) { mn = fmin_ref(mn, dcur1); mx = fmax_ref(mx, dcur1); }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            float a = __shfl_xor_sync(0xFFFFFFFFu, mn, o), b = __shfl_xor_sync(0xFFFFFFFFu, mx, o);
            mn = fmin_ref(mn, a);
            mx = fmax_ref(mx, b);
        }
        hiz_min = mn;
        hiz_max = mx;
        __syncwarp();
    }

    // shade the final winners, one pixel-shader invocation per written pixel, compacted over the
    // warp so that a partly covered tile needs one pass
    const uint32_t m0 = __ballot_sync(0xFFFFFFFFu, win0 != 0xFFFFFFFFu && valid0);
    const uint32_t m1 = __ballot_sync(0xFFFFFFFFu, win1 != 0xFFFFFFFFu && valid1);
    const uint32_t n0 = __popc(m0), n = n0 + __popc(m1);
    for (uint32_t q0 = 0; q0 < n; q0 += 32) {
        const uint32_t q = q0 + lane;
        const uint32_t half = q < n0 ? 0u : 1u;
        uint32_t src = 0;
        if (q < n) {
            const uint32_t m = half ? m1 : m0, k = half ? q - n0 : q;
            src = m == 0xFFFFFFFFu ? k : nth_set_bit(m, k);   // a full half needs no search
        }
        const uint32_t wa = __shfl_sync(0xFFFFFFFFu, win0, src), wb = __shfl_sync(0xFFFFFFFFu, win1, src);
        if (q >= n) continue;
        shade_pixel<COHERENT>(bp, V, half ? wb : wa, x0 + (int32_t)(src & 7), y0 + (int32_t)(src >> 3) + (half ? 4 : 0));
    }
    // pixels no draw wrote still owe their folded clears
    if (V.clear_flags) {
        if (valid0 && win0 == 0xFFFFFFFFu) write_cleared(V, o0, dcur0);
        if (valid1 && win1 == 0xFFFFFFFFu) write_cleared(V, o1, dcur1);
    }
    if (lane == 0) {
        V.tile_min[t] = hiz_min;
        V.tile_max[t] = hiz_max;
    }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_tile(BatchParams bp) {
    __shared__ TileSmem<WARPS> sm;
    pdl_wait();
    if (ld_volatile_u32(bp.error)) return;
    commit_stats(bp, blockIdx.x);
    if (blockIdx.x == 0 && threadIdx.x == 0) reset_batch_counters(bp);
    tile_warp<WARPS>(bp, blockIdx.x * WARPS + (threadIdx.x >> 5), sm);
    pdl_trigger();
}

// One tile per CTA, its triangles shared by WARPS warps: each warp takes an equal share of a bin's
// entries (most bins hold fewer than 32, so chunk-wise sharing would leave the other warps idle),
// all fold into the CTA's best keys. For frames whose triangles crowd into few tiles (a single
// large mesh): k_tile leaves most of the GPU idle behind those tiles' warps. Same results
// as k_tile: the per-pixel max (min) of (depth, key) does not depend on which warp finds it, and
// thread t < 64 owns pixel t for the fold, the hierarchical-Z bounds and the pixel shader.
template <int WARPS>
struct CoopSmem {
    __align__(16) uint32_t stage[WARPS][32 * kStage];
    unsigned long long best[64];
    float depth[64];
    float hiz[2];
    uint32_t pref[WARPS][32];
    unsigned long long mask[WARPS][32];
};

// Tile blk, shared by the CTA's WARPS warps; k_tile_coop and the persistent launch run it. Every
// return and barrier is uniform over the CTA (the error word is read only where no kernel of the
// batch can still set it: k_tile_coop's start; the persistent launch checks it at its barrier).
template <int WARPS, bool CHECK_ERROR = true, bool COHERENT = false>
__device__ __forceinline__ void tile_coop_body(const BatchParams &bp, uint32_t blk, CoopSmem<WARPS> &sm) {
    static_assert(WARPS >= 2, "threads 0-63 own the tile's pixels");
    auto &s_best = sm.best;
    auto &s_depth = sm.depth;
    auto &s_hiz = sm.hiz;
    auto &s_stage = sm.stage;
    auto &s_pref = sm.pref;
    auto &s_mask = sm.mask;
    if (CHECK_ERROR && ld_volatile_u32(bp.error)) return;   // uniform: set only by earlier kernels
    commit_stats(bp, blk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t gtile = blk;
    if (gtile >= bp.total_tiles) return;
    const uint32_t vi = find_view(bp, gtile);
    const ViewDesc &V = bp.views[vi];
    const uint32_t t = gtile - V.tile_base;
    const uint32_t tx = t % V.tiles_x, ty = t / V.tiles_x;
    const uint32_t bin0 = V.bin_base + t * V.draw_count;
    const uint32_t dc = V.draw_count;
    const uint32_t my_start = lane <= dc ? ld_stage<COHERENT>(bp.bin_start + bin0 + lane) : 0u;
    const uint32_t last = dc < 32 ? __shfl_sync(0xFFFFFFFFu, my_start, dc) : ld_stage<COHERENT>(bp.bin_start + bin0 + dc);

    const int32_t x0 = (int32_t)tx * kTile, y0 = (int32_t)ty * kTile;
    const int pix = (int)threadIdx.x;           // pixel of threads 0-63: row-major in the tile
    const bool owner = pix < 64;
    const int32_t px = x0 + (pix & 7), py = y0 + (pix >> 3);
    const bool valid = owner && px < (int32_t)V.width && py < (int32_t)V.height;
    const size_t o = (size_t)py * V.width + px;
    const bool depth_cleared = (V.clear_flags & kClearDepth) != 0;
    if (__shfl_sync(0xFFFFFFFFu, my_start, 0) == last) {   // uniform: no draw binned a triangle here
        if (V.clear_flags) {
            if (valid) write_cleared(V, o, V.clear_depth);
            if (threadIdx.x == 0 && depth_cleared) {   // main.c:1212-1214
                V.tile_min[t] = 0.0f;
                V.tile_max[t] = 1.0f;
            }
        }
        return;
    }
    float dcur = valid ? (depth_cleared ? V.clear_depth : V.depth[o]) : 0.0f;
    uint32_t win = 0xFFFFFFFFu;
    if (owner) s_depth[pix] = dcur;
    float hiz_min = depth_cleared ? 0.0f : V.tile_min[t], hiz_max = depth_cleared ? 1.0f : V.tile_max[t];
    const bool capture = bp.info_mask != nullptr;

    for (uint32_t dd = 0; dd < dc; ++dd) {
        if (dc < 32) {   // skip to the next draw with entries here (lane d: draw d has some)
            const uint32_t next = __shfl_down_sync(0xFFFFFFFFu, my_start, 1);   // every lane takes part
            const uint32_t rest = __ballot_sync(0xFFFFFFFFu, (uint32_t)lane >= dd && (uint32_t)lane < dc &&
                                                                 my_start != next);
            if (!rest) break;
            dd = (uint32_t)__ffs(rest) - 1u;
        }
        uint32_t s, e;
        if (dd + 1 < 32) {
            s = __shfl_sync(0xFFFFFFFFu, my_start, dd);
            e = __shfl_sync(0xFFFFFFFFu, my_start, dd + 1);
        } else {
            s = ld_stage<COHERENT>(bp.bin_start + bin0 + dd);
            e = ld_stage<COHERENT>(bp.bin_start + bin0 + dd + 1);
        }
        if (s == e) continue;   // uniform over the CTA
        const DrawDesc &D = bp.draws[V.draw_begin + dd];
        const bool less = D.depth_less != 0;
        const bool top_left = (D.raster_flags & kRasterTopLeft) != 0;
        const unsigned long long sentinel = less ? ~0ull : 0ull;
        if (owner) s_best[pix] = sentinel;
        __syncthreads();   // the keys are reset and the depths at draw start are in place
        const float hiz = less ? hiz_max : hiz_min;
        const uint32_t n = e - s, per = (n + WARPS - 1) / WARPS;
        const uint32_t ws = s + min(n, per * (uint32_t)warp), we = s + min(n, per * (uint32_t)(warp + 1));
        unsigned long long fa = sentinel, fb = sentinel;
        for (uint32_t chunk = ws; chunk < we; chunk += 32)
            tile_chunk<COHERENT>(bp, chunk, we, x0, y0, less, top_left, hiz, s_stage[warp], s_pref[warp], s_mask[warp],
                       s_best, s_depth, capture, lane, fa, fb);
        // the warp's whole-tile results: lane holds pixels lane and lane + 32
        if (fa != sentinel) { if (less) atomicMin(&s_best[lane], fa); else atomicMax(&s_best[lane], fa); }
        if (fb != sentinel) { if (less) atomicMin(&s_best[lane + 32], fb); else atomicMax(&s_best[lane + 32], fb); }
        __syncthreads();   // every warp's fragments are in
        if (owner) {
            const unsigned long long k = s_best[pix];
            if (k != sentinel) { dcur = depth_from_key((uint32_t)(k >> 32)); win = (uint32_t)k; }
            s_depth[pix] = dcur;
        }
        __syncthreads();
        if (warp == 0) {
            // write_tile's bounds (main.c:589-603), combined in the same order as k_tile: pixel
            // lane, then lane + 32, then across lanes
            const bool v0 = x0 + (lane & 7) < (int32_t)V.width && y0 + (lane >> 3) < (int32_t)V.height;
            const bool v1 = x0 + (lane & 7) < (int32_t)V.width && y0 + (lane >> 3) + 4 < (int32_t)V.height;
            const float d0 = s_depth[lane], d1 = s_depth[lane + 32];
            float mn = 1.0f, mx = 0.0f;
            if (v0) { mn = fmin_ref(mn, d0); mx = fmax_ref(mx, d0); }
            if (v1) { mn = fmin_ref(mn, d1); mx = fmax_ref(mx, d1); }
#pragma unroll
            for (int sh = 16; sh > 0; sh >>= 1) {
                float a = __shfl_xor_sync(0xFFFFFFFFu, mn, sh), b = __shfl_xor_sync(0xFFFFFFFFu, mx, sh);
                mn = fmin_ref(mn, a);
                mx = fmax_ref(mx, b);
            }
            if (lane == 0) { s_hiz[0] = mn; s_hiz[1] = mx; }
        }
        __syncthreads();
        hiz_min = s_hiz[0];
        hiz_max = s_hiz[1];
    }

    if (valid && win != 0xFFFFFFFFu) shade_pixel<COHERENT>(bp, V, win, px, py);
    if (valid && win == 0xFFFFFFFFu && V.clear_flags) write_cleared(V, o, dcur);
    if (threadIdx.x == 0) {
        V.tile_min[t] = hiz_min;
        V.tile_max[t] = hiz_max;
    }
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 32 / WARPS) k_tile_coop(BatchParams bp) {
    __shared__ CoopSmem<WARPS> sm;
    pdl_wait();
    if (blockIdx.x == 0 && threadIdx.x == 0 && !ld_volatile_u32(bp.error)) reset_batch_counters(bp);
    tile_coop_body<WARPS>(bp, blockIdx.x, sm);
    pdl_trigger();
}

// ------------------------------------------------------------------ persistent launch
//
// The binned pipeline of a batch as one launch: a grid of at most as many CTAs as fit on the GPU at
// once (a cooperative launch, which guarantees that they are all resident) runs the stages in turn, with
// a grid-wide barrier where the separate kernels have a launch boundary:
//   vertex shading (k_vertex) | geometry (k_geometry) | clipping (k_clip) | ranks (k_rank, when
//   requested) and the bin scan (k_scan) | scatter (k_scatter) | tiles (k_tile<8>, or k_tile_coop<8>
//   when tiles are shared by warps)
// Each stage runs the same body as its kernel, over the same blocks, so the results are the same.
// The scans take their blocks in a fixed order instead of from tickets (see kTicket).
constexpr int kBatchBlock = 256;                     // 8 warps
constexpr uint32_t kGridSpinLimit = 1u << 22;        // a second or more of waiting, with the backoff
constexpr uint32_t kGridSpinLimitDebug = 1u << 14;   // kDebugStallGrid: milliseconds

union BatchSmem {
    TileSmem<kBatchBlock / 32> tile;
    CoopSmem<kBatchBlock / 32> coop;
    ScatterSmem scatter;
    ClipSmem<kBatchBlock / 32> clip;
    ScanSmem scan;
};

// Grid barrier `round` (1, 2, ...) of the persistent launch. The arrival counter starts at zero
// for every batch and counts up over the launch's barriers, so barrier `round` is passed once it
// reaches round * gridDim.x. Thread 0 of each CTA makes the CTA's writes visible (fence), arrives
// and waits; the wait is bounded, and when it runs out the error bit is set. Returns false,
// uniformly over the CTA, when the CTA must leave: its wait ran out, or an error bit is set (an
// earlier stage overflowed or timed out; the separate kernels return early on it too).
__device__ __forceinline__ bool grid_barrier(const BatchParams &bp, uint32_t round, uint32_t *s_go) {
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t go = 0;
        // failure-detection tests (kDebugStallGrid): CTA 0 leaves without arriving, so the waits of
        // all the others run out
        if (!((bp.debug_flags & kDebugStallGrid) && blockIdx.x == 0)) {
            go = 1;
            __threadfence();
            atomicAdd(bp.counters + kCtrGrid, 1u);
            const uint32_t target = round * gridDim.x;
            const uint32_t limit = (bp.debug_flags & kDebugStallGrid) ? kGridSpinLimitDebug : kGridSpinLimit;
            uint32_t spins = 0;
            while (ld_acquire_u32(bp.counters + kCtrGrid) < target) {
                if (++spins > limit) {
                    atomicOr(bp.error, kErrGridTimeout);
                    go = 0;
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
            if (ld_volatile_u32(bp.error)) go = 0;
        }
        *s_go = go;
    }
    __syncthreads();
    return *s_go != 0;
}

// Runs body(b) for every block b in [0, nb) on the persistent grid: each CTA first takes block
// blockIdx.x, then claims the next unclaimed one from the counter, one ahead (the claim is in
// flight while the current block runs). Blocks of uneven cost (tiles, triangles of a frame's
// visible and culled regions) then balance over the CTAs as a separate kernel's blocks do on the
// hardware's block scheduler. Every thread of the CTA calls it; the loop is uniform over the CTA.
template <typename Body>
__device__ __forceinline__ void claim_blocks(uint32_t *counter, uint32_t nb, uint32_t *s_next, Body &&body) {
    uint32_t b = blockIdx.x;
    while (b < nb) {
        uint32_t next = 0;
        if (threadIdx.x == 0) next = gridDim.x + atomicAdd(counter, 1u);
        body(b);
        __syncthreads();   // every thread has read the previous block number
        if (threadIdx.x == 0) *s_next = next;
        __syncthreads();
        b = *s_next;
    }
}

template <bool COOP>
__global__ void __launch_bounds__(kBatchBlock, 4) k_batch(BatchParams bp) {
    __shared__ BatchSmem sm;
    __shared__ uint32_t s_go, s_next;
    constexpr int W = kBatchBlock / 32;
    const uint32_t nctas = gridDim.x;
    uint32_t round = 0;
    if (bp.total_vertices) {   // draws whose vertices are shaded once
        const uint32_t nb = (bp.total_vertices + kVertexBlock - 1) / kVertexBlock;
        static_assert(kVertexBlock == kBatchBlock, "one vertex a thread");
        for (uint32_t b = blockIdx.x; b < nb; b += nctas) vertex_body(bp, b);
        if (!grid_barrier(bp, ++round, &s_go)) return;
    }
    claim_blocks(bp.counters + kCtrClaimGeometry, (bp.total_tris + kBatchBlock - 1) / kBatchBlock, &s_next,
                 [&](uint32_t b) { geometry_warp<true>(bp, b * kBatchBlock + threadIdx.x); });
    if (!grid_barrier(bp, ++round, &s_go)) return;
    clip_body<W, true>(bp, blockIdx.x, nctas, sm.clip);
    if (!grid_barrier(bp, ++round, &s_go)) return;
    if (bp.want_rank) {
        static_assert(kRankBlock == kBatchBlock, "rank block");
        const uint32_t per = kRankBlock * kRankItems;
        const uint32_t nb = bp.total_tris > per ? (bp.total_tris + per - 1) / per : 1u;
        for (uint32_t b = blockIdx.x; b < nb; b += nctas) {
            rank_body(bp, b, nb, sm.scan);
            __syncthreads();
        }
    }
    {
        static_assert(kScanBlock == kBatchBlock, "scan block");
        const uint32_t per = kScanBlock * kScanItems;
        const uint32_t nb = bp.total_bins > per ? (bp.total_bins + per - 1) / per : 1u;
        for (uint32_t b = blockIdx.x; b < nb; b += nctas) {
            scan_body(bp, b, nb, sm.scan);
            __syncthreads();
        }
    }
    if (!grid_barrier(bp, ++round, &s_go)) return;
    static_assert(kScatterBlock == kBatchBlock, "scatter block");
    scatter_body<false, true>(bp, blockIdx.x, nctas, sm.scatter);
    if (!grid_barrier(bp, ++round, &s_go)) return;
    if (COOP) {
        claim_blocks(bp.counters + kCtrClaimTiles, bp.total_tiles, &s_next,
                     [&](uint32_t b) { tile_coop_body<W, false, true>(bp, b, sm.coop); });
    } else {
        commit_stats(bp, blockIdx.x);
        claim_blocks(bp.counters + kCtrClaimTiles, (bp.total_tiles + W - 1) / W, &s_next,
                     [&](uint32_t b) { tile_warp<W, true>(bp, b * W + (threadIdx.x >> 5), sm.tile); });
    }
    // the last CTA to finish (one more arrival on the barrier counter) zeroes the per-batch
    // counters for the next batch, claims and arrivals included
    __syncthreads();
    if (threadIdx.x == 0 && atomicAdd(bp.counters + kCtrGrid, 1u) == (round + 1) * gridDim.x - 1) {
        __threadfence();
        reset_batch_counters(bp);
    }
    pdl_trigger();
}

// ------------------------------------------------------------------ small-draw path
//
// A batch whose every view has exactly one draw (a single mesh drawn once: the plain single draw,
// or many views of one mesh each: the differentiable loop's visibility pass) runs as three
// kernels instead of five, with no binning:
//   k_direct_raster   vertex shader per index (as main.c:698-734 does), primitive assembly, clipping
//                     and setup, then rasterisation of the CTA's triangles: hierarchical Z per
//                     (tile, triangle) against the draw-start snapshot (main.c:1005-1010), coverage
//                     (main.c:1015-1028), quantised depth (main.c:1092-1102, 1131-1132) and the test
//                     against the draw-start depth (main.c:1164-1168), each passing fragment folded
//                     into its pixel's 64-bit key (depth, order) with a global atomic max (see
//                     below). Small triangles are rasterised by their own lane, mid-sized ones by
//                     the CTA's warps (kDirectLanePixels* and the others below), larger ones and
//                     clip fans go to a queue in chunks of 4 tiles.
//   k_direct_queue    the queued chunks, spread over the whole GPU, a tile (two pixels a lane) at a time;
//                     in a batch that folds no clear, also the list of the marked tiles.
//   k_direct_resolve  one warp per 8x8 tile (per listed tile when the batch folds no clear): the
//                     winners' pixel shader and output merger, colour and
//                     depth written once (main.c:1046-1189), hierarchical Z from the new depths
//                     (write_tile, main.c:589-603), folded clears, and the keys reset to zero.
// The per-pixel result is the same fold the tile kernel computes per draw (see the top of this
// file), so outputs are bit-identical to the binned path. The keys live in one array per view, all
// zero between draws: GREATER_EQUAL keeps the maximum of (depth_key << 32 | order); LESS keeps the
// minimum, stored complemented so that both are a maximum over values that are never zero for a
// fragment that passed (0 = no fragment). The reference's binner statistics come from the
// triangles' bin rectangles: entries are summed, and every binned tile is marked in bin_count (one
// word per tile of a one-draw view), which the resolve counts, uses to skip empty tiles, and clears.
constexpr int kDirectBlock = 128;              // 4 warps
constexpr int kDirectWarps = kDirectBlock / 32;
// How a job is rasterised, by its size (measured on the single draw and the 256-view visibility
// pass). Small batches (one set-up warp per CTA, whose other warps are free): up to 8 sample pixels
// by the triangle's own lane, up to 4096 by a whole warp over the spans of its rows. Large batches
// (every warp sets up its own, mostly tiny, triangles): up to 256 pixels by the lane. Larger jobs
// and clip fans are queued.
constexpr uint32_t kDirectLanePixelsSmall = 8, kDirectWarpPixels = 4096;
constexpr uint32_t kDirectLanePixelsLarge = 256;
constexpr uint32_t kDirectChunk = 4;           // tiles per queue entry
constexpr int kDirectListCap = 64;             // per CTA: queued jobs and marked rectangles
constexpr uint32_t kJobLess = 1u << 8, kJobTopLeft = 1u << 9;   // DirectJob::flags above the bias bits

// A rasterisation job: one emitted triangle's coverage and depth parameters, from its raster
// record (TriRaster), order key and draw.
struct DirectJob {
    uint32_t A[3], B[3], C[3];        // E(x, y) = A x + B y + C, A = a << 4, B = b << 4 (wrapping:
                                      // the reference's ((a x) << 4) + ((b y) << 4) + c, main.c:1015-1025)
    float inv_area, z0, dz1, dz2;     // quantised barycentrics and depth (main.c:1092-1102, 1131-1132)
    float zbound;                     // depth bound for hierarchical Z (main.c:871)
    uint32_t key, flags;              // order key; top-left bias bits (edge k needs E >= 1) | kJob*
    uint32_t view;
    int32_t x0, y0, x1, y1;           // sample box
    uint32_t tx0, ty0, ntx, nty;      // the 8x8 tiles it spans
};

__device__ __forceinline__ DirectJob direct_job(const int4 w0, const int4 w1, const int4 w2, const int4 w3,
                                                uint32_t key, const DrawDesc &d) {
    DirectJob J;
    const uint32_t a0 = w0.x, b0 = w0.y, a1 = w0.w, b1 = w1.x, a2 = w1.z, b2 = w1.w;
    J.A[0] = a0 << kSubpix; J.B[0] = b0 << kSubpix; J.C[0] = (uint32_t)w0.z;
    J.A[1] = a1 << kSubpix; J.B[1] = b1 << kSubpix; J.C[1] = (uint32_t)w1.y;
    J.A[2] = a2 << kSubpix; J.B[2] = b2 << kSubpix; J.C[2] = (uint32_t)w2.x;
    J.inv_area = __int_as_float(w2.y);
    J.z0 = __int_as_float(w2.w);
    J.dz1 = __int_as_float(w3.x) - J.z0;
    J.dz2 = __int_as_float(w3.y) - J.z0;
    J.zbound = __int_as_float(w2.z);
    J.key = key;
    J.flags = ((int32_t)a0 > 0 || (a0 == 0 && (int32_t)b0 > 0) ? 0u : 1u) |
              ((int32_t)a1 > 0 || (a1 == 0 && (int32_t)b1 > 0) ? 0u : 2u) |
              ((int32_t)a2 > 0 || (a2 == 0 && (int32_t)b2 > 0) ? 0u : 4u) |
              (d.depth_less ? kJobLess : 0u) | ((d.raster_flags & kRasterTopLeft) ? kJobTopLeft : 0u);
    J.view = d.view;
    J.x0 = (int16_t)(w3.z & 0xFFFF); J.y0 = w3.z >> 16;
    J.x1 = (int16_t)(w3.w & 0xFFFF); J.y1 = w3.w >> 16;
    J.tx0 = (uint32_t)J.x0 >> 3; J.ty0 = (uint32_t)J.y0 >> 3;
    J.ntx = ((uint32_t)J.x1 >> 3) - J.tx0 + 1;
    J.nty = ((uint32_t)J.y1 >> 3) - J.ty0 + 1;
    return J;
}

// The fields of a view the rasteriser reads, in registers: read through the descriptor in global
// memory they would be reloaded after every atomic.
struct DirectView {
    const float *depth, *hiz;         // hiz: tile_min (GREATER_EQUAL) or tile_max (LESS)
    unsigned long long *keys;         // the view's keys
    uint32_t width, tiles_x;
    float clear_depth;
    bool depth_cleared;
};

__device__ __forceinline__ DirectView direct_view(const BatchParams &bp, const ViewDesc &V, bool less) {
    DirectView v;
    v.depth = V.depth;
    v.hiz = less ? V.tile_max : V.tile_min;
    v.keys = bp.keys + V.key_base;
    v.width = V.width;
    v.tiles_x = V.tiles_x;
    v.clear_depth = V.clear_depth;
    v.depth_cleared = (V.clear_flags & kClearDepth) != 0;
    return v;
}

// Hierarchical Z per (tile, triangle) against the draw-start snapshot (main.c:1005-1010; the
// mirrored maximum for LESS); a depth clear folded into this batch resets it (main.c:1212-1214).
__device__ __forceinline__ bool direct_hiz_rejects(const DirectView &V, const DirectJob &J, uint32_t tile) {
    const bool less = (J.flags & kJobLess) != 0;
    const float hiz = V.depth_cleared ? (less ? 1.0f : 0.0f) : V.hiz[tile];
    return less ? (J.zbound > hiz) : (J.zbound < hiz);
}

// One covered-sample candidate: coverage (main.c:1028, or the top-left rule), quantised depth, the
// test against the draw-start depth (main.c:1164-1168), and the fold into the pixel's key.
__device__ __forceinline__ void direct_pixel(const DirectView &V, const DirectJob &J, uint32_t x, uint32_t y,
                                             uint32_t E0, uint32_t E1, uint32_t E2) {
    const uint32_t f = J.flags;
    const bool covered = (f & kJobTopLeft) ? (int32_t)((E0 - (f & 1u)) | (E1 - ((f >> 1) & 1u)) | (E2 - ((f >> 2) & 1u))) >= 0
                                           : (int32_t)(E0 | E1 | E2) > 0;
    if (!covered) return;
    const float bb1 = (float)((int32_t)E1 >> (kSubpix * 2)) * J.inv_area;
    const float bb2 = (float)((int32_t)E2 >> (kSubpix * 2)) * J.inv_area;
    float z = J.z0 + J.dz1 * bb1;
    z = z + J.dz2 * bb2;
    const size_t o = (size_t)y * V.width + x;
    const float dstart = V.depth_cleared ? V.clear_depth : V.depth[o];
    const bool less = (f & kJobLess) != 0;
    if (!(less ? (z < dstart) : (z >= dstart))) return;
    const unsigned long long k = ((unsigned long long)depth_key(z) << 32) | J.key;
    atomicMax(V.keys + o, less ? ~k : k);
}

// One 8x8 tile (tx, ty) of a job by the warp: lane owns pixel (lane & 7, lane >> 3) and the one 4
// rows below.
__device__ __forceinline__ void direct_tile(const DirectView &V, const DirectJob &J, uint32_t tx, uint32_t ty, int lane) {
    if (direct_hiz_rejects(V, J, ty * V.tiles_x + tx)) return;   // uniform over the warp
    const int32_t px = (int32_t)(tx * 8 + (lane & 7)), pya = (int32_t)(ty * 8 + (lane >> 3)), pyb = pya + 4;
    const bool in_x = px >= J.x0 && px <= J.x1;
    const bool ina = in_x && pya >= J.y0 && pya <= J.y1, inb = in_x && pyb >= J.y0 && pyb <= J.y1;
    const uint32_t ux = (uint32_t)px, uy = (uint32_t)pya;
    const uint32_t E0 = J.A[0] * ux + J.B[0] * uy + J.C[0];
    const uint32_t E1 = J.A[1] * ux + J.B[1] * uy + J.C[1];
    const uint32_t E2 = J.A[2] * ux + J.B[2] * uy + J.C[2];
    if (ina) direct_pixel(V, J, ux, uy, E0, E1, E2);
    if (inb) direct_pixel(V, J, ux, uy + 4, E0 + (J.B[0] << 2), E1 + (J.B[1] << 2), E2 + (J.B[2] << 2));
}

// The span of row y of a job where all three edge values can be >= 0, clamped to the sample box
// (lo > hi: none), and the edge values at (x0, y). A covered sample has every edge value >= 0 (the
// inclusive rule's (E0|E1|E2) > 0 as int32, and the top-left rule's E >= bias): with e = E(x0, y),
// edge k allows x - x0 >= -e / A (A > 0) or x - x0 <= -e / A (A < 0), or nothing when A = 0 and
// e < 0. The edge values are exact integers over the box (its extent is at most 1024 pixels, see
// setup_triangle), and the crossing -e / A computed as float(-e) times a correctly rounded 1/A has a
// relative error below 2^-22, so it is within a pixel wherever it falls inside a box (crossings
// further out are clamped away); widened by one pixel the span is conservative, and the exact
// integer test then decides every pixel in it.
__device__ __forceinline__ void direct_span(const DirectJob &J, const float *rA, int32_t y, int32_t &lo, int32_t &hi,
                                            uint32_t *E) {
    const uint32_t uy = (uint32_t)y, ux0 = (uint32_t)J.x0;
    lo = J.x0;
    hi = J.x1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        E[k] = J.A[k] * ux0 + J.B[k] * uy + J.C[k];
        const int32_t a = (int32_t)J.A[k], e = (int32_t)E[k];
        const int32_t cross = (int32_t)floorf(-(float)e * rA[k]);   // where E crosses 0, from x0
        if (a > 0) lo = max(lo, J.x0 + cross - 1);
        else if (a < 0) hi = min(hi, J.x0 + cross + 1);
        else if (e < 0) hi = lo - 1;
    }
}

__device__ __forceinline__ void direct_reciprocals(const DirectJob &J, float *rA) {
#pragma unroll
    for (int k = 0; k < 3; ++k) rA[k] = J.A[k] ? __frcp_rn((float)(int32_t)J.A[k]) : 0.0f;
}

// A small job by its own lane, row by row: the whole row of a box at most 2 pixels wide or of at
// most 64 pixels, else the row's span (direct_span), with the edge values stepped by A along the row (E(x + 1) = E(x) + A,
// wrapping like the reference's int32 sums) and the hierarchical-Z test once per tile the walk
// enters.
__device__ __forceinline__ void direct_lane(const DirectView &V, const DirectJob &J) {
    const bool narrow = J.x1 - J.x0 < 2 || (uint32_t)(J.x1 - J.x0 + 1) * (uint32_t)(J.y1 - J.y0 + 1) <= 64u;
    float rA[3];
    if (!narrow) direct_reciprocals(J, rA);
    uint32_t tile_seen = 0xFFFFFFFFu;
    bool rejected = false;
    for (int32_t y = J.y0; y <= J.y1; ++y) {
        const uint32_t uy = (uint32_t)y;
        int32_t lo = J.x0, hi = J.x1;
        uint32_t E[3];
        if (narrow) {
#pragma unroll
            for (int k = 0; k < 3; ++k) E[k] = J.A[k] * (uint32_t)J.x0 + J.B[k] * uy + J.C[k];
        } else {
            direct_span(J, rA, y, lo, hi, E);
            if (lo > hi) continue;
        }
        const uint32_t skip = (uint32_t)(lo - J.x0);
        uint32_t E0 = E[0] + J.A[0] * skip, E1 = E[1] + J.A[1] * skip, E2 = E[2] + J.A[2] * skip;
        for (int32_t x = lo; x <= hi; ++x, E0 += J.A[0], E1 += J.A[1], E2 += J.A[2]) {
            const uint32_t tile = (uy >> 3) * V.tiles_x + ((uint32_t)x >> 3);
            if (tile != tile_seen) {
                tile_seen = tile;
                rejected = direct_hiz_rejects(V, J, tile);
            }
            if (!rejected) direct_pixel(V, J, (uint32_t)x, uy, E0, E1, E2);
        }
    }
}

// A job of at most kDirectWarpPixels sample pixels, by the whole warp, 32 rows at a time: lane r
// takes the span of row r of the group, a warp scan lays the spans end to end, and their pixels
// are dealt to the lanes 32 at a time (each lane finds its pixel's row by a binary search over the
// scan, held in registers and read with shuffles), so that every lane tests a pixel of the
// triangle's span rather than of its box.
__device__ __forceinline__ void direct_warp(const DirectView &V, const DirectJob &J, int lane) {
    float rA[3];
    direct_reciprocals(J, rA);
    for (int32_t ybase = J.y0; ybase <= J.y1; ybase += 32) {
        const int32_t y = ybase + lane;
        int32_t lo = 0, hi = -1;
        uint32_t E[3];
        if (y <= J.y1) direct_span(J, rA, y, lo, hi, E);
        const uint32_t n = hi >= lo ? (uint32_t)(hi - lo + 1) : 0u;
        uint32_t incl = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31), excl = incl - n;
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t i = base + (uint32_t)lane;
            // the row of pixel i: the last lane whose span starts at or before i (rows with an
            // empty span start where the next one does, so they are never the last)
            uint32_t r = 0;
#pragma unroll
            for (uint32_t step = 16; step; step >>= 1) {
                const uint32_t s0 = __shfl_sync(0xFFFFFFFFu, excl, (int)(r + step));
                if (s0 <= i) r += step;
            }
            const uint32_t s_r = __shfl_sync(0xFFFFFFFFu, excl, (int)r);
            const int32_t lo_r = __shfl_sync(0xFFFFFFFFu, lo, (int)r);
            if (i >= total) continue;
            const uint32_t ux = (uint32_t)(lo_r + (int32_t)(i - s_r)), uy = (uint32_t)(ybase + (int32_t)r);
            if (direct_hiz_rejects(V, J, (uy >> 3) * V.tiles_x + (ux >> 3))) continue;
            direct_pixel(V, J, ux, uy, J.A[0] * ux + J.B[0] * uy + J.C[0], J.A[1] * ux + J.B[1] * uy + J.C[1],
                         J.A[2] * ux + J.B[2] * uy + J.C[2]);
        }
    }
}

// Queues the chunks of a large job (or a clip fan): entries (key, record slot, first tile, tiles).
__device__ __forceinline__ void direct_push(const BatchParams &bp, uint32_t key, uint32_t rec, uint32_t ntiles,
                                            uint32_t lane_in, uint32_t lanes) {
    const uint32_t nchunks = (ntiles + kDirectChunk - 1) / kDirectChunk;
    uint32_t base = 0;
    if (lane_in == 0) base = atomicAdd(bp.counters + kCtrQueue, nchunks);
    if (lanes > 1) base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (base + nchunks > bp.queue_capacity) {
        if (lane_in == 0) {
            atomicOr(bp.error, kErrQueueOverflow);
            atomicMin(bp.error + 1, bp.batch_seq);
            atomicMax(bp.error + 5, base + nchunks);
        }
        return;
    }
    for (uint32_t c = lane_in; c < nchunks; c += lanes)
        bp.queue[base + c] = make_uint4(key, rec, c * kDirectChunk, min(kDirectChunk, ntiles - c * kDirectChunk));
}

// SW warps of the CTA set up 32 input triangles each (the others only take part in the vertex
// shader and the rasterisation): 1 for small batches, whose triangles spread thinly over the GPU,
// 4 for large ones, where the set-up is the work.
template <int SW>
__global__ void __launch_bounds__(kDirectBlock) k_direct_raster(BatchParams bp) {
    constexpr int NT = 32 * SW;                        // input triangles per CTA
    __shared__ Vtx s_v[NT][3];
    __shared__ DirectJob s_job[SW == 1 ? NT : 1];     // SW == 1: jobs for a whole warp
    __shared__ uint32_t s_cnt[SW == 1 ? NT : 1];      // 1: staged
    __shared__ uint4 s_push[kDirectListCap];           // jobs to queue: key, record, tiles
    __shared__ uint4 s_mark[kDirectListCap];           // bin rectangles to mark: first bin, nx, ny, row stride
    __shared__ uint32_t s_npush, s_nmark;
    __shared__ uint32_t s_draw;
    __shared__ uint32_t s_clip[NT], s_nclip;          // the CTA's triangles that need clipping
    __shared__ Vtx s_poly[kDirectWarps][2][kMaxClipVertices];
    pdl_wait();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t g0 = blockIdx.x * NT;
    if (warp == 0) {
        // the draw of all of the CTA's triangles when they share one (kNoDraw otherwise)
        const uint32_t last = min(g0 + NT, bp.total_tris) - 1;
        const uint32_t d = warp_find_last_le(bp.num_draws, g0, [&](uint32_t i) { return __ldg(&bp.draws[i].tri_begin); },
                                             lane);
        if (lane == 0) {
            s_npush = 0;
            s_nmark = 0;
            s_nclip = 0;
            s_draw = d + 1 < bp.num_draws && __ldg(&bp.draws[d + 1].tri_begin) <= last ? kNoDraw : d;
        }
    }
    __syncthreads();
    const uint32_t cta_draw = s_draw;
    // vertex shader, one invocation per (triangle, vertex), per index as the reference shades
    if (cta_draw != kNoDraw && !bp.draws[cta_draw].vs_cached) {
        // the CTA's triangles share a draw: a thread's invocations load all their indices, then
        // all their vertices, then shade, so that its loads are in flight together
        constexpr int kPer = (3 * NT + kDirectBlock - 1) / kDirectBlock;
        const DrawDesc &d = bp.draws[cta_draw];
        int64_t idx[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t i = threadIdx.x + (uint32_t)j * kDirectBlock, t = i / 3, g = g0 + t;
            idx[j] = -1;
            if (i < 3u * NT && g < bp.total_tris) {
                const uint32_t at = d.start_index + 3 * (g - d.tri_begin) + (i - 3 * t);
                idx[j] = (d.ib ? (int64_t)__ldg(d.ib + at) : (int64_t)at) + d.base_vertex;
            }
        }
        float in[kPer][8];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
#pragma unroll
            for (int c = 0; c < 8; ++c) in[j][c] = 0.0f;   // D3D11: out-of-range vertex fetch reads zeros
            if (idx[j] >= 0 && idx[j] < (int64_t)d.vertex_count) {
                const uint8_t *p = d.vb + (size_t)idx[j] * d.vb_stride;
                if ((((uintptr_t)p) & 15) == 0) {
                    const float4 a = __ldg((const float4 *)p), b = __ldg((const float4 *)p + 1);
                    in[j][0] = a.x; in[j][1] = a.y; in[j][2] = a.z; in[j][3] = a.w;
                    in[j][4] = b.x; in[j][5] = b.y; in[j][6] = b.z; in[j][7] = b.w;
                } else {
#pragma unroll
                    for (int c = 0; c < 8; ++c) in[j][c] = __ldg((const float *)p + c);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint32_t i = threadIdx.x + (uint32_t)j * kDirectBlock, t = i / 3, g = g0 + t;
            if (i >= 3u * NT || g >= bp.total_tris) continue;
            if (idx[j] < 0 || idx[j] >= (int64_t)d.vertex_count) atomicOr(bp.error + 2, kErrBadIndex);
            run_vs(d.vs, in[j], d.cb, d.vs_tex, s_v[t][i - 3 * t].v);
        }
    } else {
        for (uint32_t i = threadIdx.x; i < 3u * NT; i += kDirectBlock) {
            const uint32_t t = i / 3, k = i - 3 * t, g = g0 + t;
            if (g < bp.total_tris) {
                const DrawDesc &d = bp.draws[cta_draw != kNoDraw ? cta_draw : find_draw(bp, g)];
                triangle_vertex(bp, d, d.start_index + 3 * (g - d.tri_begin) + k, s_v[t][k].v);
            }
        }
    }
    __syncthreads();
    if (warp < SW) {
        // primitive assembly, clipping and setup (main.c:736-913), one thread per input triangle
        const uint32_t t = (uint32_t)(warp * 32 + lane), g = g0 + t;
        uint32_t mask = 0, entries = 0;
        if (SW == 1) s_cnt[lane] = 0;
        if (g < bp.total_tris) {
            const DrawDesc &d = bp.draws[cta_draw != kNoDraw ? cta_draw : find_draw(bp, g)];
            const ViewDesc &V = bp.views[d.view];
            const float *p0 = s_v[t][0].v, *p1 = s_v[t][1].v, *p2 = s_v[t][2].v;
            bool reject = p0[3] == 0 || p1[3] == 0 || p2[3] == 0;   // main.c:759-781
            reject = reject || (p0[0] < -p0[3] && p1[0] < -p1[3] && p2[0] < -p2[3]) ||
                     (p0[0] > +p0[3] && p1[0] > +p1[3] && p2[0] > +p2[3]) ||
                     (p0[1] < -p0[3] && p1[1] < -p1[3] && p2[1] < -p2[3]) ||
                     (p0[1] > +p0[3] && p1[1] > +p1[3] && p2[1] > +p2[3]) ||
                     (p0[2] < 0.f && p1[2] < 0.f && p2[2] < 0.f) ||
                     (p0[2] > +p0[3] && p1[2] > +p1[3] && p2[2] > +p2[3]);
            if (!reject) {
                const bool clipped = !((p0[0] >= -p0[3] && p1[0] >= -p1[3] && p2[0] >= -p2[3]) &&
                                       (p0[0] <= +p0[3] && p1[0] <= +p1[3] && p2[0] <= +p2[3]) &&
                                       (p0[1] >= -p0[3] && p1[1] >= -p1[3] && p2[1] >= -p2[3]) &&
                                       (p0[1] <= +p0[3] && p1[1] <= +p1[3] && p2[1] <= +p2[3]) &&
                                       (p0[2] >= 0.f && p1[2] >= 0.f && p2[2] >= 0.f) &&
                                       (p0[2] <= +p0[3] && p1[2] <= +p1[3] && p2[2] <= +p2[3]));
                // one emitted triangle: its bin rectangle, its record where something reads it, and
                // its job (the lane's own, or queued)
                auto emit = [&](const Setup &su, const Vtx &a, const Vtx &b, const Vtx &c, uint32_t rec, uint32_t key,
                                bool may_stage) {
                    int32_t tx0, ty0, tx1, ty1;
                    tile_range(V, su.minx, su.miny, su.maxx, su.maxy, tx0, ty0, tx1, ty1);
                    if (tx1 < tx0 || ty1 < ty0) return;
                    const uint32_t nx = (uint32_t)(tx1 - tx0 + 1), ny = (uint32_t)(ty1 - ty0 + 1);
                    const uint32_t first = V.bin_base + (uint32_t)ty0 * V.tiles_x + (uint32_t)tx0;
                    entries += nx * ny;
                    if (nx * ny <= 4) {
                        for (uint32_t y = 0; y < ny; ++y)
                            for (uint32_t x = 0; x < nx; ++x) bp.bin_count[first + y * V.tiles_x + x] = 1u;
                    } else {
                        const uint32_t m = atomicAdd(&s_nmark, 1u);
                        if (m < kDirectListCap) {
                            s_mark[m] = make_uint4(first, nx, ny, V.tiles_x);
                        } else {
                            for (uint32_t u = 0; u < nx * ny; ++u) bp.bin_count[first + (u / nx) * V.tiles_x + u % nx] = 1u;
                        }
                    }
                    if (su.tminx > su.tmaxx || su.tminy > su.tmaxy) return;   // covers no sample
                    int4 R[4];
                    raster_words(su, R);
                    const DirectJob J = direct_job(R[0], R[1], R[2], R[3], key, d);
                    const uint32_t npix = (uint32_t)(J.x1 - J.x0 + 1) * (uint32_t)(J.y1 - J.y0 + 1);
                    const uint32_t ntiles = J.ntx * J.nty;
                    const bool local = may_stage && npix <= (SW == 1 ? kDirectWarpPixels : kDirectLanePixelsLarge);
                    // the resolve reads a record unless the depth and ids come from the keys alone;
                    // the queue always rebuilds its jobs from the record
                    if (!bp.keys_only || !local) write_record(bp, rec, 0, d.ps, true, su, a, b, c);
                    if (local && npix <= (SW == 1 ? kDirectLanePixelsSmall : kDirectLanePixelsLarge)) {
                        direct_lane(direct_view(bp, V, d.depth_less != 0), J);
                    } else if (SW == 1 && local) {   // (in large batches every local job is the lane's)
                        s_job[lane] = J;
                        s_cnt[lane] = 1u;
                    } else {
                        const uint32_t m = atomicAdd(&s_npush, 1u);
                        if (m < kDirectListCap) s_push[m] = make_uint4(key, rec, ntiles, 0u);
                        else direct_push(bp, key, rec, ntiles, 0, 1);
                    }
                };
                if (!clipped) {
                    Setup su;
                    if (setup_triangle(d, s_v[t][0], s_v[t][1], s_v[t][2], su)) {
                        mask = 1;
                        emit(su, s_v[t][0], s_v[t][1], s_v[t][2], g, g << 3, true);
                    }
                } else {
                    s_clip[atomicAdd(&s_nclip, 1u)] = t;   // clipped below by a whole warp
                }
            }
        }
        // statistics (main.c:1238 and the binner's entries, main.c:937-944), staged until the
        // resolve commits them
        const uint32_t n = __reduce_add_sync(0xFFFFFFFFu, (uint32_t)__popc(mask));
        entries = __reduce_add_sync(0xFFFFFFFFu, entries);
        if (lane == 0 && n) atomicAdd(bp.stats + kStatAssembled, (unsigned long long)n);
        if (lane == 0 && entries) atomicAdd(bp.stats + kStatBinEntries, (unsigned long long)entries);
    }
    __syncthreads();
    const uint32_t nclip = s_nclip;
    if (nclip) {   // uniform over the CTA
        // the triangles that need clipping, one warp each (main.c:649-661, then 662-913): the warp
        // clips (clip_by_plane_warp), lane f sets up fan f, records it and queues it
        for (uint32_t q = (uint32_t)warp; q < nclip; q += kDirectWarps) {
            const uint32_t t = s_clip[q], g = g0 + t;
            const DrawDesc &d = bp.draws[cta_draw != kNoDraw ? cta_draw : find_draw(bp, g)];
            const ViewDesc &V = bp.views[d.view];
            Vtx *poly = s_poly[warp][0], *other = s_poly[warp][1];
            if (lane < 3) poly[lane] = s_v[t][lane];
            __syncwarp();
            int count = 3;
            for (int p = 0; p < 6; ++p)
                if (clip_by_plane_warp(poly, other, count, c_clip_planes[p], lane)) {
                    Vtx *tp = poly;
                    poly = other;
                    other = tp;
                }
            const int nf = count - 2;
            if (nf <= 0) continue;
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(bp.counters + kCtrOverflow, (uint32_t)nf);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + (uint32_t)nf > bp.overflow_capacity) {
                if (lane == 0) {
                    atomicOr(bp.error, kErrRecordOverflow);
                    atomicMin(bp.error + 1, bp.batch_seq);
                    atomicMax(bp.error + 4, base + (uint32_t)nf);
                }
                continue;
            }
            bool ok = false;
            uint32_t entries = 0;
            if (lane < min(nf, 7)) {
                Setup su;
                ok = setup_triangle(d, poly[0], poly[lane + 1], poly[lane + 2], su);
                int32_t tx0, ty0, tx1, ty1;
                if (ok) tile_range(V, su.minx, su.miny, su.maxx, su.maxy, tx0, ty0, tx1, ty1);
                if (ok && tx1 >= tx0 && ty1 >= ty0) {
                    const uint32_t rec = bp.total_tris + base + (uint32_t)lane, key = (g << 3) | (uint32_t)(lane + 1);
                    const uint32_t nx = (uint32_t)(tx1 - tx0 + 1), ny = (uint32_t)(ty1 - ty0 + 1);
                    const uint32_t first = V.bin_base + (uint32_t)ty0 * V.tiles_x + (uint32_t)tx0;
                    entries = nx * ny;
                    for (uint32_t u = 0; u < nx * ny; ++u) bp.bin_count[first + (u / nx) * V.tiles_x + u % nx] = 1u;
                    if (su.tminx <= su.tmaxx && su.tminy <= su.tmaxy) {   // covers some sample
                        int4 R[4];
                        raster_words(su, R);
                        const DirectJob J = direct_job(R[0], R[1], R[2], R[3], key, d);
                        write_record(bp, rec, 0, d.ps, true, su, poly[0], poly[lane + 1], poly[lane + 2]);
                        direct_push(bp, key, rec, J.ntx * J.nty, 0, 1);
                    }
                }
            }
            const uint32_t fans = __ballot_sync(0xFFFFFFFFu, ok);
            entries = __reduce_add_sync(0xFFFFFFFFu, entries);
            if (lane == 0) {
                // slot g holds the fans' base, by which record_of finds them from a key
                bp.raster[g].w[0] = make_int4((int)base, 0, 0, 0);
                if (fans) atomicAdd(bp.stats + kStatAssembled, (unsigned long long)__popc(fans));   // main.c:1238
                if (entries) atomicAdd(bp.stats + kStatBinEntries, (unsigned long long)entries);
            }
            __syncwarp();
        }
        __syncthreads();
    }
    // queued jobs, each pushed by a whole warp; the binned tiles of the larger rectangles, by the CTA
    const uint32_t np = min(s_npush, (uint32_t)kDirectListCap);
    for (uint32_t i = (uint32_t)warp; i < np; i += kDirectWarps) {
        const uint4 e = s_push[i];
        direct_push(bp, e.x, e.y, e.z, (uint32_t)lane, 32u);
    }
    const uint32_t nm = min(s_nmark, (uint32_t)kDirectListCap);
    for (uint32_t i = 0; i < nm; ++i) {
        const uint4 r = s_mark[i];
        for (uint32_t u = threadIdx.x; u < r.y * r.z; u += kDirectBlock) bp.bin_count[r.x + (u / r.y) * r.w + u % r.y] = 1u;
    }
    if (SW == 1) {
        // the staged jobs, one at a time by a whole warp, dealt round-robin to the CTA's 4 warps
        for (uint32_t j = (uint32_t)warp; j < (uint32_t)NT; j += kDirectWarps) {
            if (!s_cnt[j]) continue;   // uniform over the warp
            const DirectJob J = s_job[j];
            direct_warp(direct_view(bp, bp.views[J.view], (J.flags & kJobLess) != 0), J, lane);
        }
    }
    pdl_trigger();
}

// The queued chunks (large triangles and clip fans), one warp per chunk.
__global__ void __launch_bounds__(kDirectBlock) k_direct_queue(BatchParams bp) {
    pdl_wait();
    if (ld_volatile_u32(bp.error)) {   // uniform: set only by the raster kernel
        pdl_trigger();
        return;
    }
    const int lane = threadIdx.x & 31;
    const uint32_t n = min(ld_volatile_u32(bp.counters + kCtrQueue), bp.queue_capacity);
    const uint32_t nwarps = gridDim.x * kDirectWarps;
    for (uint32_t i = blockIdx.x * kDirectWarps + (threadIdx.x >> 5); i < n; i += nwarps) {
        const uint4 e = bp.queue[i];
        const DrawDesc &d = bp.draws[warp_find_last_le(bp.num_draws, e.x >> 3,
                                                       [&](uint32_t k) { return __ldg(&bp.draws[k].tri_begin); }, lane)];
        const int4 *R = bp.raster[e.y].w;
        const DirectJob J = direct_job(__ldg(R), __ldg(R + 1), __ldg(R + 2), __ldg(R + 3), e.x, d);
        const DirectView V = direct_view(bp, bp.views[J.view], d.depth_less != 0);
        for (uint32_t t = e.z; t < e.z + e.w; ++t) {
            const uint32_t ty = t / J.ntx, tx = t - ty * J.ntx;
            direct_tile(V, J, J.tx0 + tx, J.ty0 + ty, lane);
        }
    }
    if (bp.mark_list) {
        // the tiles the raster kernel marked (all marks are set: it has finished), listed for the
        // resolve, 32 tiles a warp round: one load a lane, one atomic a warp. On the small-draw
        // path a view's bins are its tiles, so a bin index is the batch's tile index.
        const uint32_t nwarps2 = gridDim.x * kDirectWarps;
        for (uint32_t base = (blockIdx.x * kDirectWarps + (threadIdx.x >> 5)) * 32u; base < bp.total_tiles;
             base += nwarps2 * 32u) {
            const uint32_t tile = base + (uint32_t)lane;
            const bool marked = tile < bp.total_tiles && bp.bin_count[tile] != 0u;
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, marked);
            if (!m) continue;
            uint32_t at = 0;
            if (lane == 0) at = atomicAdd(bp.counters + kCtrMarked, (uint32_t)__popc(m));
            at = __shfl_sync(0xFFFFFFFFu, at, 0) + (uint32_t)__popc(m & ((1u << lane) - 1u));
            if (marked && at < bp.total_tiles) bp.marked[at] = tile;
        }
    }
    pdl_trigger();
}

// One warp per 8x8 tile of the batch's views: the fragments the keys name are the draw's winners;
// shading, colour and depth writes, hierarchical Z and the folded clears as k_tile does them, then
// the keys and the tile's mark are cleared for the next draw. With keys_only the winner's depth
// and ids come from its key (the depth key is exact for every depth but -0, which a draw whose
// viewport's min_depth is +0 never produces) and no record is read.
constexpr int kResolveWarps = 4;

__global__ void __launch_bounds__(kResolveWarps * 32) k_direct_resolve(BatchParams bp) {
    __shared__ uint32_t s_active;
    pdl_wait();
    if (ld_volatile_u32(bp.error)) return;   // uniform: set only by earlier kernels
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        reset_batch_counters(bp);
        // the raster kernel's staged statistics; active bins are added below by every CTA
        for (int k : {(int)kStatAssembled, (int)kStatBinEntries}) {
            atomicAdd(bp.stats + kStatTotal + k, bp.stats[k]);
            bp.stats[k] = 0;
        }
    }
    if (threadIdx.x == 0) s_active = 0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // tile gtile of the batch, by the whole warp
    auto resolve_tile = [&](uint32_t gtile) {
        const ViewDesc &V = bp.views[find_view(bp, gtile)];
        const uint32_t t = gtile - V.tile_base;
        const DrawDesc &D = bp.draws[V.draw_begin];
        const bool less = D.depth_less != 0;
        const uint32_t tx = t % V.tiles_x, ty = t / V.tiles_x;
        const int32_t x0 = (int32_t)tx * kTile, y0 = (int32_t)ty * kTile;
        const int32_t px = x0 + (lane & 7), py0 = y0 + (lane >> 3), py1 = py0 + 4;
        const bool valid0 = px < (int32_t)V.width && py0 < (int32_t)V.height;
        const bool valid1 = px < (int32_t)V.width && py1 < (int32_t)V.height;
        const size_t o0 = (size_t)py0 * V.width + px, o1 = (size_t)py1 * V.width + px;
        const bool depth_cleared = (V.clear_flags & kClearDepth) != 0;
        unsigned long long *keys = bp.keys + V.key_base;
        const uint32_t bin = V.bin_base + t;
        const uint32_t marked = bp.bin_count[bin];
        if (!marked) {   // no triangle binned here (uniform over the warp)
            if (V.clear_flags) {
                if (valid0) write_cleared(V, o0, V.clear_depth);
                if (valid1) write_cleared(V, o1, V.clear_depth);
                if (lane == 0 && depth_cleared) {   // main.c:1212-1214
                    V.tile_min[t] = 0.0f;
                    V.tile_max[t] = 1.0f;
                }
            }
        } else {
            if (lane == 0) {
                bp.bin_count[bin] = 0u;
                atomicAdd(&s_active, 1u);
            }
            unsigned long long k0 = 0, k1 = 0;
            if (valid0) { k0 = keys[o0]; if (k0) keys[o0] = 0ull; }
            if (valid1) { k1 = keys[o1]; if (k1) keys[o1] = 0ull; }
            if (less) { k0 = k0 ? ~k0 : 0ull; k1 = k1 ? ~k1 : 0ull; }
            const uint32_t win0 = k0 ? (uint32_t)k0 : 0xFFFFFFFFu, win1 = k1 ? (uint32_t)k1 : 0xFFFFFFFFu;
            float dcur0 = 0.0f, dcur1 = 0.0f;
            if (valid0) dcur0 = k0 ? depth_from_key((uint32_t)(k0 >> 32)) : (depth_cleared ? V.clear_depth : V.depth[o0]);
            if (valid1) dcur1 = k1 ? depth_from_key((uint32_t)(k1 >> 32)) : (depth_cleared ? V.clear_depth : V.depth[o1]);
            // write_tile's bounds (main.c:589-603), in k_tile's order
            float mn = 1.0f, mx = 0.0f;
            if (valid0) { mn = fmin_ref(mn, dcur0); mx = fmax_ref(mx, dcur0); }
            if (valid1) { mn = fmin_ref(mn, dcur1); mx = fmax_ref(mx, dcur1); }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float a = __shfl_xor_sync(0xFFFFFFFFu, mn, o), b = __shfl_xor_sync(0xFFFFFFFFu, mx, o);
                mn = fmin_ref(mn, a);
                mx = fmax_ref(mx, b);
            }
            if (bp.keys_only) {
                // the null pixel shader with depth, draw-id and primitive-id outputs only
                auto keyed = [&](size_t o, uint32_t win, float dnew) {
                    if (V.clear_flags & kClearColor) V.color[o] = V.clear_color;
                    V.depth[o] = dnew;
                    if (V.vis_draw) V.vis_draw[o] = D.draw_seq;
                    if (V.vis_prim) V.vis_prim[o] = (win >> 3) - D.tri_begin;
                };
                if (valid0 && win0 != 0xFFFFFFFFu) keyed(o0, win0, dcur0);
                if (valid1 && win1 != 0xFFFFFFFFu) keyed(o1, win1, dcur1);
            } else {
                // one pixel-shader invocation per written pixel, compacted over the warp
                const uint32_t m0 = __ballot_sync(0xFFFFFFFFu, win0 != 0xFFFFFFFFu && valid0);
                const uint32_t m1 = __ballot_sync(0xFFFFFFFFu, win1 != 0xFFFFFFFFu && valid1);
                const uint32_t n0 = __popc(m0), n = n0 + __popc(m1);
                for (uint32_t q0 = 0; q0 < n; q0 += 32) {
                    const uint32_t q = q0 + lane;
                    const uint32_t half = q < n0 ? 0u : 1u;
                    uint32_t src = 0;
                    if (q < n) {
                        const uint32_t m = half ? m1 : m0, k = half ? q - n0 : q;
                        src = m == 0xFFFFFFFFu ? k : nth_set_bit(m, k);
                    }
                    const uint32_t wa = __shfl_sync(0xFFFFFFFFu, win0, src), wb = __shfl_sync(0xFFFFFFFFu, win1, src);
                    if (q >= n) continue;
                    shade_pixel(bp, V, half ? wb : wa, x0 + (int32_t)(src & 7), y0 + (int32_t)(src >> 3) + (half ? 4 : 0));
                }
            }
            if (V.clear_flags) {
                if (valid0 && win0 == 0xFFFFFFFFu) write_cleared(V, o0, dcur0);
                if (valid1 && win1 == 0xFFFFFFFFu) write_cleared(V, o1, dcur1);
            }
            if (lane == 0) {
                V.tile_min[t] = mn;
                V.tile_max[t] = mx;
            }
        }
    };
    if (bp.mark_list) {
        // only the tiles the raster kernel listed (no view folds a clear, so an unmarked tile
        // owes nothing), a warp per listed tile
        const uint32_t n = min(ld_volatile_u32(bp.counters + kCtrMarked), bp.total_tiles);
        for (uint32_t i = blockIdx.x * kResolveWarps + warp; i < n; i += gridDim.x * kResolveWarps)
            resolve_tile(bp.marked[i]);
    } else {
        const uint32_t gtile = blockIdx.x * kResolveWarps + warp;
        if (gtile < bp.total_tiles) resolve_tile(gtile);
    }
    __syncthreads();
    // active-bin statistic (main.c:937-944), straight to the totals: this kernel runs only for a
    // batch that completed
    if (threadIdx.x == 0 && s_active) atomicAdd(bp.stats + kStatTotal + kStatActiveBins, (unsigned long long)s_active);
    // the list's counter is read by every CTA, so the last one to finish zeroes it
    if (bp.mark_list && threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(bp.counters + kCtrMarkedDone, 1u) == gridDim.x - 1) {
            bp.counters[kCtrMarked] = 0u;
            bp.counters[kCtrMarkedDone] = 0u;
        }
    }
    pdl_trigger();
}

// ------------------------------------------------------------------ clears

// A grouped upload's placement: job blockIdx.y's range, 16 bytes a thread per step (the bytes past
// the last whole 16 one at a time). Sources are 16-byte aligned in the staging area, destinations
// in their resources (checked on the host).
__global__ void __launch_bounds__(256) k_upload_scatter(const uint8_t *staging, UploadJobs jobs) {
    const UploadJob j = jobs.job[blockIdx.y];
    const uint4 *src = reinterpret_cast<const uint4 *>(staging + j.src);
    uint4 *dst = reinterpret_cast<uint4 *>(j.dst);
    const uint64_t n16 = j.size >> 4;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x)
        dst[i] = __ldg(src + i);
    if (blockIdx.x == 0 && threadIdx.x < (j.size & 15u))
        j.dst[(n16 << 4) + threadIdx.x] = staging[j.src + (n16 << 4) + threadIdx.x];
}

// An eager batch's draw and view descriptors, passed in the launch's parameter block and written
// to the workspace by one CTA, so that no copy-engine transfers stand in front of the batch's
// kernels (the kernel is chained to the previous batch's like the pipeline's own: it waits until
// that batch is done reading the descriptors it overwrites).
struct DescWords {
    uint32_t w[kDescParamWords];
};

__global__ void __launch_bounds__(256) k_put_descriptors(const __grid_constant__ DescWords src, uint32_t na,
                                                         uint32_t *dst_a, uint32_t nb, uint32_t *dst_b) {
    pdl_wait();
    for (uint32_t i = threadIdx.x; i < na + nb; i += blockDim.x) {
        if (i < na) dst_a[i] = src.w[i];
        else dst_b[i - na] = src.w[i];
    }
    pdl_trigger();
}

__global__ void k_fill_u32(uint32_t *p, size_t n, uint32_t value, const uint32_t *error) {
    pdl_wait();
    if (error && ld_volatile_u32(error)) return;
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n4 = n / 4;
    const uint4 v4 = make_uint4(value, value, value, value);
    if ((((uintptr_t)p) & 15) == 0) {
        for (size_t k = i; k < n4; k += (size_t)gridDim.x * blockDim.x) reinterpret_cast<uint4 *>(p)[k] = v4;
        for (size_t k = n4 * 4 + i; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = value;
    } else {
        for (size_t k = i; k < n; k += (size_t)gridDim.x * blockDim.x) p[k] = value;
    }
}

// All clears of a segment in one launch: each block fills whole chunks of kFillChunk words,
// finding its job by binary search over chunk_begin. The jobs write disjoint memory (a segment's
// clears are de-duplicated per target on the host, keeping the last).
constexpr int kFillBlock = 256;

__global__ void __launch_bounds__(kFillBlock) k_fill_many(const FillJob *jobs, uint32_t njobs, uint32_t nchunks,
                                                          const uint32_t *error) {
    pdl_wait();
    if (error && ld_volatile_u32(error)) return;
    for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        uint32_t lo = 0, hi = njobs;   // last job with chunk_begin <= c
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(&jobs[mid].chunk_begin) <= c) lo = mid; else hi = mid;   // fill jobs
        }
        const FillJob j = jobs[lo];
        const uint64_t begin = (uint64_t)(c - j.chunk_begin) * kFillChunk;
        const uint64_t end = min(begin + kFillChunk, j.n);
        uint32_t *p = j.p + begin;
        const uint32_t cnt = (uint32_t)(end - begin);
        if ((((uintptr_t)p) & 15) == 0) {
            const uint4 v4 = make_uint4(j.value, j.value, j.value, j.value);
            for (uint32_t k = threadIdx.x; k < cnt / 4; k += kFillBlock) reinterpret_cast<uint4 *>(p)[k] = v4;
            for (uint32_t k = (cnt & ~3u) + threadIdx.x; k < cnt; k += kFillBlock) p[k] = j.value;
        } else {
            for (uint32_t k = threadIdx.x; k < cnt; k += kFillBlock) p[k] = j.value;
        }
    }
    pdl_trigger();
}

// ------------------------------------------------------------------ host-side launchers

// Launches a pipeline kernel with programmatic stream serialisation: it may be scheduled while
// the previous kernel on the stream finishes (it waits for that kernel in pdl_wait()).
template <typename... Params, typename... Args>
static cudaError_t launch_chained(void (*kernel)(Params...), uint32_t grid, uint32_t block, cudaStream_t stream,
                                  Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// a_bytes + b_bytes at most kDescParamWords * 4, both multiples of 4 (checked by the caller)
cudaError_t launch_put_descriptors(const void *a, uint32_t a_bytes, void *dst_a, const void *b, uint32_t b_bytes,
                                   void *dst_b, cudaStream_t stream) {
    DescWords src;
    memcpy(src.w, a, a_bytes);
    memcpy(src.w + a_bytes / 4, b, b_bytes);
    return launch_chained(k_put_descriptors, 1u, 256u, stream, src, a_bytes / 4, (uint32_t *)dst_a, b_bytes / 4,
                          (uint32_t *)dst_b);
}

cudaError_t launch_fill_many(const FillJob *d_jobs, uint32_t njobs, uint32_t nchunks, const uint32_t *error,
                             cudaStream_t stream) {
    if (njobs == 0 || nchunks == 0) return cudaSuccess;
    const uint32_t blocks = nchunks < 152u * 8u ? nchunks : 152u * 8u;
    return launch_chained(k_fill_many, blocks, kFillBlock, stream, d_jobs, njobs, nchunks, error);
}

void set_clip_planes(const float planes[6][4], cudaStream_t stream) {
    cudaMemcpyToSymbolAsync(c_clip_planes, planes, sizeof(float) * 24, 0, cudaMemcpyHostToDevice, stream);
}

cudaError_t launch_fill_u32(uint32_t *p, size_t n, uint32_t value, const uint32_t *error, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    int threads = 256;
    size_t blocks = (n / 4 + threads - 1) / threads;
    if (blocks < 1) blocks = 1;
    if (blocks > 152 * 16) blocks = 152 * 16;
    return launch_chained(k_fill_u32, (uint32_t)blocks, (uint32_t)threads, stream, p, n, value, error);
}

cudaError_t launch_vertex(const BatchParams &bp, cudaStream_t stream) {
    if (bp.total_vertices == 0) return cudaSuccess;
    return launch_chained(k_vertex, (bp.total_vertices + kVertexBlock - 1) / kVertexBlock, kVertexBlock, stream, bp);
}

// up to kUploadJobsPerLaunch ranges; x: CTAs per range (the largest range's 16-byte units over 256
// threads, at most 2 per SM)
cudaError_t launch_upload_scatter(const uint8_t *staging, const UploadJobs &jobs, uint32_t njobs, uint64_t max_size,
                                  int num_sms, cudaStream_t stream) {
    if (njobs == 0) return cudaSuccess;
    uint64_t x = (max_size / 16 + 255) / 256;
    const uint64_t cap = 2u * (uint64_t)(num_sms > 0 ? num_sms : 1);
    x = x < 1 ? 1 : (x > cap ? cap : x);
    k_upload_scatter<<<dim3((uint32_t)x, njobs), 256, 0, stream>>>(staging, jobs);
    return cudaGetLastError();
}

// k_geometry, then k_clip (a grid of up to 8 CTAs per SM: one warp for each listed triangle, in
// one round for up to 32 a SM)
cudaError_t launch_geometry(const BatchParams &bp, uint32_t block, int num_sms, cudaStream_t stream) {
    if (bp.total_tris == 0) return cudaSuccess;
    cudaError_t e;
    switch (block) {
        case 128: e = launch_chained(k_geometry<128>, (bp.total_tris + 127) / 128, 128, stream, bp); break;
        case 512: e = launch_chained(k_geometry<512>, (bp.total_tris + 511) / 512, 512, stream, bp); break;
        default: e = launch_chained(k_geometry<256>, (bp.total_tris + 255) / 256, 256, stream, bp); break;
    }
    if (e != cudaSuccess) return e;
    const uint32_t blocks_needed = (bp.total_tris + kClipBlock / 32 - 1) / (kClipBlock / 32);
    const uint32_t cap = 8u * (uint32_t)(num_sms > 0 ? num_sms : 1);
    return launch_chained(k_clip, blocks_needed < cap ? blocks_needed : cap, kClipBlock, stream, bp);
}

cudaError_t launch_rank(const BatchParams &bp, cudaStream_t stream) {
    const uint32_t per = kRankBlock * kRankItems;
    const uint32_t blocks = (bp.total_tris + per - 1) / per;
    return launch_chained(k_rank, blocks ? blocks : 1, kRankBlock, stream, bp);
}

cudaError_t launch_scan(const BatchParams &bp, cudaStream_t stream) {
    if (bp.total_bins <= kSmallScanBins) return launch_chained(k_scan_small, 1u, (uint32_t)kSmallScanBlock, stream, bp);
    const uint32_t per = kScanBlock * kScanItems;
    const uint32_t blocks = (bp.total_bins + per - 1) / per;
    return launch_chained(k_scan, blocks ? blocks : 1, kScanBlock, stream, bp);
}

cudaError_t launch_scatter(const BatchParams &bp, int num_sms, cudaStream_t stream) {
    // a grid of up to 8 blocks per SM strides over the input triangles (a grid of one thread per
    // triangle measured slower: more triangles in flight contend for the same bin counters)
    uint32_t blocks = (bp.total_tris + kScatterBlock - 1) / kScatterBlock;
    uint32_t cap = (uint32_t)num_sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return launch_chained(k_scatter, blocks, kScatterBlock, stream, bp);
}

cudaError_t launch_direct_raster(const BatchParams &bp, int num_sms, cudaStream_t stream) {
    // one set-up warp per CTA while that still gives every SM a few CTAs, else four
    if (bp.total_tris <= (uint32_t)num_sms * 32u * 16u)
        return launch_chained(k_direct_raster<1>, (bp.total_tris + 31) / 32, (uint32_t)kDirectBlock, stream, bp);
    return launch_chained(k_direct_raster<4>, (bp.total_tris + 127) / 128, (uint32_t)kDirectBlock, stream, bp);
}

cudaError_t launch_direct_queue(const BatchParams &bp, int num_sms, cudaStream_t stream) {
    return launch_chained(k_direct_queue, (uint32_t)num_sms * 4u, (uint32_t)kDirectBlock, stream, bp);
}

cudaError_t launch_direct_resolve(const BatchParams &bp, int num_sms, cudaStream_t stream) {
    uint32_t grid = (bp.total_tiles + kResolveWarps - 1) / kResolveWarps;
    // with a marked-tile list the CTAs stride over the listed tiles, whose number only the device
    // knows: up to 8 CTAs an SM
    if (bp.mark_list) grid = std::min<uint32_t>(grid, 8u * (uint32_t)(num_sms > 0 ? num_sms : 1));
    return launch_chained(k_direct_resolve, grid, (uint32_t)(kResolveWarps * 32), stream, bp);
}

// The persistent launch: at most as many CTAs as are resident at once (cooperative: the launch
// fails rather than start a grid whose CTAs could not all run together).
cudaError_t launch_persistent(const BatchParams &bp, uint32_t warps_per_tile, int num_sms, cudaStream_t stream) {
    const bool coop = warps_per_tile > 1;
    void (*kernel)(BatchParams) = coop ? k_batch<true> : k_batch<false>;
    static int resident[2] = {0, 0};   // CTAs per SM, the same on every device of this build's arch
    if (resident[coop] == 0) {
        int n = 0;
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, kBatchBlock, 0);
        if (e != cudaSuccess) return e;
        if (n < 1) return cudaErrorInvalidConfiguration;
        resident[coop] = n;
    }
    // no more CTAs than the batch's largest stage has blocks for: a small batch's barriers then
    // gather a few CTAs instead of every SM's (the other stages stride over whatever grid there is)
    constexpr uint32_t W = kBatchBlock / 32;
    uint64_t want = std::max<uint64_t>((bp.total_vertices + kBatchBlock - 1) / kBatchBlock,
                                       (bp.total_tris + kBatchBlock - 1) / kBatchBlock);
    want = std::max<uint64_t>(want, coop ? bp.total_tiles : (bp.total_tiles + W - 1) / W);
    const uint64_t fit = (uint64_t)resident[coop] * (uint64_t)(num_sms > 0 ? num_sms : 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((uint32_t)std::max<uint64_t>(1, std::min(want, fit)));
    cfg.blockDim = dim3(kBatchBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, bp);
}

cudaError_t launch_tile(const BatchParams &bp, uint32_t warps, uint32_t warps_per_tile, cudaStream_t stream) {
    if (warps_per_tile == 2) return launch_chained(k_tile_coop<2>, bp.total_tiles, 64, stream, bp);
    if (warps_per_tile == 4) return launch_chained(k_tile_coop<4>, bp.total_tiles, 128, stream, bp);
    if (warps_per_tile == 8) return launch_chained(k_tile_coop<8>, bp.total_tiles, 256, stream, bp);
    switch (warps) {
        case 2: return launch_chained(k_tile<2>, (bp.total_tiles + 1) / 2, 64, stream, bp);
        case 8: return launch_chained(k_tile<8>, (bp.total_tiles + 7) / 8, 256, stream, bp);
        default: return launch_chained(k_tile<4>, (bp.total_tiles + 3) / 4, 128, stream, bp);
    }
}

}  // namespace mlv
