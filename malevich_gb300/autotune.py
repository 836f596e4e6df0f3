"""Launch-shape autotuner for a batched workload.

The reference has no counterpart: its tile and bin sizes are compile-time constants of a CPU
binner (source/main.c:24-30) and its work per thread is one 8-wide SIMD triangle. On the GPU
the same pipeline has free launch shapes that change the speed but never the output: the tile
kernel's warps per CTA (how many 8x8 tiles a CTA carries, one warp each) or, instead, how many
warps share one tile's triangles (for frames whose triangles crowd into few tiles), the geometry
kernel's CTA size (how
many input triangles one CTA sets up and bins), and the threshold above which a triangle's bins
are counted and scattered cooperatively by a whole warp instead of by its own thread
(triangles-per-warp against warps-per-triangle), and whether the binned pipeline runs as a kernel
per stage or as one persistent launch (a grid of resident CTAs with grid-wide barriers between the
stages). The hierarchical-Z tile and the bins stay 8x8
pixels: the tile grid is observable through the reference's per-tile depth bounds
(main.c:1005-1010), so it is not tuned.

`autotune` times a renderer's batched execution (its command list, replayed as a CUDA graph)
with CUDA events on the context's stream, flushing L2 between timed runs, and leaves the fastest
setting on the context. It first picks the path: the small-draw path (no binning, for batches of
one draw per view) or the binned one (`small_draw_triangles` 0); when the small-draw path wins for
a batch that takes it, the binned path's launch shapes have no effect and are not swept. Otherwise
it sweeps every point of the launch-shape space. A batch the small-draw path cannot take (views
of several draws) leaves the context's path setting as it was.
"""
import itertools

SPACE = {
    "tile_warps_per_block": (2, 4, 8),
    "warps_per_tile": (1, 2, 4, 8),
    "geometry_block": (128, 256, 512),
    "big_triangle_tiles": (4, 8, 16, 32),
    "persistent_launch": (0, 1),
}

# The persistent launch's fixed shapes: 8 warps a CTA (8 tiles, or one tile shared by all 8 when
# warps_per_tile > 1) and 256 triangles a geometry block.
PERSISTENT_SHAPE = {"tile_warps_per_block": 8, "geometry_block": 256}


def _one_value(space, key, prefer):
    vals = space[key]
    return prefer if prefer in vals else vals[0]


def candidates(space=None):
    """Every point of the search space as a dict, in a fixed order. With several warps per tile
    the tile kernel runs one tile per CTA and tile_warps_per_block has no effect, so those points
    are kept for one value of it only (4 when the space has it, else its first). The persistent
    launch has fixed shapes (PERSISTENT_SHAPE; any warps_per_tile above 1 shares a tile among all 8
    warps), so its points are kept for those values, and for warps_per_tile 1 and its largest."""
    space = SPACE if space is None else space
    keys = sorted(space)
    points = [dict(zip(keys, vals)) for vals in itertools.product(*(space[k] for k in keys))]

    def keep(p):
        if p.get("persistent_launch"):
            for k, v in PERSISTENT_SHAPE.items():
                if k in space and p[k] != _one_value(space, k, v):
                    return False
            return "warps_per_tile" not in p or p["warps_per_tile"] in (1, max(space["warps_per_tile"]))
        if "warps_per_tile" in space and "tile_warps_per_block" in space:
            return p["warps_per_tile"] == 1 or p["tile_warps_per_block"] == _one_value(space, "tile_warps_per_block", 4)
        return True

    return [p for p in points if keep(p)]


def pick(results):
    """The fastest point of [(point, ms)]; ties keep the earlier point."""
    best = None
    for point, ms in results:
        if best is None or ms < best[1]:
            best = (point, ms)
    return best


def event_timer(context, repeats=5, warmup=2, flush_bytes=256 << 20):
    """A timer for `autotune`: runs fn warmup + repeats times on the context's stream and returns
    the median device time of the timed runs in ms (L2 flushed before each)."""
    import torch
    stream = torch.cuda.ExternalStream(context.stream())
    flush = torch.empty(flush_bytes // 4, dtype=torch.int32, device="cuda") if flush_bytes else None

    def time_fn(fn):
        for _ in range(warmup):
            fn()
        times = []
        for i in range(repeats):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                if flush is not None:
                    flush.fill_(i)
                a.record(stream)
            fn()
            with torch.cuda.stream(stream):
                b.record(stream)
            b.synchronize()
            times.append(a.elapsed_time(b))
        times.sort()
        return times[len(times) // 2]

    return time_fn


# small_draw_triangles: the binned path only, or the small-draw path wherever a batch allows it
PATHS = (0, 0xFFFFFFFF)


def launches_per_batch(ctx, renderer):
    """Kernel launches one `render_batched()` makes with the context's current tuning (None when
    the context keeps no statistics)."""
    if not hasattr(ctx, "reset_stats"):
        return None
    ctx.reset_stats()
    renderer.render_batched()
    return ctx.stats()["kernel_launches"]


def autotune(device, renderer, space=None, time_fn=None, repeats=5, warmup=2, choose_path=True):
    """Tunes `renderer.render_batched()` on the device's immediate context: the path first (when
    choose_path), then, unless the small-draw path won for this batch, every point of the
    launch-shape space. Sets the fastest setting and returns {"best": setting, "ms": ms,
    "results": [(point, ms)] of the sweep, "path": [(setting, ms)] of the path choice}. The outputs
    depend on neither; `time_fn(fn) -> ms` may be given (the default times with CUDA events)."""
    ctx = device.immediate
    time_fn = time_fn or event_timer(ctx, repeats=repeats, warmup=warmup)
    base = ctx.tuning()
    results, path = [], []
    try:
        fixed = {}
        if choose_path:
            launches = []
            # the binned path as a kernel per stage while the path is chosen (its launch count
            # tells the paths apart)
            chained = {"persistent_launch": 0} if "persistent_launch" in base else {}
            for sd in PATHS:
                ctx.set_tuning(small_draw_triangles=sd, **chained)
                launches.append(launches_per_batch(ctx, renderer))
                path.append(({"small_draw_triangles": sd}, float(time_fn(renderer.render_batched))))
            # the small-draw path runs 3 kernels a batch where the binned one runs 6 (and the same
            # clears): fewer launches with it allowed means the batch takes it. Where it does not,
            # the two settings run the same kernels, and the context keeps its own setting (which
            # decides the path of other batches, such as single draws, that were not timed)
            small = None not in launches and launches[1] < launches[0]
            if small:
                fixed, path_ms = pick(path)
            else:
                fixed = {"small_draw_triangles": base["small_draw_triangles"]}
            if small and fixed["small_draw_triangles"]:
                restore = {k: base[k] for k in chained}   # other batches keep the context's form
                ctx.set_tuning(**fixed, **restore)
                return {"best": dict(fixed), "ms": path_ms, "results": [], "path": path}
            ctx.set_tuning(**fixed)
        for point in candidates(space):
            ctx.set_tuning(**dict(point, **fixed))
            results.append((dict(point, **fixed), float(time_fn(renderer.render_batched))))
    except Exception:
        ctx.set_tuning(**base)
        raise
    best, ms = pick(results)
    ctx.set_tuning(**best)
    return {"best": best, "ms": ms, "results": results, "path": path}
