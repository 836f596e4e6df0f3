"""Benchmark of the Malevich draw path on GB300.

Workload: the scene-scale frame (1920x1080 RGBA8 + D32, 12 draws, ~1.1M input triangles: a
512x512-cell heightfield and 11 icospheres/boxes of 5k-60k triangles; vertex_lighting_vs +
env_lighting_ps with a 2048x1024 RGBA16F radiance map and a 64x32 RGBA32F irradiance map), seeded
synthetic data. One step renders the whole frame (clears + 12 draws) as one batched command list
(a CUDA graph). The L2 cache is flushed between steps (a 256 MB write, outside the timed events).

value     input triangles per second over the K timed steps (Mtri/s), inputs resident in HBM.
e2e       the same frame through the C ABI from host buffers: every step uploads the vertex and
          index buffers and both textures from pinned host memory and reads the colour target back;
          three device handles take turns so that a step's readback overlaps the next ones' uploads;
          the inputs go up as one grouped upload (mlv_update_resources_async): one copy a step
          (e2e.serial: one context, step after step).
per_draw  the same frame drawn per draw on the immediate context (one launch sequence per draw).
gpix_per_s fragments written (the oracle's count of covered, hierarchical-Z and depth-test passing
          fragments in serial order) per second.
roofline  the dominant kernel's algorithmic bytes per launch over its CUDA-event duration, against
          the measured HBM copy bandwidth.
cpu_baseline the oracle port of the reference's pipeline core on the host cores (all threads).

--impl reference times the CPU implementation instead (the reference's own AVX2 core cannot build
on an aarch64 host, so the oracle port stands in for it there) and prints its line.
N > 1 (torchrun): every rank renders its own replica of the frame (replicas only: the path has no
exchange step); value aggregates all ranks over the max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpix/s & Mtri/s, batched vs per-draw on 1 GB300; fwd+bwd ms/view at FD tol"
WORKLOAD = ("scene-scale frame 1920x1080 RGBA8+D32, 12 draws, ~1.1M input triangles (512x512-cell "
            "heightfield + 11 icospheres/boxes of 5k-60k), vertex_lighting_vs + env_lighting_ps, "
            "radiance 2048x1024 RGBA16F, irradiance 64x32 RGBA32F, reference depth mode")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--cpu-sample-frames", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable sections")
    ap.add_argument("--no-autotune", action="store_true", help="default launch shapes for the scene frame")
    ap.add_argument("--diff-steps", type=int, default=100)
    ap.add_argument("--profile-once", action="store_true",
                    help="render the frame once (batched, eager) and exit: a short launch sequence for ncu")
    ap.add_argument("--profile-workload", default="scene", choices=["scene", "single", "multiview"],
                    help="--profile-once: the scene frame, the single draw (icosphere L5 at 1280x720) or "
                         "the 64-view batch (one batched execution at the default launch shapes)")
    ap.add_argument("--persistent", action="store_true",
                    help="--profile-once: the batch as one persistent launch (k_batch)")
    ap.add_argument("--warps-per-tile", type=int, default=0,
                    help="--profile-once: this tile-kernel shape (1, 2, 4 or 8) instead of the default")
    ap.add_argument("--small-draw-triangles", type=int, default=-1,
                    help="--profile-once / --profile-diff-views: this small-draw threshold instead of the default")
    ap.add_argument("--port-vs-reference", action="store_true",
                    help="with --impl reference: time the reference's own core and the oracle port on the same "
                         "frame and threads (x86-64 only) and exit")
    ap.add_argument("--profile-diff-views", type=int, default=0,
                    help="run the differentiable loop's visibility pass, forward and adjoint once over this "
                         "many views of its 256x256 heightfield workload and exit (a short sequence for ncu)")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (profiles/), if present."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    v = d.get(kernel)
    return None if v is None else float(v.get("bytes_per_launch", 0)) or None


def cpu_baseline(frame, frames):
    """The oracle port of the reference's pipeline core, all host threads, on `frames` frames.
    Returns the seconds per frame, the threads used and the last frame's output."""
    from oracle import pyoracle
    lib = pyoracle.oracle_lib()
    cores = os.cpu_count() or 1
    lib.orc_set_threads(cores)
    pyoracle.render_oracle(frame)   # warm-up (page-in, thread pool)
    t0 = time.perf_counter()
    out = None
    for _ in range(frames):
        out = pyoracle.render_oracle(frame)
    dt = (time.perf_counter() - t0) / frames
    return dt, cores, out


def unique_vertices(frame):
    n = 0
    for d in frame.draws:
        n += len(np.unique(d.ib[d.start_index:d.start_index + d.index_count])) if d.ib is not None else d.index_count
    return n


def frame_bytes(frame, fragments):
    """Algorithmic bytes of one frame, as the hot-path measurement plan defines them:
    4 I (indices) + 32 V (each unique vertex's 32-byte input once) + per texture
    min(its bytes, 4 taps x texel bytes x the fragments (pixel textures) or vertices (vertex
    textures) that sample it) + 8 W H (colour and depth written once; the frame's clears are
    folded into that write, so no target is read). Every datum the frame must touch, once."""
    from malevich_gb300 import scenes
    idx = sum(d.index_count for d in frame.draws)
    verts = unique_vertices(frame)
    texel = {scenes.FMT_RGBA8: 4, scenes.FMT_RGBA16F: 8, scenes.FMT_RGBA32F: 16}
    tex, seen = 0, set()
    for d in frame.draws:
        # only the shaders that sample: vertex_lighting_vs; basic, env_lighting and colour x texel PS
        vs_t = d.vs_tex if d.vs == scenes.VS_VERTEX_LIGHTING else None
        ps_t = d.ps_tex if d.ps in (scenes.PS_BASIC, scenes.PS_ENV_LIGHTING, scenes.PS_COLOR_TIMES_TEXEL) else None
        for t, users in ((ps_t, fragments), (vs_t, verts)):
            if t is not None and id(t.data) not in seen:
                seen.add(id(t.data))
                tex += min(t.data.nbytes, 4 * texel[t.format] * users)
    loaded = 0 if (frame.clear_color is not None and frame.clear_depth is not None) else 4 * frame.width * frame.height
    return {"indices": 4 * idx, "vertices": 32 * verts, "textures": tex,
            "targets": 8 * frame.width * frame.height + loaded}


def algorithmic_bytes(frame, dev_stats, written_pixels):
    """Bytes one launch of each of the two main kernels must move, counting the pipeline's own
    intermediate records as well (unlike frame_bytes): every datum the kernel touches counted once
    (re-reads that caches serve are not counted). Records are counted for every assembled
    triangle, although those that cover no sample get none (3% of the scene frame's): an
    overcount of about 1% of k_tile's bytes."""
    idx = sum(d.index_count for d in frame.draws) * 4
    uniq = 0
    for d in frame.draws:
        uniq += len(np.unique(d.ib[:d.index_count])) if d.ib is not None else d.index_count
    assembled = dev_stats["assembled_triangle_count"]
    entries = dev_stats["total_triangle_count_in_bins"]
    tris = frame.input_triangles
    # k_geometry: indices, the shaded vertices (48 B each, once), the per-input-triangle info word,
    # the assembled triangles' records (64 B raster + 80 B shading) and one bin count per entry
    geometry = idx + uniq * 48 + tris * 2 + assembled * (64 + 80) + entries * 4
    w, h = frame.width, frame.height
    bins = w * h // 64 * len(frame.draws)
    tex = 0
    seen = set()
    for d in frame.draws:
        t = d.ps_tex
        if t is not None and id(t.data) not in seen:
            seen.add(id(t.data))
            tex += t.data.nbytes
    # k_tile: bin bounds, list entries, each assembled triangle's records once, the sampled texture
    # once (capped at the footprint of 4 taps per written pixel), and the targets: when the frame
    # clears both, the clears are folded into the kernel, which writes colour + depth of every
    # pixel and reads none; otherwise it reads the depth buffer and writes the written pixels
    tex = min(tex, written_pixels * 4 * 8)
    folded = frame.clear_color is not None and frame.clear_depth is not None
    targets = w * h * 8 if folded else w * h * 4 + written_pixels * 8
    tile = bins * 4 + entries * 4 + assembled * (64 + 80) + targets + tex
    return {"k_geometry": geometry, "k_tile": tile}


def run_single_draw_section(dev, args):
    """The plain single draw: a level-5 icosphere (20,480 triangles) with basic_vs + basic_ps over a
    1024x1024 RGBA8 noise texture into 1280x720 RGBA8 + D32 (depth LESS, cleared to 1.0). The frame
    (both clears and the draw) is timed as 1,000 back-to-back frames recorded in one command list
    (one CUDA graph launch; its 8 MB working set stays in L2, which is stated) and as single-frame
    graph launches with L2 flushed before each (these include the launch latency). Algorithmic bytes per frame: indices + unique vertices (32 B) + the
    texture footprint (min(size, 4 taps x 4 B x fragments)) + colour and depth written once."""
    import torch
    from malevich_gb300 import api, autotune, scenes
    from oracle import pyoracle
    frame = scenes.config1_plain()
    ctx = dev.immediate
    base_tuning = ctx.tuning()
    r = api.FrameRenderer(dev, frame)
    r.render_batched()
    # its own launch shapes: one mesh crowds its triangles into few tiles
    tuned = autotune.autotune(dev, r, repeats=5, warmup=2) if not args.no_autotune else None
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")
    for _ in range(5):
        r.render_batched()
    ctx.finish()
    # 1,000 frames back to back in one command list (one graph launch): the device time per frame
    n = 1000
    rep = r.record_repeated(n)
    for _ in range(3):
        ctx.execute_command_list(rep)
    ctx.finish()
    reps = []
    for _ in range(5):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
        ctx.execute_command_list(rep)
        with torch.cuda.stream(stream):
            b.record(stream)
        reps.append((a, b))
    ctx.finish()
    warm_ms = float(np.median([x.elapsed_time(y) for x, y in reps])) / n
    rep.destroy()
    cold = []
    for i in range(20):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(i)
            e0.record(stream)
        r.render_batched()
        with torch.cuda.stream(stream):
            e1.record(stream)
        cold.append((e0, e1))
    ctx.finish()
    cold_ms = float(np.median([x.elapsed_time(y) for x, y in cold]))
    ctx.set_profiling(True)
    ctx.reset_stats()
    for _ in range(10):
        r.render_batched()
    stages = {k: round(v[0] / max(v[1], 1), 4) for k, v in ctx.stage_times().items()}
    st = ctx.stats()
    ctx.set_profiling(False)
    if st["kernel_launches"] == 3 * st["batch_count"]:
        # the small-draw path: its raster, queue and resolve kernels report as stages 1, 3 and 4
        stages = {"raster": stages["geometry"], "queue": stages["bin_scatter"], "resolve": stages["tile"]}
    got = r.read(0)
    r.destroy()
    ctx.set_tuning(**base_tuning)
    ost = pyoracle.render_oracle(frame)
    same_depth = bool(np.array_equal(got["depth"].view(np.uint32), ost["depth"].view(np.uint32)))
    frags = int(ost["stats"]["fragments_written"])
    d = frame.draws[0]
    nbytes = (d.index_count * 4 + len(np.unique(d.ib[:d.index_count])) * 32 + min(d.ps_tex.data.nbytes, 16 * frags)
              + frame.width * frame.height * 8)
    peak, peak_kind = measured_peaks()
    tris = frame.input_triangles
    return {"workload": "icosphere L5, 20,480 triangles, 1280x720 RGBA8 + D32, basic_vs + basic_ps, LESS",
            "ms_per_frame_back_to_back": round(warm_ms, 5), "ms_per_frame_l2_flushed": round(cold_ms, 5),
            "mtri_per_s": round(tris / (warm_ms / 1e3) / 1e6, 1), "gpix_per_s": round(frags / (warm_ms / 1e3) / 1e9, 3),
            "launch_shapes": tuned["best"] if tuned else "defaults",
            "fragments_written": frags, "depth_bit_exact_vs_oracle": same_depth, "stage_ms_eager": stages,
            "algorithmic_bytes_per_frame": int(nbytes),
            "roofline": {"bound": "hbm", "achieved_gbs_l2_flushed": round(nbytes / (cold_ms / 1e3) / 1e9, 1),
                         "peak": peak, "peak_kind": peak_kind,
                         "frac_l2_flushed": round(nbytes / (cold_ms / 1e3) / 1e9 / peak, 4),
                         "traffic": ncu_traffic("single_draw_frame")}}


def persistent_point(tuned):
    """The autotuner's fastest persistent-launch point (the defaults when it did not run)."""
    best = None
    for point, ms in (tuned or {}).get("results", []):
        if point.get("persistent_launch") and (best is None or ms < best[1]):
            best = (point, ms)
    return dict(best[0]) if best else {"persistent_launch": 1, "warps_per_tile": 1}


def time_persistent(ctx, r, point, timed, steps, reference, n_views=1):
    """The renderer's batch as one persistent launch (the binned pipeline's stages in one
    cooperative launch with grid barriers between them, `point`'s shapes): ms per batch by the
    caller's `timed`, kernel launches per batch, and whether every view's colour and depth equal
    `reference` (the kernel-per-stage outputs) bit for bit. The context's tuning is restored."""
    base = ctx.tuning()
    try:
        ctx.set_tuning(**point)
        r.render_batched()
        ms = timed(r.render_batched, steps)
        ctx.reset_stats()
        r.render_batched()
        launches = ctx.stats()["kernel_launches"]
        same = all(np.array_equal(r.read(i)[k].view(np.uint32), reference[i][k].view(np.uint32))
                   for i in range(n_views) for k in ("color", "depth"))
    finally:
        ctx.set_tuning(**base)
    return {"ms": round(ms, 4), "launches": int(launches), "images_identical": bool(same),
            "launch_shapes": {k: v for k, v in point.items() if k in ("persistent_launch", "warps_per_tile",
                                                                        "big_triangle_tiles")}}


def run_multiview_section(dev, args):
    """Batched multi-view: 64 views at seeded resolutions in {256..1024}^2, 16 icosphere/heightfield
    meshes of 2k-200k triangles, 4-16 draws per view, basic_vs + basic_ps. Launch shapes come from
    the autotuner; the batched command list (one CUDA graph) is timed against per-draw launches
    and compared with them view by view (colour and depth bit for bit)."""
    import torch
    from malevich_gb300 import api, autotune, scenes
    frames = scenes.config3_batched(seed=3)
    ctx = dev.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(dev, frames)
    r.render_batched()
    tuned = autotune.autotune(dev, r, repeats=3, warmup=1)
    stream = torch.cuda.ExternalStream(ctx.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")

    def timed(fn, n):
        for _ in range(3):
            fn()
        ctx.finish()
        evs = []
        for i in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.fill_(i)
                a.record(stream)
            fn()
            with torch.cuda.stream(stream):
                b.record(stream)
            evs.append((a, b))
        ctx.finish()
        return float(np.mean([a.elapsed_time(b) for a, b in evs]))

    ctx.reset_stats()
    batched_ms = timed(r.render_batched, args.steps)
    st = ctx.stats()
    batched = [r.read(i) for i in range(len(frames))]
    pers = time_persistent(ctx, r, persistent_point(tuned), timed, max(3, args.steps // 2), batched,
                           n_views=len(frames))
    per_draw_ms = timed(r.render_per_draw, max(3, args.steps // 2))
    same = 0
    for i in range(len(frames)):
        o = r.read(i)
        same += all(np.array_equal(o[k].view(np.uint32), batched[i][k].view(np.uint32)) for k in ("color", "depth"))
    tris = sum(d.index_count // 3 for f in frames for d in f.draws)
    pixels = sum(f.width * f.height for f in frames)
    runs = st["batch_count"] or 1
    r.destroy()
    ctx.set_tuning(**base)
    return {"views": len(frames), "draws": sum(len(f.draws) for f in frames), "input_triangles": tris,
            "pixels": pixels, "batched_ms": round(batched_ms, 4), "per_draw_ms": round(per_draw_ms, 4),
            "batched_speedup": round(per_draw_ms / batched_ms, 3),
            "batched_mtri_per_s": round(tris / (batched_ms / 1e3) / 1e6, 1),
            "assembled_per_run": st["assembled_triangle_count"] // runs,
            "views_identical_to_per_draw": "%d/%d" % (same, len(frames)),
            "persistent_launch": dict(pers, kernel_per_stage_ms=round(batched_ms, 4),
                                      speed_vs_kernel_per_stage=round(batched_ms / pers["ms"], 3)),
            "autotuned": tuned["best"], "autotune_points": len(tuned["results"]),
            "l2": "flushed between steps (256 MB write outside the timed events)"}


def run_diff_sections(dev, args):
    """The differentiable configurations through the C ABI (no autograd): (4) forward + backward
    time per view for 16 views at 512x512 of a 50k-triangle sphere; (5) an Adam loop over 256 views
    at 256x256 of a 200k-triangle heightfield with a 2048x2048 RGBA32F texture initialised to 0.5,
    fitting texture and vertex colours to a target rendered from a noise texture and colours."""
    import ctypes
    import torch
    from malevich_gb300.diff import DiffScene, visibility
    from malevich_gb300 import api, scenes
    lib = api.load_library()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    out = {}

    # --- configuration 4: forward + backward per view
    sc = scenes.diff_scene(seed=4)
    prims = visibility(dev, sc)
    ds = DiffScene(sc, prims)
    col = torch.from_numpy(sc["col"]).cuda()
    tex = torch.from_numpy(sc["tex"]).cuda()
    pos = torch.from_numpy(sc["pos"]).cuda()
    image = torch.empty((ds.views, ds.height, ds.width, 3), device="cuda")
    target = torch.rand_like(image)
    g_col, g_tex, g_pos = torch.zeros_like(col), torch.zeros_like(tex), torch.zeros_like(pos)

    def fwd_bwd():
        d = ds.desc(col, tex, pos, image=image)
        lib.mlv_diff_forward(ctypes.byref(d), sp)
        gi = 2.0 * (image - target) * ds.mask
        d = ds.desc(col, tex, pos, grad_image=gi, g_col=g_col, g_tex=g_tex, g_pos=g_pos)
        lib.mlv_diff_backward(ctypes.byref(d), sp)

    for _ in range(3):
        fwd_bwd()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    n = 20
    for _ in range(n):
        fwd_bwd()
    b.record(stream)
    torch.cuda.synchronize()
    warm = a.elapsed_time(b) / n
    # the same with L2 flushed before each forward + backward (the 16 MB texture and the images
    # would otherwise stay in the 129 MB L2 from one iteration to the next)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")
    evs = []
    for i in range(n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.fill_(i)
        e0.record(stream)
        fwd_bwd()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    cold = float(np.mean([e0.elapsed_time(e1) for e0, e1 in evs]))
    del flush
    out["config4"] = {"views": ds.views, "resolution": [ds.width, ds.height], "triangles": ds.n_tris,
                      "fwd_bwd_ms_per_view": round(cold / ds.views, 5),
                      "l2": "flushed before each forward + backward (256 MB write outside the events)",
                      "fwd_bwd_ms_per_view_back_to_back": round(warm / ds.views, 5),
                      "gradient_check": "tests/test_gpu_adjoint.py: 1e-4 relative vs the FP64 oracle adjoint"}
    del ds, image, target, g_col, g_tex, g_pos

    # --- configuration 5: batched + differentiable optimisation loop. Everything runs on the
    # immediate context's stream: the visibility command list (one graph launch for all views,
    # null pixel shader, primitive ids written straight into one [views][H][W] array), the
    # forward, the loss gradient, the adjoint and Adam. A device object of its own, so that its
    # workspace (and the HBM footprint reported) is the loop's alone.
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info()
    dev5 = api.Device(dev.ordinal)
    sc = scenes.diff_scene(seed=5, n_views=256, size=256, tex_size=2048, heightfield_cells=316)
    rng = np.random.default_rng(55)
    ctx = dev5.immediate
    cstream = torch.cuda.ExternalStream(ctx.stream())
    csp = ctypes.c_void_p(ctx.stream())
    with torch.cuda.stream(cstream):
        tex_true = torch.from_numpy(rng.random(sc["tex"].shape).astype(np.float32)).cuda()
        col_true = torch.from_numpy(sc["col"]).cuda()
        V, S = sc["pos"].shape[0], sc["width"]
        prim = torch.empty((V, S, S), dtype=torch.int32, device="cuda")
        frames = scenes.diff_frames(sc, shade=False)
        vr = api.FrameRenderer(dev5, frames, primitive_id_memory=[prim[i].data_ptr() for i in range(V)])
        vr.render_batched()                  # sizes the workspace, captures the graph
        ds = DiffScene(sc, prim)
        pos = torch.from_numpy(sc["pos"]).cuda()
        target = torch.empty((ds.views, ds.height, ds.width, 3), device="cuda")
        d = ds.desc(col_true, tex_true, pos, image=target)
        lib.mlv_diff_forward(ctypes.byref(d), csp)
        tex = torch.full_like(tex_true, 0.5).requires_grad_()
        col = torch.full_like(col_true, 0.5).requires_grad_()
        tex.grad = torch.zeros_like(tex)
        col.grad = torch.zeros_like(col)
        opt = torch.optim.Adam([tex, col], lr=1e-2, fused=True, capturable=True)
        image = torch.empty_like(target)
        gi = torch.empty_like(target)
        d_fwd = ds.desc(col, tex, pos, image=image)
        d_bwd = ds.desc(col, tex, pos, grad_image=gi, g_col=col.grad, g_tex=tex.grad)
        phases = ("visibility", "forward", "loss_grad", "adjoint", "adam")
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(phases) + 1)] for _ in range(args.diff_steps)]

        def step(e=None):
            rec = (lambda k: e[k].record(cstream)) if e else (lambda k: None)
            rec(0)
            vr.render_batched()              # visibility of all views: one graph launch
            rec(1)
            lib.mlv_diff_forward(ctypes.byref(d_fwd), csp)
            rec(2)
            torch.sub(image, target, out=gi).mul_(2.0)
            tex.grad.zero_()
            col.grad.zero_()
            rec(3)
            lib.mlv_diff_backward(ctypes.byref(d_bwd), csp)
            rec(4)
            opt.step()
            rec(5)

        def forward_adjoint():
            # the part of a step after the visibility pass, captured below as one CUDA graph
            lib.mlv_diff_forward(ctypes.byref(d_fwd), csp)
            torch.sub(image, target, out=gi).mul_(2.0)
            tex.grad.zero_()
            col.grad.zero_()
            lib.mlv_diff_backward(ctypes.byref(d_bwd), csp)
            opt.step()

        def reset():
            # parameters and optimiser state back to the start (in place: a captured graph keeps
            # its addresses), so that every timed run is the whole fit
            tex.data.fill_(0.5)
            col.data.fill_(0.5)
            for state in opt.state.values():
                for v in state.values():
                    if torch.is_tensor(v):
                        v.zero_()

        for _ in range(3):
            step()
        # the phase breakdown: an eager run with events between the phases
        reset()
        cstream.synchronize()
        for i in range(args.diff_steps):
            step(ev[i])
        cstream.synchronize()
        phase_ms = {p: round(float(np.mean([ev[i][k].elapsed_time(ev[i][k + 1]) for i in range(args.diff_steps)])), 4)
                    for k, p in enumerate(phases)}
        # the timed run: each step is a launch pair, the visibility command list's graph and one
        # graph of forward, loss gradient, adjoint and Adam
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=cstream):
            forward_adjoint()
        reset()
        cstream.synchronize()
        free_mid, _ = torch.cuda.mem_get_info()
        g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        g0.record(cstream)
        for i in range(args.diff_steps):
            vr.render_batched()
            graph.replay()
        g1.record(cstream)
        cstream.synchronize()
        dt = (time.perf_counter() - t0) / args.diff_steps
        dev_ms = g0.elapsed_time(g1) / args.diff_steps
        free1, _ = torch.cuda.mem_get_info()
        # per-stage times of the visibility pass (one eager, profiled execution)
        ctx.set_profiling(True)
        ctx.reset_stats()
        vr.render_batched()
        vis_stages = {k: round(v[0], 4) for k, v in ctx.stage_times().items()}
        vis_stats = {k: int(v) for k, v in ctx.stats().items()}
        if vis_stats["kernel_launches"] == 3 * vis_stats["batch_count"]:   # the small-draw path
            vis_stages = {"raster": vis_stages["geometry"], "queue": vis_stages["bin_scatter"],
                          "resolve": vis_stages["tile"]}
        ctx.set_profiling(False)
        with torch.no_grad():
            gt = torch.zeros_like(tex)
            d = ds.desc(col, tex, pos, grad_image=torch.ones_like(image), g_tex=gt)
            lib.mlv_diff_backward(ctypes.byref(d), csp)
            seen = gt[..., 0] != 0
            err = (tex - tex_true)[..., :3][seen]
            rmse = float(torch.sqrt((err ** 2).mean()).item()) if err.numel() else None
            err0 = (0.5 - tex_true)[..., :3][seen]
            rmse0 = float(torch.sqrt((err0 ** 2).mean()).item()) if err0.numel() else None
            lossv = float(((image - target) ** 2).sum().item())
    out["config5"] = {"views": ds.views, "resolution": [ds.width, ds.height], "triangles": ds.n_tris,
                      "texture": [2048, 2048], "adam_steps": args.diff_steps, "lr": 1e-2,
                      "ms_per_step": round(dt * 1e3, 3), "device_ms_per_step": round(dev_ms, 3),
                      "phase_ms_eager": phase_ms, "visibility_stage_ms": vis_stages, "visibility_stats": vis_stats,
                      "hbm_footprint_gb": round((free0 - min(free_mid, free1)) / 1e9, 2),
                      "hbm_device_used_gb": round((total - min(free_mid, free1)) / 1e9, 2),
                      "texture_rmse_start": rmse0, "texture_rmse_final": rmse, "final_loss": lossv,
                      "texels_seen": int(seen.sum().item()),
                      "step": "a launch pair: the visibility pass (batched command list: one CUDA graph, null "
                              "pixel shader, the small-draw path, one draw per view) and one CUDA graph of "
                              "mlv_diff_forward + loss gradient + mlv_diff_backward + torch's fused Adam; the "
                              "phase times come from an eager run of the same step"}
    vr.destroy()
    dev5.destroy()
    return out


def profile_diff(dev, views):
    """One visibility pass (eager), forward and adjoint over `views` views of the differentiable
    loop's workload (256x256, 200k-triangle heightfield, 2048x2048 texture)."""
    import ctypes
    import torch
    from malevich_gb300.diff import DiffScene
    from malevich_gb300 import api, scenes
    lib = api.load_library()
    sc = scenes.diff_scene(seed=5, n_views=views, size=256, tex_size=2048, heightfield_cells=316)
    ctx = dev.immediate
    cstream = torch.cuda.ExternalStream(ctx.stream())
    csp = ctypes.c_void_p(ctx.stream())
    with torch.cuda.stream(cstream):
        prim = torch.empty((views, 256, 256), dtype=torch.int32, device="cuda")
        vr = api.FrameRenderer(dev, scenes.diff_frames(sc, shade=False),
                               primitive_id_memory=[prim[i].data_ptr() for i in range(views)])
        vr.render_batched()
        ds = DiffScene(sc, prim)
        col = torch.from_numpy(sc["col"]).cuda()
        tex = torch.from_numpy(sc["tex"]).cuda()
        pos = torch.from_numpy(sc["pos"]).cuda()
        image = torch.empty((views, 256, 256, 3), device="cuda")
        lib.mlv_diff_forward(ctypes.byref(ds.desc(col, tex, pos, image=image)), csp)
        g_col, g_tex = torch.zeros_like(col), torch.zeros_like(tex)
        lib.mlv_diff_backward(ctypes.byref(ds.desc(col, tex, pos, grad_image=image, g_col=g_col, g_tex=g_tex)), csp)
    cstream.synchronize()
    st = ctx.stats()
    vr.destroy()
    return {"views": views, "stats": st}


# The oracle port against the reference's own core on one x86-64 host (the reference's core is AVX2
# and builds only there), same frame, same threads: `python bench.py --impl reference
# --port-vs-reference` on that host prints these figures again.
PORT_VS_REFERENCE = {
    "host": "Intel Xeon @ 2.70 GHz, 8 logical cores (x86-64 build host)",
    "frame": "scene-scale frame, seed 2, 1,032,584 input triangles",
    "threads_8": {"reference_s_per_frame": 0.4249, "port_s_per_frame": 0.1448, "reference_over_port": 2.93},
    "threads_1": {"reference_s_per_frame": 0.9560, "port_s_per_frame": 0.8730, "reference_over_port": 1.10},
    "reading": "the port is faster than the reference on the same host, so a GPU ratio against the port "
               "understates the ratio against the reference",
}


def port_vs_reference(args):
    """Times the reference's own core and the oracle port on the same frame and threads (x86-64 with
    the reference built only), median of 7 frames after 2 warm-up frames each."""
    import platform
    from malevich_gb300 import scenes
    from oracle import pyoracle
    frame = scenes.config2_scene(seed=args.seed)
    if platform.machine() not in ("x86_64", "AMD64") or not pyoracle.reference_available(frame.width, frame.height):
        print(json.dumps({"port_vs_reference": "unavailable: the reference's core is built only on x86-64"}))
        return 0
    out = {"host_threads": os.cpu_count(), "frame_triangles": frame.input_triangles}
    for th in (os.cpu_count() or 1, 1):
        pyoracle.oracle_lib().orc_set_threads(th)

        def timed(fn):
            fn()
            fn()
            ts = []
            for _ in range(7):
                t0 = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t0)
            return statistics.median(ts)
        tr = timed(lambda: pyoracle.render_reference(frame, threads=th))
        to = timed(lambda: pyoracle.render_oracle(frame))
        out["threads_%d" % th] = {"reference_s_per_frame": round(tr, 4), "port_s_per_frame": round(to, 4),
                                  "reference_over_port": round(tr / to, 3)}
    print(json.dumps({"port_vs_reference": out}))
    return 0


def run_reference_arm(args, rank, world):
    """The reference's CPU implementation of the path on this host's cores, on the same frame: its
    own core (compiled from its sources into oracle/_ref, AVX2, x86-64 only) where it was built,
    else the oracle port of it (oracle/oracle.c, OpenMP). Rank 0 alone runs it."""
    if rank != 0:
        return 0
    import platform
    from malevich_gb300 import scenes
    frame = scenes.config2_scene(seed=args.seed)
    from oracle import pyoracle
    cores = os.cpu_count() or 1
    use_ref = platform.machine() in ("x86_64", "AMD64") and pyoracle.reference_available(frame.width, frame.height)
    if use_ref:
        render = lambda: pyoracle.render_reference(frame, threads=cores)["stats"]
        kind, note = "reference", "the reference's own core (AVX2 + OpenMP), compiled from its sources"
    else:
        pyoracle.oracle_lib().orc_set_threads(cores)
        render = lambda: pyoracle.render_oracle(frame)["stats"]
        kind, note = "port", ("the reference's own core is AVX2 C and does not build on this host (%s); the "
                              "oracle port of it (oracle/oracle.c, OpenMP) runs instead" % platform.machine())
    warmup = max(3, args.warmup)
    for _ in range(warmup):
        render()
    times, stats = [], None
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        stats = render()
        times.append(time.perf_counter() - t0)
    dt = statistics.median(times)
    tris = frame.input_triangles
    value = tris / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mtri/s", "n_gpus": world,
        "steps": len(times), "warmup": warmup, "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "input_triangles": tris, "resolution": [frame.width, frame.height],
                   "draws": len(frame.draws)},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mtri/s", "cores": cores, "kind": kind,
                         "sample": "%d full frames of the workload (median)" % len(times)},
        "e2e": {"value": round(value, 4), "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": note,
        "port_vs_reference": PORT_VS_REFERENCE,
    }
    if "fragments_written" in stats:
        line["gpix_per_s"] = round(stats["fragments_written"] / dt / 1e9, 6)
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    rank, world, local = dist_info()
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "gb300":   # the reference arm runs on the host cores only
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    if args.impl == "reference" and args.port_vs_reference:
        return port_vs_reference(args) if rank == 0 else 0
    if args.impl == "reference":
        rc = run_reference_arm(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return rc

    import torch
    from malevich_gb300 import api, build, replicas, scenes
    build.build()
    torch.cuda.set_device(local)
    dev = api.Device(local)
    ctx = dev.immediate
    if args.small_draw_triangles >= 0:
        ctx.set_tuning(small_draw_triangles=args.small_draw_triangles)
    if args.profile_diff_views:
        print(json.dumps({"profile_diff": profile_diff(dev, args.profile_diff_views)}))
        dev.destroy()
        return 0
    if args.profile_once and args.profile_workload == "single":
        frame = scenes.config1_plain()
    elif args.profile_once and args.profile_workload == "multiview":
        frame = scenes.config3_batched(seed=3)
    else:
        frame = scenes.config2_scene(seed=args.seed)
    r = api.FrameRenderer(dev, frame)
    if args.profile_once:
        if args.warps_per_tile:
            ctx.set_tuning(warps_per_tile=args.warps_per_tile)
        if args.persistent:
            ctx.set_tuning(persistent_launch=1, small_draw_triangles=0)
        r.render_batched()
        ctx.finish()
        print(json.dumps({"profile_once": True, "stats": ctx.stats()}))
        r.destroy()
        dev.destroy()
        return 0
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())

    def barrier():
        if dist:
            dist.barrier()

    # --- launch shapes from the autotuner (the outputs do not depend on them), then the warm-up
    # (the first execution sizes the workspace and captures the graph)
    from malevich_gb300 import autotune
    r.render_batched()
    # (a path forced by --small-draw-triangles stays; otherwise the tuner picks it first)
    tuned = autotune.autotune(dev, r, repeats=5, warmup=2, choose_path=args.small_draw_triangles < 0) \
        if not args.no_autotune else None
    for _ in range(max(args.warmup, 3)):
        r.render_batched()
    ctx.finish()
    st0 = ctx.stats()

    # --- timed: K batched frames, L2 flushed between them outside the events
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    wall0 = time.perf_counter()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(i)
            evs[i][0].record(stream)
        r.render_batched()
        with torch.cuda.stream(stream):
            evs[i][1].record(stream)
    ctx.finish()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier()
    clk = clocks.stop()
    st1 = ctx.stats()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = replicas.job_time(float(np.mean(step_ms)), dist, "cuda")    # the slowest rank's step
    launches = int(st1["kernel_launches"] - st0["kernel_launches"])
    frame_stats = {k: (st1[k] - st0[k]) // args.steps for k in st1}
    tris = frame.input_triangles
    value = replicas.total_units(tris, dist, "cuda") / (ms / 1e3) / 1e6   # every rank's frame

    timed_out = r.read(0)
    img, img_color = timed_out["depth"], timed_out["color"]
    r_img_written = int(np.count_nonzero(img != np.float32(frame.clear_depth)))

    # --- per-draw (immediate context, one launch sequence per draw), same flushing
    for _ in range(3):
        r.render_per_draw()
    ctx.finish()
    pd = []
    for i in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            flush.fill_(i)
            a.record(stream)
        r.render_per_draw()
        with torch.cuda.stream(stream):
            b.record(stream)
        pd.append((a, b))
    ctx.finish()
    pd_ms = float(np.mean([a.elapsed_time(b) for a, b in pd]))

    # --- the same frame as one persistent launch, timed the same way
    def timed_frames(fn, n):
        for _ in range(3):
            fn()
        ctx.finish()
        evs2 = []
        for i in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.fill_(i)
                a.record(stream)
            fn()
            with torch.cuda.stream(stream):
                b.record(stream)
            evs2.append((a, b))
        ctx.finish()
        return float(np.mean([a.elapsed_time(b) for a, b in evs2]))

    pers = time_persistent(ctx, r, persistent_point(tuned), timed_frames, args.steps, [timed_out])

    # --- per-kernel durations (stage events on the context stream), same frame, eager launches
    ctx.set_profiling(True)
    ctx.reset_stats()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(i)
        ctx.finish()
        r.render_batched()
    stages = ctx.stage_times()
    ctx.set_profiling(False)
    stage_avg = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in stages.items()}

    # --- e2e through the C ABI from pinned host buffers
    import ctypes
    pinned = {}

    def pin(a):
        if id(a) not in pinned:
            t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1)).pin_memory()
            pinned[id(a)] = (t, t.numpy())
        return pinned[id(a)][1]

    blocks = {}

    def upload_plan(rr, by_stage):
        """The renderer's resources as grouped uploads, each group one pinned block moved by one
        copy and placed by one kernel, built once and shared by the renderers of the same frame.
        by_stage: three groups, in the order the frame reads them (the vertex stage's inputs, the
        index buffers, the pixel shader's texture), so that a lone frame's earlier stages overlap
        the later copies; else one group, which with two frames in flight was faster (0.247
        against 0.263 ms per step)."""
        vs_tex_ids = {id(d.vs_tex.data) for d in frame.draws if d.vs_tex is not None}
        groups = [[], [], []] if by_stage else [[]]
        for key, (buf, arr) in rr._buffers.items():
            groups[(0 if key[1] == api.BIND_VERTEX_BUFFER else 1) if by_stage else 0].append((buf, arr))
        for tex, t in rr._textures.values():
            groups[(0 if id(t.data) in vs_tex_ids else 2) if by_stage else 0].append((tex, t.data))
        plan = []
        for g in groups:
            if not g:
                continue
            key = tuple(id(a) for _, a in g)
            if key not in blocks:
                offs, at = [], 0
                for _, a in g:
                    offs.append(at)
                    at += (a.nbytes + 15) // 16 * 16
                t = torch.empty(at, dtype=torch.uint8).pin_memory()
                block = t.numpy()
                for (_, a), o in zip(g, offs):
                    block[o:o + a.nbytes] = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
                blocks[key] = (t, block, offs)
            _, block, offs = blocks[key]
            ups = (api.Upload * len(g))()
            for i, ((res, a), o) in enumerate(zip(g, offs)):
                kind = api.UPLOAD_TEXTURE2D if isinstance(res, api.Texture2D) else api.UPLOAD_BUFFER
                ups[i] = api.Upload(kind, 0, res.handle, o, 0, a.nbytes)
            plan.append((block, ups, len(g)))
        return plan

    def issue(rr, plan):
        """One step's uploads (grouped copies from pinned blocks that stay unchanged) and its
        frame."""
        c = rr.device.immediate
        for block, ups, n in plan:
            c.lib.mlv_update_resources_async(c.handle, block.ctypes.data_as(ctypes.c_void_p), block.nbytes, ups, n)
        rr.render_batched()

    out_imgs = [torch.empty((frame.height, frame.width), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
                for _ in range(2)]

    def read(rr, k):
        c = rr.device.immediate
        c.lib.mlv_read_texture2d(c.handle, rr.targets[0][0].handle, out_imgs[k % 2].ctypes.data_as(ctypes.c_void_p), 0)

    plan1 = upload_plan(r, by_stage=True)
    h2d = sum(block.nbytes for block, _, _ in upload_plan(r, by_stage=False))
    d2h = out_imgs[0].nbytes

    # one context: upload, render and read back, step after step
    for _ in range(3):
        issue(r, plan1)
        read(r, 0)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        issue(r, plan1)
        read(r, 0)
    torch.cuda.synchronize()
    e2e_serial_s = replicas.job_time((time.perf_counter() - t0) / args.steps, dist, "cuda")

    # three device handles on this GPU, each with its own copy of the frame's resources, stream
    # and immediate context, in turn (triple-buffered frames): step k's uploads and rendering are
    # issued before step k - 2's result is read back, so frames' readbacks and rendering overlap
    # the next ones' uploads, and a step's uploads need not wait for the readback of the step
    # before it (a queued upload waits for its handle's unchecked batch). Every step still uploads
    # all its inputs and reads its image back. (Two handles: 0.246 ms per step, three: 0.239.)
    handles = 3
    extra = []
    for _ in range(handles - 1):
        dv = api.Device(local)
        dv.immediate.set_tuning(**ctx.tuning())
        rv = api.FrameRenderer(dv, frame)
        rv.render_batched()
        extra.append((dv, rv))
    ring = [(rr, upload_plan(rr, by_stage=False)) for rr in [r] + [rv for _, rv in extra]]
    for k in range(2 * handles):
        issue(*ring[k % handles])
        read(ring[k % handles][0], k)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        issue(*ring[k % handles])
        if k >= handles - 1:
            read(ring[(k - handles + 1) % handles][0], k - handles + 1)
    for k in range(max(args.steps - handles + 1, 0), args.steps):
        read(ring[k % handles][0], k)
    torch.cuda.synchronize()
    e2e_s = replicas.job_time((time.perf_counter() - t0) / args.steps, dist, "cuda")
    e2e_same = bool(np.array_equal(out_imgs[0], out_imgs[1]) and np.array_equal(out_imgs[0], r.read(0)["color"]))
    for dv, rv in extra:
        rv.destroy()
        dv.destroy()

    diff = multiview = single = None
    if not args.no_diff:
        r.destroy()
        r = None
        single = run_single_draw_section(dev, args)
        multiview = run_multiview_section(dev, args)
        diff = run_diff_sections(dev, args)

    result = None
    if rank == 0:
        # fragments written (Gpix/s numerator) and the CPU baseline come from the oracle
        cpu = None
        fragments = None
        outliers = None
        written_px = int((r_img_written) if r_img_written is not None else frame.width * frame.height)
        if not args.no_cpu_baseline:
            dt, cores, oout = cpu_baseline(frame, args.cpu_sample_frames)
            fragments = oout["stats"]["fragments_written"]
            cpu = {"value": round(tris / dt / 1e6, 4), "unit": "Mtri/s", "cores": cores, "kind": "port",
                   "sample": "%d full frames of the workload" % args.cpu_sample_frames,
                   "port_vs_reference": "on an x86-64 host with 8 threads the reference's own core took %.2fx "
                                        "the port's time on this frame (see --port-vs-reference)"
                                        % PORT_VS_REFERENCE["threads_8"]["reference_over_port"]}
            # colour parity of the timed frame against the oracle: pixels beyond +-1 LSB
            dc = np.abs(img_color.view(np.uint8).reshape(img_color.shape + (4,)).astype(np.int16) -
                        oout["color"].view(np.uint8).reshape(oout["color"].shape + (4,)).astype(np.int16)).max(axis=-1)
            nbad = int((dc > 1).sum())
            outliers = {"against": "oracle", "pixels_beyond_1lsb": nbad, "pixels": int(dc.size),
                        "fraction": round(nbad / dc.size, 7), "max_diff": int(dc.max()),
                        "depth_bit_exact": bool(np.array_equal(img.view(np.uint32), oout["depth"].view(np.uint32)))}
        peak, peak_kind = measured_peaks()
        fb = frame_bytes(frame, fragments if fragments is not None else written_px)
        fbytes = sum(fb.values())
        frame_achieved = fbytes / (ms / 1e3) / 1e9
        ab = algorithmic_bytes(frame, frame_stats, written_px)
        dominant = "k_tile" if stage_avg.get("tile", 0) >= stage_avg.get("geometry", 0) else "k_geometry"
        dur_ms = stage_avg["tile" if dominant == "k_tile" else "geometry"]
        achieved = ab[dominant] / (dur_ms / 1e3) / 1e9 if dur_ms else 0.0
        result = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mtri/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "input_triangles": tris, "resolution": [frame.width, frame.height],
                       "draws": len(frame.draws), "mode": "batched command list (CUDA graph)",
                       "launch_shapes": tuned["best"] if tuned else "defaults",
                       "l2": "flushed between steps (256 MB write outside the timed events)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "gpix_per_s": round(fragments / (ms / 1e3) / 1e9, 4) if fragments else None,
            "per_draw": {"value": round(tris / (pd_ms / 1e3) / 1e6, 3), "unit": "Mtri/s", "ms_per_frame": round(pd_ms, 4),
                         "batched_speedup": round(pd_ms / ms, 3)},
            "persistent_launch": dict(pers, speed_vs_kernel_per_stage=round(ms / pers["ms"], 3),
                                      mode="the batch's binned pipeline as one cooperative launch, grid barriers "
                                           "between its stages (the autotuner's fastest such point)"),
            "e2e": {"value": round(tris * world / e2e_s / 1e6, 3), "unit": "Mtri/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_s * 1e3, 3),
                    "mode": "three device handles in turn (triple-buffered frames): each step uploads its "
                            "inputs from pinned host memory (one grouped upload of the vertex and index buffers "
                            "and both textures: one copy, one placement kernel), renders, and reads its image "
                            "back; a step's readback overlaps the next steps' uploads",
                    "images_identical": e2e_same,
                    "serial": {"value": round(tris * world / e2e_serial_s / 1e6, 3), "unit": "Mtri/s",
                               "ms_per_step": round(e2e_serial_s * 1e3, 3),
                               "mode": "one context, upload, render and read back step after step; the uploads "
                                       "as three grouped copies, one per stage that reads them"}},
            "roofline": {"bound": "hbm", "achieved": round(frame_achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(frame_achieved / peak, 4), "peak_kind": peak_kind,
                         "counts": "the whole frame: 4 I + 32 V + sampled textures (capped at 4 taps per "
                                   "fragment or vertex) + 8 W H, over ms_per_step",
                         "algorithmic_bytes": int(fbytes), "bytes": {k: int(v) for k, v in fb.items()},
                         "traffic": ncu_traffic("frame"),
                         "kernel": {"name": dominant, "duration_ms": round(dur_ms, 4),
                                    "counts": "the kernel's own inputs and outputs once, the pipeline's "
                                              "intermediate records and bin lists included",
                                    "bytes": int(ab[dominant]), "achieved": round(achieved, 1),
                                    "frac": round(achieved / peak, 4), "traffic": ncu_traffic(dominant)}},
            "colour_outliers": outliers,
            "stage_ms": {k: round(v, 4) for k, v in stage_avg.items()},
            "frame_stats": {k: int(v) for k, v in frame_stats.items()},
            "cpu_baseline": cpu,
            "clocks": clk,
            "single_draw": single,
            "multiview": multiview,
            "differentiable": diff,
            "gpu_launches": launches,
            "wall_s_timed": round(wall, 4),
        }
        print(json.dumps(result))
    if r is not None:
        r.destroy()
    dev.destroy()
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
