"""Queued uploads run on the context's copy stream and each stage of a batch waits only for the
inputs it reads (vertex buffers and the VS texture before the vertex stage, index buffers before
geometry, the PS texture before the tile kernel), in eager execution and in graph replays alike.
New contents of every kind of input must reach the next batch, old contents must come back, and a
read-back after a queued upload must see it."""
import copy

import numpy as np
import pytest

from helpers import assert_bits_equal, assert_color_close
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _changed(frame, rng):
    """The same frame with new vertex positions, flipped windings, new VS and PS textures."""
    fr = copy.deepcopy(frame)
    for d in fr.draws:
        d.vb = np.ascontiguousarray(d.vb.copy())
        d.vb[:, 0:3] += rng.uniform(-0.2, 0.2, size=3).astype(np.float32)
        ib = d.ib.copy().reshape(-1, 3)
        ib[:, [1, 2]] = ib[:, [2, 1]]          # every triangle faces the other way
        d.ib = np.ascontiguousarray(ib.reshape(-1))
    vs0, ps0 = fr.draws[0].vs_tex, fr.draws[0].ps_tex
    vs_new = scenes.Texture(np.ascontiguousarray(vs0.data[::-1].copy()), vs0.format)
    ps_new = scenes.Texture(np.ascontiguousarray(ps0.data[:, ::-1].copy()), ps0.format)
    for d in fr.draws:
        d.vs_tex, d.ps_tex = vs_new, ps_new
    return fr


def _upload(ctx, r, frame, new):
    """Queues the contents of `new` into the resources `r` created for `frame`, in the order a
    frame consumes them."""
    bufs = {}
    for key, (buf, arr) in r._buffers.items():
        bufs[key] = buf
    for kind in (api.BIND_VERTEX_BUFFER, api.BIND_INDEX_BUFFER):
        for d_old, d_new in zip(frame.draws, new.draws):
            src = d_new.vb if kind == api.BIND_VERTEX_BUFFER else d_new.ib
            old = d_old.vb if kind == api.BIND_VERTEX_BUFFER else d_old.ib
            ctx.update_buffer_async(bufs[(id(old), kind)], np.ascontiguousarray(src))
    vs_tex = r._textures[id(frame.draws[0].vs_tex.data)][0]
    ps_tex = r._textures[id(frame.draws[0].ps_tex.data)][0]
    ctx.update_texture_async(vs_tex, new.draws[0].vs_tex.data)
    ctx.update_texture_async(ps_tex, new.draws[0].ps_tex.data)


def _check(got, want):
    assert_bits_equal(got["depth"], want["depth"], "depth")
    assert_color_close(got["color"], want["color"], max_outlier_frac=1e-3)


def test_queued_uploads_reach_eager_and_replayed_batches(device):
    rng = np.random.default_rng(51)
    fr = scenes.small_scene(52, 96, 64, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_ENV_LIGHTING, n_objects=3, level=3)
    new = _changed(fr, rng)
    want_old, want_new = pyoracle.render_oracle(fr), pyoracle.render_oracle(new)
    assert not np.array_equal(want_old["depth"], want_new["depth"])
    ctx = device.immediate
    r = api.FrameRenderer(device, fr)
    r.render_batched()                     # eager
    r.render_batched()                     # captured before any queued upload
    _check(r.read(0), want_old)
    keep = []                              # queued sources must outlive the copies
    for k in range(3):
        src = new if k % 2 == 0 else fr
        _upload(ctx, r, fr, src)
        keep.append(src)
        r.render_batched()                 # re-captured with the waits, then replayed
        _check(r.read(0), want_new if k % 2 == 0 else want_old)
    # immediate (eager) draws after a queued upload
    _upload(ctx, r, fr, new)
    r.render_per_draw()
    _check(r.read(0), want_new)
    _upload(ctx, r, fr, fr)
    ctx.finish()
    r.destroy()


def test_readback_after_a_queued_upload_sees_it(device):
    ctx = device.immediate
    data = np.arange(32 * 16, dtype=np.uint32).reshape(16, 32)
    tex = api.Texture2D(device, 32, 16, api.FORMAT_R8G8B8A8_UNORM)
    ctx.update_texture_async(tex, data)
    assert np.array_equal(ctx.read_texture(tex), data)
    tex.destroy()


def _pack(arrays, align=16):
    """One byte block holding the arrays at 16-byte aligned offsets, and those offsets."""
    offs, at = [], 0
    for a in arrays:
        offs.append(at)
        at += (a.nbytes + align - 1) // align * align
    block = np.zeros(max(at, 1), np.uint8)
    for a, o in zip(arrays, offs):
        block[o:o + a.nbytes] = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    return block, offs


def _upload_grouped(ctx, r, frame, new):
    """The same contents as _upload, in three grouped uploads (vertex-stage inputs, index buffers,
    the pixel shader's texture), each one copy and one placement kernel."""
    groups = [[], [], []]
    for d_old, d_new in zip(frame.draws, new.draws):
        groups[0].append((r._buffers[(id(d_old.vb), api.BIND_VERTEX_BUFFER)][0], d_new.vb))
        groups[1].append((r._buffers[(id(d_old.ib), api.BIND_INDEX_BUFFER)][0], d_new.ib))
    groups[0].append((r._textures[id(frame.draws[0].vs_tex.data)][0], new.draws[0].vs_tex.data))
    groups[2].append((r._textures[id(frame.draws[0].ps_tex.data)][0], new.draws[0].ps_tex.data))
    for g in groups:
        block, offs = _pack([a for _, a in g])
        ctx.update_resources_async(block, [(res, o, a.nbytes) for (res, a), o in zip(g, offs)])


def test_grouped_uploads_reach_eager_and_replayed_batches(device):
    rng = np.random.default_rng(53)
    fr = scenes.small_scene(54, 96, 64, vs=scenes.VS_VERTEX_LIGHTING, ps=scenes.PS_ENV_LIGHTING, n_objects=3, level=3)
    new = _changed(fr, rng)
    want_old, want_new = pyoracle.render_oracle(fr), pyoracle.render_oracle(new)
    ctx = device.immediate
    r = api.FrameRenderer(device, fr)
    r.render_batched()
    r.render_batched()
    _check(r.read(0), want_old)
    for k in range(4):
        src = new if k % 2 == 0 else fr
        _upload_grouped(ctx, r, fr, src)
        r.render_batched()
        _check(r.read(0), want_new if k % 2 == 0 else want_old)
    # grouped and per-resource uploads give the same image
    _upload(ctx, r, fr, new)
    r.render_batched()
    one = r.read(0)
    _upload_grouped(ctx, r, fr, new)
    r.render_batched()
    two = r.read(0)
    assert np.array_equal(one["color"], two["color"]) and np.array_equal(one["depth"].view(np.uint32), two["depth"].view(np.uint32))
    r.destroy()


def test_grouped_upload_places_ranges_and_partial_tails(device):
    ctx = device.immediate
    a = np.arange(37 * 11, dtype=np.uint32).reshape(11, 37)           # 1,628 bytes: a 12-byte tail
    b = (np.arange(8 * 8, dtype=np.uint32) * 2654435761).astype(np.uint32).reshape(8, 8)
    ta = api.Texture2D(device, 37, 11, api.FORMAT_R8G8B8A8_UNORM)
    tb = api.Texture2D(device, 8, 8, api.FORMAT_R8G8B8A8_UNORM)
    block, offs = _pack([b, a])
    ctx.update_resources_async(block, [(ta, offs[1], a.nbytes), (tb, offs[0], b.nbytes)])
    assert np.array_equal(ctx.read_texture(ta), a)
    assert np.array_equal(ctx.read_texture(tb), b)
    ta.destroy()
    tb.destroy()


def test_grouped_upload_checks_its_arguments(device):
    ctx = device.immediate
    t = api.Texture2D(device, 8, 8, api.FORMAT_R8G8B8A8_UNORM)
    buf = api.Buffer(device, byte_width=256, bind=api.BIND_VERTEX_BUFFER)
    block = np.zeros(512, np.uint8)
    for bad in ([(t, 8, 256)],            # source not 16-byte aligned
                [(t, 0, 255)],            # a texture takes its whole size
                [(buf, 0, 16, 8)],        # destination not 16-byte aligned
                [(buf, 0, 512)],          # beyond the buffer
                [(buf, 400, 256)]):       # beyond the block
        with pytest.raises(api.MalevichError):
            ctx.update_resources_async(block, bad)
    ctx.update_resources_async(block, [(buf, 16, 240, 16), (t, 256, 256)])
    ctx.update_resources_async(block, [])
    ctx.finish()
    t.destroy()
    buf.destroy()
