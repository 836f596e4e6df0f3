"""The Python binding keeps the host arrays of queued uploads alive until the context next
synchronises, because the C ABI copies from them in the background. Checked on CPU, with a
stand-in for the library's calls that reports success."""
import gc
import weakref

import numpy as np

from malevich_gb300 import api


class _OkLibrary:
    def __getattr__(self, name):
        return lambda *args: api.MLV_OK


class _Resource:
    handle = None


def _queued_context(monkeypatch):
    monkeypatch.setattr(api, "load_library", lambda: _OkLibrary())
    return api.Context(None, None)


def test_queued_sources_live_until_the_context_synchronises(monkeypatch):
    ctx = _queued_context(monkeypatch)
    a = np.arange(64, dtype=np.float32)
    b = np.zeros((4, 8), np.uint32)
    refs = [weakref.ref(a), weakref.ref(b)]
    ctx.update_buffer_async(_Resource(), a)
    ctx.update_texture_async(_Resource(), b)
    del a, b
    gc.collect()
    assert all(r() is not None for r in refs)
    ctx.stats()          # a synchronising call
    gc.collect()
    assert all(r() is None for r in refs)


def test_each_synchronising_call_releases_them(monkeypatch):
    ctx = _queued_context(monkeypatch)
    calls = [ctx.finish, ctx.reset_stats, lambda: ctx.update_buffer(_Resource(), np.zeros(4, np.float32)),
             lambda: ctx.update_texture(_Resource(), np.zeros((2, 2), np.uint32))]
    for sync in calls:
        a = np.ones(16, np.float32)
        r = weakref.ref(a)
        ctx.update_buffer_async(_Resource(), a)
        del a
        gc.collect()
        assert r() is not None
        sync()
        gc.collect()
        assert r() is None
