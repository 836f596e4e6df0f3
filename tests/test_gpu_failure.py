"""Failure detection on the GPU without a fault: a bounded device-side wait that runs out.

The bin scan's blocks wait for their predecessors' prefixes (a decoupled look-back), every wait
bounded. The debug flag MLV_DEBUG_STALL_LOOKBACK makes the scan's first block never publish its
prefix - a flag nothing sets - so the blocks after it give up after their iteration limit, set the
error word and publish what they have; the later kernels of the batch then skip their writes. The
test checks that the next synchronisation reports MLV_ERROR_TIMEOUT within seconds, and that the
same context then renders correctly again."""
import time

import numpy as np
import pytest

from helpers import assert_bits_equal
from malevich_gb300 import api, scenes
from oracle import pyoracle

pytestmark = pytest.mark.gpu

TIMEOUT = 5


def test_bounded_lookback_wait_runs_out_and_context_recovers(device):
    # 1920x1080: 32,400 bins, the multi-block scan with look-back (the binned path is forced)
    fr = scenes.small_scene(2600, 1920, 1080, n_objects=2, native=True)
    ctx = device.immediate
    base = ctx.tuning()
    r = api.FrameRenderer(device, fr)
    try:
        ctx.set_tuning(small_draw_triangles=0, debug_flags=api.DEBUG_STALL_LOOKBACK)
        t0 = time.perf_counter()
        with pytest.raises(api.MalevichError) as err:
            r.render_per_draw()
            ctx.finish()
        elapsed = time.perf_counter() - t0
        assert err.value.status == TIMEOUT, str(err.value)
        assert elapsed < 60.0, elapsed
        print("the bounded waits gave up after %.2f s" % elapsed)
        # the same context works again: flag off, frame rendered and checked
        ctx.set_tuning(**base)
        r.render_per_draw()
        got = r.read(0)
        want = pyoracle.render_oracle(fr)
        assert_bits_equal(got["depth"], want["depth"], "depth after the timeout")
        assert np.count_nonzero(want["depth"] != np.float32(fr.clear_depth)) > 1000
    finally:
        ctx.set_tuning(**base)
        r.destroy()
