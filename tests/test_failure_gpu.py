"""Failure detection without a GPU fault: a decoupled look-back wait whose
predecessor never publishes gives up after its bounded wait (about one
second), the kernel finishes, the host reports CLC_ERROR_OPENCL, and the same
context keeps working."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_lookback_timeout_is_reported_and_context_survives(ctx, gbc, orc):
    t0 = time.perf_counter()
    status = gbc.lib.clc_selftest_lookback_timeout(ctx.handle)
    elapsed = time.perf_counter() - t0
    assert status == gbc.ERROR_OPENCL
    assert b"timed out" in gbc.lib.clc_last_error()
    assert 0.5 < elapsed < 60
    # the error was consumed; the context is usable and correct afterwards
    ctx.finish()
    x = np.arange(100000, dtype=np.int32) % 7 - 3
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    ob = gbc.DeviceBuffer(ctx, x.size, np.int32)
    gbc.inclusive_scan(ctx, xb, ob)
    assert np.array_equal(ob.to_host(), orc.std_scan(x))
