"""clc_scan_i32_noalloc: the allocation-free scan for callers that cannot
allocate device memory (their memory belongs to another allocator, or a
cudaFree's device-wide synchronisation is not acceptable). It is checked
against the regular scan entry point (clc_scan_raw) through the C ABI on two
calls in a row, so the second call also proves that the shared built-in
scratch is cleared between calls. Integer scans: exact, tolerance 0.

This file is named to be collected last: a failure here leaves every other
test already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX = 1 << 28


def _regular_scan(gbc, ctx, xb, n, exclusive):
    ob = gbc.DeviceBuffer(ctx, n, np.int32)
    gbc.scan_raw(ctx, xb.device_pointer, ob.device_pointer, n, np.int32, exclusive=exclusive)
    return ob.to_host()


def test_noalloc_scan_matches_regular_scan_twice(gbc, ctx):
    rng = np.random.default_rng(77)
    cases = [((1 << 20) + 3, True), (500009, False)]  # exclusive first, then a shorter inclusive call
    for n, exclusive in cases:
        x = rng.integers(-1000, 1001, size=n, dtype=np.int64).astype(np.int32)
        xb = gbc.DeviceBuffer.from_host(ctx, x)
        ob = gbc.DeviceBuffer(ctx, n, np.int32)
        ctx.finish()
        before = ctx.memory_stats().total_allocations
        status = gbc.lib.clc_scan_i32_noalloc(C.c_void_p(xb.device_pointer), C.c_void_p(ob.device_pointer), n,
                                              int(exclusive), C.c_void_p(ctx.stream))
        assert status == gbc.SUCCESS, gbc.lib.clc_last_error()
        got = ob.to_host()  # blocking read on the same stream
        assert ctx.memory_stats().total_allocations == before  # nothing came from the context's pool
        expected = _regular_scan(gbc, ctx, xb, n, exclusive)
        np.testing.assert_array_equal(got, expected)


def test_noalloc_scan_in_place_and_limits(gbc, ctx):
    x = (np.arange(16384 * 3 + 17, dtype=np.int64) % 13 - 6).astype(np.int32)  # 3 tiles and a partial one
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    expected = _regular_scan(gbc, ctx, xb, x.size, False)
    p = C.c_void_p(xb.device_pointer)
    assert gbc.lib.clc_scan_i32_noalloc(p, p, x.size, 0, C.c_void_p(ctx.stream)) == gbc.SUCCESS
    np.testing.assert_array_equal(xb.to_host(), expected)
    # beyond the built-in scratch: rejected before anything is launched
    assert gbc.lib.clc_scan_i32_noalloc(p, p, MAX + 1, 0, C.c_void_p(ctx.stream)) == gbc.ERROR_INVALID_ARGUMENT
    assert b"2^28" in gbc.lib.clc_last_error()
    assert gbc.lib.clc_scan_i32_noalloc(p, p, 0, 0, C.c_void_p(ctx.stream)) == gbc.SUCCESS
