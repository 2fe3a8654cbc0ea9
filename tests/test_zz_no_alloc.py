"""clc_scan_i32_noalloc: the allocation-free scan for callers that cannot
allocate device memory (their memory belongs to another allocator, or a
cudaFree's device-wide synchronisation is not acceptable). It is checked
against the regular scan entry point (clc_scan_raw, itself checked against the
oracle) through the C ABI on two calls in a row, so the second call also
proves that the shared built-in scratch is cleared between calls. Integer
scans: exact, tolerance 0. The device's free memory is compared around warm
calls (nothing allocated), and a look-back wait that runs out is reported by
clc_scan_i32_noalloc_status instead of passing silently.

This file is named to be collected last: a failure here leaves every other
test already run."""
import ctypes as C
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX = 1 << 28
TILE = 16384


def _regular_scan(gbc, ctx, xb, n, exclusive):
    ob = gbc.DeviceBuffer(ctx, n, np.int32)
    gbc.scan_raw(ctx, xb.device_pointer, ob.device_pointer, n, np.int32, exclusive=exclusive)
    return ob.to_host()


def _free_device_bytes():
    torch = pytest.importorskip("torch")
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_scan_matches_regular_scan_twice(gbc, ctx):
    rng = np.random.default_rng(77)
    cases = [((1 << 20) + 3, True), (500009, False)]  # exclusive first, then a shorter inclusive call
    stream = C.c_void_p(ctx.stream)
    for n, exclusive in cases:
        x = rng.integers(-1000, 1001, size=n, dtype=np.int64).astype(np.int32)
        xb = gbc.DeviceBuffer.from_host(ctx, x)
        ob = gbc.DeviceBuffer(ctx, n, np.int32)
        ctx.finish()
        status = gbc.lib.clc_scan_i32_noalloc(C.c_void_p(xb.device_pointer), C.c_void_p(ob.device_pointer), n,
                                              int(exclusive), stream)
        assert status == gbc.SUCCESS, gbc.lib.clc_last_error()
        got = ob.to_host()  # blocking read on the same stream
        assert gbc.lib.clc_scan_i32_noalloc_status(stream) == gbc.SUCCESS, gbc.lib.clc_last_error()
        expected = _regular_scan(gbc, ctx, xb, n, exclusive)
        np.testing.assert_array_equal(got, expected)


def test_noalloc_scan_allocates_nothing(gbc, ctx):
    n = (1 << 22) + 5
    x = (np.arange(n, dtype=np.int64) % 2001 - 1000).astype(np.int32)
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    ob = gbc.DeviceBuffer(ctx, n, np.int32)
    stream = C.c_void_p(ctx.stream)
    args = (C.c_void_p(xb.device_pointer), C.c_void_p(ob.device_pointer), n, 1, stream)
    assert gbc.lib.clc_scan_i32_noalloc(*args) == gbc.SUCCESS  # the device's one-time set-up
    ctx.finish()
    free_before = _free_device_bytes()
    pool_before = ctx.memory_stats().total_allocations
    for _ in range(3):
        assert gbc.lib.clc_scan_i32_noalloc(*args) == gbc.SUCCESS
    ctx.finish()
    assert _free_device_bytes() == free_before
    assert ctx.memory_stats().total_allocations == pool_before
    assert gbc.lib.clc_scan_i32_noalloc_status(stream) == gbc.SUCCESS
    np.testing.assert_array_equal(ob.to_host(), _regular_scan(gbc, ctx, xb, n, True))


def test_noalloc_timeout_is_reported_then_cleared(gbc, ctx):
    n = 2 * TILE
    buf = gbc.DeviceBuffer.from_host(ctx, np.ones(n, dtype=np.int32))
    stream = C.c_void_p(ctx.stream)
    t0 = time.perf_counter()
    assert gbc.lib.clc_selftest_noalloc_timeout(C.c_void_p(buf.device_pointer), n, stream) == gbc.SUCCESS
    status = gbc.lib.clc_scan_i32_noalloc_status(stream)
    elapsed = time.perf_counter() - t0
    assert status == gbc.ERROR_OPENCL
    assert b"timed out" in gbc.lib.clc_last_error()
    assert 0.5 < elapsed < 60
    # reported once, then cleared; the next call is correct again
    assert gbc.lib.clc_scan_i32_noalloc_status(stream) == gbc.SUCCESS
    x = (np.arange(n + 11, dtype=np.int64) % 5 - 2).astype(np.int32)
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    ob = gbc.DeviceBuffer(ctx, x.size, np.int32)
    assert gbc.lib.clc_scan_i32_noalloc(C.c_void_p(xb.device_pointer), C.c_void_p(ob.device_pointer), x.size, 0,
                                        stream) == gbc.SUCCESS
    assert gbc.lib.clc_scan_i32_noalloc_status(stream) == gbc.SUCCESS
    np.testing.assert_array_equal(ob.to_host(), _regular_scan(gbc, ctx, xb, x.size, False))


def test_noalloc_scan_in_place_and_limits(gbc, ctx):
    x = (np.arange(TILE * 3 + 17, dtype=np.int64) % 13 - 6).astype(np.int32)  # 3 tiles and a partial one
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    expected = _regular_scan(gbc, ctx, xb, x.size, False)
    p = C.c_void_p(xb.device_pointer)
    stream = C.c_void_p(ctx.stream)
    assert gbc.lib.clc_scan_i32_noalloc(p, p, x.size, 0, stream) == gbc.SUCCESS
    np.testing.assert_array_equal(xb.to_host(), expected)
    # beyond the built-in scratch: rejected before anything is launched
    assert gbc.lib.clc_scan_i32_noalloc(p, p, MAX + 1, 0, stream) == gbc.ERROR_INVALID_ARGUMENT
    assert b"2^28" in gbc.lib.clc_last_error()
    assert gbc.lib.clc_scan_i32_noalloc(p, p, 0, 0, stream) == gbc.SUCCESS
    assert gbc.lib.clc_scan_i32_noalloc_status(stream) == gbc.SUCCESS
