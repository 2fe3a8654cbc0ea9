"""The largest sizes one call takes (2^31 - 1 elements, the reference's
uint work-size limit carried as check_size) and the first size past it, for
the element-wise, compaction, reduction, scan, histogram and sort paths.
Inputs come from clc_sequence (x[i] = i in the element type, wrapping), so
every result is known in closed form and only slices are read back."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NMAX = (1 << 31) - 1


def read_slice(gbc, ctx, buf, start, count):
    out = np.empty(count, dtype=buf.dtype)
    st = gbc.lib.clc_buffer_read(ctx.handle, buf.handle, start * buf.dtype.itemsize, out.nbytes,
                                 out.ctypes.data_as(C.c_void_p))
    assert st == gbc.SUCCESS, gbc.lib.clc_last_error()
    return out


def test_transform_and_copy_if_at_the_limit(ctx, gbc):
    x = gbc.DeviceBuffer(ctx, NMAX, np.uint8)
    gbc.sequence(ctx, x)  # i mod 256
    y = gbc.DeviceBuffer(ctx, NMAX, np.uint8)
    gbc.transform(ctx, x, y, "x + 1")
    for start in (0, NMAX - 300):
        idx = np.arange(start, start + 300, dtype=np.int64)
        assert np.array_equal(read_slice(gbc, ctx, y, start, 300), ((idx + 1) % 256).astype(np.uint8))
    kept = gbc.copy_if(ctx, x, y, "x == 255")
    assert kept == (NMAX - 255 + 255) // 256  # i = 255, 511, ... < NMAX
    assert np.all(read_slice(gbc, ctx, y, 0, 100) == 255) and np.all(read_slice(gbc, ctx, y, kept - 100, 100) == 255)
    del y
    too_many = gbc.DeviceBuffer(ctx, NMAX + 1, np.uint8)
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.transform(ctx, too_many, too_many, "x + 1")


def test_reduce_scan_and_histogram_at_the_limit(ctx, gbc):
    x = gbc.DeviceBuffer(ctx, NMAX, np.int32)
    gbc.sequence(ctx, x)  # i: no wrap below 2^31
    total = NMAX * (NMAX - 1) // 2
    assert int(gbc.reduce(ctx, x)) == (total + 2**31) % 2**32 - 2**31  # int32 sum wraps
    y = gbc.DeviceBuffer(ctx, NMAX, np.int32)
    wide = gbc.exclusive_scan(ctx, x, y, total=True)
    assert int(wide) == total  # the exact int64 total
    last = read_slice(gbc, ctx, y, NMAX - 3, 3).astype(np.int64)
    want = [((k * (k - 1) // 2) + 2**31) % 2**32 - 2**31 for k in (NMAX - 3, NMAX - 2, NMAX - 1)]
    assert list(last) == want
    del y
    b = gbc.DeviceBuffer(ctx, NMAX, np.uint8)
    gbc.sequence(ctx, b)
    hist = gbc.DeviceBuffer(ctx, 256, np.uint32)
    gbc.histogram_even(ctx, b, hist, 0.0, 256.0)
    want_h = np.full(256, NMAX // 256, dtype=np.int64)
    want_h[: NMAX % 256] += 1
    assert np.array_equal(hist.to_host().astype(np.int64), want_h)


def test_sort_at_the_limit(ctx, gbc):
    keys = gbc.DeviceBuffer(ctx, NMAX, np.uint32)
    vals = gbc.DeviceBuffer(ctx, NMAX, np.uint32)
    gbc.sequence(ctx, keys, NMAX - 1, np.uint32(0xFFFFFFFF))  # n-1, n-2, ..., 0 (step -1 wraps)
    gbc.sequence(ctx, vals)
    gbc.sort_by_key(ctx, keys, vals)
    for start in (0, NMAX // 2, NMAX - 257):
        idx = np.arange(start, start + 257, dtype=np.int64)
        assert np.array_equal(read_slice(gbc, ctx, keys, start, 257), idx.astype(np.uint32))
        assert np.array_equal(read_slice(gbc, ctx, vals, start, 257), (NMAX - 1 - idx).astype(np.uint32))
