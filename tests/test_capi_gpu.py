"""The reference's C-interface test (lib/test/Compute/capi.c:51-190, 306-342)
replayed through ctypes against libgbcompute.so on the GPU."""
import ctypes as C

import numpy as np
import pytest
from helpers import GOLDEN

pytestmark = pytest.mark.gpu


def ok(gbc, status):
    assert status == gbc.SUCCESS, gbc.lib.clc_last_error()


def test_devices(gbc):
    L = gbc.lib
    n = C.c_size_t(0)
    ok(gbc, L.clc_device_count(C.byref(n)))
    assert n.value > 0
    info = gbc.DeviceInfo()
    ok(gbc, L.clc_device_get_info(0, C.byref(info)))
    assert len(info.name) > 0 and info.is_gpu == 1 and info.has_fp64 == 1
    assert L.clc_device_get_info(n.value, C.byref(info)) == gbc.ERROR_INVALID_ARGUMENT
    assert len(L.clc_last_error()) > 0
    missing = C.c_void_p()
    assert L.clc_context_create(1000000, C.byref(missing)) == gbc.ERROR_NO_DEVICE
    assert missing.value is None


def test_buffers(gbc, ctx):
    L, h = gbc.lib, ctx.handle
    host = (np.arange(100, dtype=np.int32) * 3 - 50)
    a, b, empty = C.c_void_p(), C.c_void_p(), C.c_void_p()
    ok(gbc, L.clc_buffer_alloc(h, host.nbytes, C.byref(a)))
    ok(gbc, L.clc_buffer_alloc(h, host.nbytes, C.byref(b)))
    ok(gbc, L.clc_buffer_alloc(h, 0, C.byref(empty)))
    assert L.clc_buffer_size(a) == host.nbytes and L.clc_buffer_size(empty) == 0
    ok(gbc, L.clc_buffer_write(h, a, 0, host.nbytes, host.ctypes.data_as(C.c_void_p)))
    ok(gbc, L.clc_buffer_copy(h, a, 40, b, 0, 60 * 4))
    back = np.zeros(100, dtype=np.int32)
    ok(gbc, L.clc_buffer_read(h, b, 0, 60 * 4, back.ctypes.data_as(C.c_void_p)))
    assert np.array_equal(back[:60], host[10:70])
    assert L.clc_buffer_read(h, a, 4, host.nbytes, back.ctypes.data_as(C.c_void_p)) == gbc.ERROR_INVALID_ARGUMENT
    assert L.clc_buffer_write(h, empty, 0, 0, None) == gbc.SUCCESS
    for x in (a, b, empty):
        L.clc_buffer_release(x)
    L.clc_buffer_release(None)


def test_algorithms(gbc, ctx):
    L, h = gbc.lib, ctx.handle
    N = 10007
    i = np.arange(N, dtype=np.int64)
    host = (i * 7919 % 1000 - 500).astype(np.int32)
    expected = int(host.astype(np.int64).sum())
    inp, dst = C.c_void_p(), C.c_void_p()
    ok(gbc, L.clc_buffer_alloc(h, N * 4, C.byref(inp)))
    ok(gbc, L.clc_buffer_alloc(h, N * 4, C.byref(dst)))
    ok(gbc, L.clc_buffer_write(h, inp, 0, N * 4, host.ctypes.data_as(C.c_void_p)))
    init, res = np.zeros(1, np.int32), np.zeros(1, np.int32)
    ok(gbc, L.clc_reduce(h, inp, N, gbc.TYPE_I32, b"(a + b)", b"0", init.ctypes.data, res.ctypes.data))
    assert res[0] == GOLDEN["capi"]["sum_i32"] == np.int32(expected)
    init[0] = np.iinfo(np.int32).min
    ok(gbc, L.clc_reduce(h, inp, N, gbc.TYPE_I32, b"max(a, b)", b"INT_MIN", init.ctypes.data, res.ctypes.data))
    assert res[0] == 499
    ok(gbc, L.clc_scan(h, inp, dst, N, gbc.TYPE_I32, b"(a + b)", b"0", 0))
    out = np.zeros(N, np.int32)
    ok(gbc, L.clc_buffer_read(h, dst, 0, N * 4, out.ctypes.data_as(C.c_void_p)))
    assert out[0] == host[0] and out[N - 1] == np.int32(expected)
    ok(gbc, L.clc_sort(h, inp, gbc.TYPE_I32, None, N, 0))
    ok(gbc, L.clc_buffer_read(h, inp, 0, N * 4, out.ctypes.data_as(C.c_void_p)))
    assert np.all(out[1:] >= out[:-1])
    start, step, zero = np.array([5], np.int32), np.array([2], np.int32), np.zeros(1, np.int32)
    ok(gbc, L.clc_sequence(h, dst, N, gbc.TYPE_I32, start.ctypes.data, step.ctypes.data))
    ok(gbc, L.clc_buffer_read(h, dst, 0, N * 4, out.ctypes.data_as(C.c_void_p)))
    assert out[0] == 5 and out[N - 1] == 5 + 2 * (N - 1)
    ok(gbc, L.clc_fill(h, dst, N, gbc.TYPE_I32, zero.ctypes.data))
    ok(gbc, L.clc_buffer_read(h, dst, 0, 4, out.ctypes.data_as(C.c_void_p)))
    assert out[0] == 0
    # too many elements for the buffer; 64-bit keys through clc_sort
    assert L.clc_fill(h, dst, N + 1, gbc.TYPE_I32, zero.ctypes.data) == gbc.ERROR_INVALID_ARGUMENT
    assert L.clc_sort(h, dst, gbc.TYPE_I64, None, N // 2, 0) == gbc.ERROR_INVALID_ARGUMENT
    # an expression outside the compiled operator table
    assert L.clc_reduce(h, inp, N, gbc.TYPE_I32, b"a - b", b"0", init.ctypes.data, res.ctypes.data) == \
        gbc.ERROR_UNSUPPORTED
    # fp64 is supported on the GPU
    d = (host.astype(np.float64) * 0.25)
    db = C.c_void_p()
    ok(gbc, L.clc_buffer_alloc(h, N * 8, C.byref(db)))
    ok(gbc, L.clc_buffer_write(h, db, 0, N * 8, d.ctypes.data_as(C.c_void_p)))
    dinit, dsum = np.zeros(1), np.zeros(1)
    ok(gbc, L.clc_reduce(h, db, N, gbc.TYPE_F64, b"(a + b)", b"0.0", dinit.ctypes.data, dsum.ctypes.data))
    assert abs(dsum[0] - d.sum()) <= 1e-9 * abs(d.sum()) + 1e-9
    for x in (inp, dst, db):
        L.clc_buffer_release(x)


def test_buffer_outlives_context(gbc):
    L = gbc.lib
    c, survivor = C.c_void_p(), C.c_void_p()
    ok(gbc, L.clc_context_create(gbc.DEFAULT_DEVICE, C.byref(c)))
    v, back = np.array([42], np.int32), np.zeros(1, np.int32)
    ok(gbc, L.clc_buffer_alloc(c, 4, C.byref(survivor)))
    ok(gbc, L.clc_buffer_write(c, survivor, 0, 4, v.ctypes.data))
    ok(gbc, L.clc_buffer_read(c, survivor, 0, 4, back.ctypes.data))
    assert back[0] == 42
    L.clc_context_release(c)
    L.clc_buffer_release(survivor)


def test_context_info_and_stream(gbc, ctx):
    info = ctx.info()
    assert b"GB300" in info.name or len(info.name) > 0
    assert ctx.stream != 0
    ctx.finish()
