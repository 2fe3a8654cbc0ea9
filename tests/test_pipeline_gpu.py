"""The sort -> reduce_by_key -> 65,536-bin histogram pipeline on the GPU
against the CPU std:: pipeline (stable_sort, a run loop, a histogram loop),
exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pipeline_gpu(gbc, ctx, keys, vals):
    n = keys.size
    kin, vin = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    ks, vs = gbc.DeviceBuffer(ctx, n, keys.dtype), gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.sort_raw(ctx, kin.device_pointer, ks.device_pointer, keys.dtype, n, vin.device_pointer, vs.device_pointer)
    ko, so = gbc.DeviceBuffer(ctx, max(n, 1), keys.dtype), gbc.DeviceBuffer(ctx, max(n, 1), np.uint64)
    co, hist = gbc.DeviceBuffer(ctx, max(n, 1), np.uint32), gbc.DeviceBuffer(ctx, 65536, np.uint32)
    runs = gbc.reduce_by_key_raw(ctx, ks.device_pointer, keys.dtype, vs.device_pointer, n, ko.device_pointer,
                                 so.device_pointer, co.device_pointer, hist.device_pointer)
    return ko.to_host()[:runs], so.to_host()[:runs], co.to_host()[:runs], hist.to_host()


@pytest.mark.parametrize("n", [1, 2, 2047, 2048, 2049, 100003, 1 << 21])
def test_pipeline_zipf_u64(ctx, gbc, orc, n):
    keys = orc.zipf_keys(n, 1.1, 1 << 16, seed=6)
    vals = np.random.default_rng(7).integers(0, 1 << 16, size=n, dtype=np.int64).astype(np.uint32)
    sk, sv = orc.std_sort(keys, vals)
    eko, eso, eco, eh = orc.std_reduce_by_key(sk, sv)
    ko, so, co, h = pipeline_gpu(gbc, ctx, keys, vals)
    assert np.array_equal(ko, eko) and np.array_equal(so, eso) and np.array_equal(co, eco)
    assert np.array_equal(h, eh) and int(h.sum()) == n


def test_reduce_by_key_long_runs_and_u32(ctx, gbc, orc):
    # runs spanning many tiles, a single run, alternating keys
    for keys in (np.repeat(np.arange(7, dtype=np.uint32), [1, 5000, 3, 20000, 1, 2, 70000]),
                 np.zeros(30000, dtype=np.uint32),
                 (np.arange(50001, dtype=np.uint32) % 2)):
        vals = (np.arange(keys.size, dtype=np.uint64) * 2654435761 % 65536).astype(np.uint32)
        eko, eso, eco, eh = orc.std_reduce_by_key(keys, vals)
        kb, vb = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
        ko, so = gbc.DeviceBuffer(ctx, keys.size, np.uint32), gbc.DeviceBuffer(ctx, keys.size, np.uint64)
        co, hist = gbc.DeviceBuffer(ctx, keys.size, np.uint32), gbc.DeviceBuffer(ctx, 65536, np.uint32)
        runs = gbc.reduce_by_key_raw(ctx, kb.device_pointer, np.uint32, vb.device_pointer, keys.size, ko.device_pointer,
                                     so.device_pointer, co.device_pointer, hist.device_pointer)
        assert runs == eko.size
        assert np.array_equal(ko.to_host()[:runs], eko) and np.array_equal(so.to_host()[:runs], eso)
        assert np.array_equal(co.to_host()[:runs], eco) and np.array_equal(hist.to_host(), eh)


def _rbk_device(gbc, ctx, keys, vals, offset):
    """reduce_by_key from device copies that start `offset` elements into
    their buffers (offset 1: keys and values not 16-byte aligned)."""
    n = keys.size
    kb = gbc.DeviceBuffer.from_host(ctx, np.concatenate([np.zeros(offset, keys.dtype), keys]))
    vb = gbc.DeviceBuffer.from_host(ctx, np.concatenate([np.zeros(offset, np.uint32), vals]))
    ko, so = gbc.DeviceBuffer(ctx, n, keys.dtype), gbc.DeviceBuffer(ctx, n, np.uint64)
    co, hist = gbc.DeviceBuffer(ctx, n, np.uint32), gbc.DeviceBuffer(ctx, 65536, np.uint32)
    runs = gbc.reduce_by_key_raw(ctx, kb.device_pointer + offset * keys.itemsize, keys.dtype,
                                 vb.device_pointer + offset * 4, n, ko.device_pointer, so.device_pointer,
                                 co.device_pointer, hist.device_pointer)
    return ko.to_host()[:runs], so.to_host()[:runs], co.to_host()[:runs], hist.to_host()


@pytest.mark.parametrize("variant", [0, 1, 2])  # 128, 64 and 256 threads per CTA
@pytest.mark.parametrize("dtype", [np.uint32, np.uint64])
def test_reduce_by_key_chunk_edges(ctx, gbc, orc, variant, dtype):
    # The kernels work on chunks of 32,768 keys: runs that start exactly at a
    # chunk's first key, end at its last, span whole chunks (no run start in
    # them), single keys on both sides of a boundary, sizes one off a chunk,
    # and unaligned keys and values.
    c = 32768
    rng = np.random.default_rng(variant * 10 + np.dtype(dtype).itemsize)
    cases = [
        np.repeat(np.arange(4, dtype=dtype), [c, c, 1, c - 1]),
        np.repeat(np.arange(5, dtype=dtype), [c - 1, 1, 3 * c, 1, 5]),
        np.repeat(np.arange(3, dtype=dtype), [1, 2 * c - 2, 1]),
        np.arange(c + 1, dtype=dtype),
        np.zeros(c - 1, dtype=dtype),
        np.sort(rng.integers(0, 2000, size=5 * c + 123).astype(dtype)),
    ]
    key = "reduce_by_key:" + ("u32" if dtype == np.uint32 else "u64")
    ctx.tuning_set(key, variant)
    try:
        for keys in cases:
            vals = rng.integers(0, 2**32, size=keys.size, dtype=np.uint64).astype(np.uint32)
            want = orc.std_reduce_by_key(keys, vals)
            for offset in (0, 1):
                got = _rbk_device(gbc, ctx, keys, vals, offset)
                for g, w in zip(got, want):
                    assert np.array_equal(g, w)
    finally:
        ctx.tuning_set(key, 0)


def test_compute_pipeline_sample_flow(ctx, gbc, orc):
    # samples/core/compute-pipeline/main.cpp:94-183 with its default 1,000,000
    # readings, minus the file I/O, bitpack and static_map stages (outside the
    # primitive core): the calibration table lookup stands in as sensor % 7,
    # computed on the host. mt19937(42) raw outputs, four per reading (the
    # reading's two draws taken left to right).
    n = 1_000_000
    r = orc.random_uints(4 * n, 0xFFFFFFFF, 42).astype(np.uint64)
    sensors = (r[1::4] % 1000).astype(np.uint32)
    readings = (150 + r[2::4] % 300 + np.where(r[3::4] % 1000 == 0, 600, 0)).astype(np.uint32)
    offsets = sensors % np.uint32(7)

    d_readings = gbc.DeviceBuffer.from_host(ctx, readings)
    d_offsets = gbc.DeviceBuffer.from_host(ctx, offsets)
    gbc.transform(ctx, d_readings, d_offsets, d_readings, "x + y")  # calibrate in place
    cal = readings + offsets
    hottest = gbc.reduce(ctx, d_readings, gbc.ops.maximum(np.uint32), 0)
    hist = gbc.DeviceBuffer(ctx, 12, np.uint32)
    gbc.histogram_even(ctx, d_readings, hist, 0.0, 1200.0)
    d_alarms = gbc.DeviceBuffer(ctx, n, np.uint32)
    alarms = gbc.copy_if(ctx, d_readings, d_alarms, "x >= 700u")
    d_f = gbc.DeviceBuffer(ctx, n, np.float32)
    gbc.transform(ctx, d_readings, d_f, "x * 0.18f + 32.0f")
    d_order = gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.sequence(ctx, d_order)
    gbc.sort_by_key(ctx, d_readings, d_order, descending=True)
    top = d_order.to_host()

    # the sample's own host checks
    assert hottest == cal.max()
    assert alarms == int((cal >= 700).sum())
    assert np.array_equal(hist.to_host(), np.bincount(cal[cal < 1200] // 100, minlength=12).astype(np.uint32))
    assert cal[top[0]] == cal.max()
    # and every array exactly
    assert np.array_equal(d_alarms.to_host()[:alarms], cal[cal >= 700])
    assert np.array_equal(d_f.to_host(), cal.astype(np.float32) * np.float32(0.18) + np.float32(32.0))
    assert np.array_equal(top, np.argsort(-cal.astype(np.int64), kind="stable").astype(np.uint32))
    assert np.array_equal(d_readings.to_host(), cal[top])
