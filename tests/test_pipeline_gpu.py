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
