"""The autotuner: every candidate runs, the fastest is stored under the
workload's tuning key, and the data it leaves behind is correctly sorted."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,with_values", [(np.uint32, False), (np.uint32, True), (np.uint64, True)])
def test_autotune_sort_stores_the_fastest_variant(ctx, gbc, dtype, with_values):
    rng = np.random.default_rng(7)
    n = (1 << 20) + 3
    keys = rng.integers(0, np.iinfo(dtype).max, size=n, dtype=dtype)
    kin, kout = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer(ctx, n, dtype)
    vin = gbc.DeviceBuffer.from_host(ctx, np.arange(n, dtype=np.uint32)) if with_values else None
    vout = gbc.DeviceBuffer(ctx, n, np.uint32) if with_values else None
    best, ms = gbc.autotune_sort(ctx, kin.device_pointer, kout.device_pointer, dtype, n,
                                 vin.device_pointer if vin else 0, vout.device_pointer if vout else 0, repetitions=2)
    kb = np.dtype(dtype).itemsize
    assert 0 <= best < gbc.tuning_sort_variants(kb, with_values) and ms > 0
    assert ctx.tuning_get(gbc.tuning_sort_key(kb, with_values, n)) == best
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(kout.to_host(), keys[order])
    if with_values:
        assert np.array_equal(vout.to_host(), order.astype(np.uint32))


def test_autotune_segmented_sort_stores_a_capacity(ctx, gbc, orc):
    off = orc.lognormal_segments(3000, 256, 2.0, 1, 1 << 16, seed=3)
    n = int(off[-1])
    rng = np.random.default_rng(8)
    keys = rng.integers(0, np.iinfo(np.uint64).max, size=n, dtype=np.uint64)
    vals = rng.integers(0, 1 << 30, size=n, dtype=np.uint32)
    kin, kout = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer(ctx, n, np.uint64)
    vin, vout = gbc.DeviceBuffer.from_host(ctx, vals), gbc.DeviceBuffer(ctx, n, np.uint32)
    offd = gbc.DeviceBuffer.from_host(ctx, off.astype(np.uint32))
    cap, ms = gbc.autotune_segmented_sort(ctx, kin.device_pointer, kout.device_pointer, np.uint64, n,
                                          offd.device_pointer, off.size - 1, vin.device_pointer, vout.device_pointer,
                                          repetitions=2)
    assert 1024 <= cap and ms > 0
    rk, rv = orc.std_segmented_sort(keys, off, vals)
    assert np.array_equal(kout.to_host(), rk) and np.array_equal(vout.to_host(), rv)
    # every stage stored its choice under the workload's key
    k = 0
    while (1 << k) < n:
        k += 1
    a = 0
    while (1 << a) < n // (off.size - 1):
        a += 1
    key = f"segsort:u64kv:2^{k}:avg2^{a}"
    assert ctx.tuning_get(key) == cap
    assert ctx.tuning_get(key + ":threads") in (256, 512)
    assert ctx.tuning_get(key + ":batch") in range(0, 5)
    for suffix in ("", ":msd", ":threads", ":batch"):
        ctx.tuning_set(key + suffix, 0)


def test_autotune_rejects_in_place(ctx, gbc):
    buf = gbc.DeviceBuffer.from_host(ctx, np.arange(100, dtype=np.uint32))
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.autotune_sort(ctx, buf.device_pointer, buf.device_pointer, np.uint32, 100)
