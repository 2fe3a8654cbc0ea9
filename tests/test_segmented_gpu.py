"""Batched segmented sort and scan on the GPU against the std:: oracle (per
segment std::stable_sort, restarted sequential scans), bit for bit, and their
CUDA-graph capture and replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def offsets_from_lengths(lens):
    off = np.zeros(len(lens) + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    return off.astype(np.uint32)


LAYOUTS = {
    # tiny, small (warp), medium (CTA) and large (batched onesweep) segments mixed
    "lognormal": lambda orc: orc.lognormal_segments(3000, 256, 2.0, 1, 1 << 17, seed=4),
    "empty_and_single": lambda orc: offsets_from_lengths([0, 1, 0, 0, 2, 1, 0, 33, 0, 1]),
    "one_large": lambda orc: offsets_from_lengths([300001]),
    "cta_boundaries": lambda orc: offsets_from_lengths([256, 257, 6144, 6145, 8192, 8193, 255, 1]),
}


@pytest.mark.parametrize("layout", list(LAYOUTS))
@pytest.mark.parametrize("key_dtype", [np.uint64, np.uint32, np.int32, np.float64])
@pytest.mark.parametrize("with_values", [True, False])
def test_segmented_sort(ctx, gbc, orc, layout, key_dtype, with_values):
    off = LAYOUTS[layout](orc)
    n = int(off[-1])
    rng = np.random.default_rng(5)
    raw = rng.integers(0, 2**63, size=n, dtype=np.uint64)
    raw[::7] = raw[0]  # duplicates inside segments exercise stability
    keys = raw.astype(key_dtype) if np.dtype(key_dtype).kind != "f" else raw.view(np.float64).astype(key_dtype)
    if np.dtype(key_dtype).kind == "f":
        keys = rng.standard_normal(n).astype(key_dtype)
        keys[::11] = -0.0
        keys[1::13] = 0.0
    vals = np.arange(n, dtype=np.uint32)
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    vb = gbc.DeviceBuffer.from_host(ctx, vals) if with_values else None
    ob = gbc.DeviceBuffer.from_host(ctx, off)
    gbc.segmented_sort(ctx, kb, ob, vb)
    ek, ev = orc.std_segmented_sort(keys, off, vals if with_values else None)
    assert np.array_equal(kb.to_host().view(np.uint8), ek.view(np.uint8))
    if with_values:
        assert np.array_equal(vb.to_host(), ev)


@pytest.mark.parametrize("threads", [256, 512])
@pytest.mark.parametrize("key_dtype,with_values", [(np.uint64, True), (np.uint32, False), (np.uint32, True)])
def test_one_cta_sort_thread_counts(ctx, gbc, orc, threads, key_dtype, with_values):
    # The one-CTA segment sorts at 256 threads and at 512 (taken wherever the
    # capacity's shared memory fits, else 256), at two capacities: the
    # type's largest and 2,048 keys.
    off = offsets_from_lengths([256, 257, 700, 2047, 2048, 2049, 5000, 8191, 8192, 10240, 16384, 3, 1])
    n = int(off[-1])
    rng = np.random.default_rng(threads)
    keys = rng.integers(0, 2**63, size=n, dtype=np.uint64).astype(key_dtype)
    keys[::5] = keys[0]
    vals = np.arange(n, dtype=np.uint32)
    ek, ev = orc.std_segmented_sort(keys, off, vals if with_values else None)
    ob = gbc.DeviceBuffer.from_host(ctx, off)
    tag = "u64" if np.dtype(key_dtype).itemsize == 8 else "u32"
    key = f"segsort:{tag}{'kv' if with_values else 'k'}:{_size_class(n)}:avg{_size_class(n // (off.size - 1))}"
    try:
        ctx.tuning_set("segsort:cta_threads", threads)
        for cap in (0, 2048):  # 0: the type's largest capacity
            ctx.tuning_set(key, cap)
            kb = gbc.DeviceBuffer.from_host(ctx, keys)
            vb = gbc.DeviceBuffer.from_host(ctx, vals) if with_values else None
            gbc.segmented_sort(ctx, kb, ob, vb)
            assert np.array_equal(kb.to_host(), ek), (threads, cap)
            if with_values:
                assert np.array_equal(vb.to_host(), ev), (threads, cap)
    finally:
        ctx.tuning_set("segsort:cta_threads", 0)
        ctx.tuning_set(key, 0)


def test_segmented_sort_out_of_place_descending(ctx, gbc, orc):
    off = orc.lognormal_segments(2000, 128, 2.0, 1, 1 << 16, seed=8)
    n = int(off[-1])
    rng = np.random.default_rng(9)
    keys = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32) & np.uint32(0xFFFF)
    vals = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    kin, vin = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    kout, vout = gbc.DeviceBuffer(ctx, n, np.uint32), gbc.DeviceBuffer(ctx, n, np.uint32)
    ob = gbc.DeviceBuffer.from_host(ctx, off)
    gbc.segmented_sort_raw(ctx, kin.device_pointer, kout.device_pointer, np.uint32, n, ob.device_pointer,
                           off.size - 1, vin.device_pointer, vout.device_pointer, descending=True)
    ek, ev = orc.std_segmented_sort(keys, off, vals, descending=True)
    assert np.array_equal(kout.to_host(), ek) and np.array_equal(vout.to_host(), ev)
    assert np.array_equal(kin.to_host(), keys)


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.uint32])
@pytest.mark.parametrize("exclusive", [False, True])
@pytest.mark.parametrize("opname", ["plus", "maximum", "right"])
def test_segmented_scan(ctx, gbc, orc, dtype, exclusive, opname):
    off = orc.lognormal_segments(5000, 64, 2.0, 0, 1 << 15, seed=3)
    n = int(off[-1])
    rng = np.random.default_rng(6)
    x = rng.integers(-1000, 1001, size=n, dtype=np.int64).astype(dtype)
    if opname == "plus":
        op, code, ident = gbc.ops.plus(), orc.OP_PLUS, 0
    elif opname == "maximum":
        op, code, ident = gbc.ops.maximum(dtype), orc.OP_MAX, np.iinfo(dtype).min
    else:
        op, code, ident = gbc.binary_op("b", "0"), orc.OP_RIGHT, 0
    xb, yb, ob = gbc.DeviceBuffer.from_host(ctx, x), gbc.DeviceBuffer(ctx, n, dtype), gbc.DeviceBuffer.from_host(ctx, off)
    gbc.segmented_scan(ctx, xb, yb, ob, op, exclusive)
    assert np.array_equal(yb.to_host(), orc.std_segmented_scan(x, off, code, ident, exclusive))


def test_graph_capture_replays_segmented_sort_and_scan(ctx, gbc, orc):
    off = orc.lognormal_segments(4000, 256, 2.0, 1, 1 << 17, seed=12)
    n = int(off[-1])
    rng = np.random.default_rng(13)
    keys = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    vals = np.arange(n, dtype=np.uint32)
    x = rng.integers(-1000, 1001, size=n, dtype=np.int64).astype(np.int32)
    kin, vin = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    kout, vout = gbc.DeviceBuffer(ctx, n, np.uint64), gbc.DeviceBuffer(ctx, n, np.uint32)
    xb, yb = gbc.DeviceBuffer.from_host(ctx, x), gbc.DeviceBuffer(ctx, n, np.int32)
    ob = gbc.DeviceBuffer.from_host(ctx, off)

    def batch():
        gbc.segmented_sort_raw(ctx, kin.device_pointer, kout.device_pointer, np.uint64, n, ob.device_pointer,
                               off.size - 1, vin.device_pointer, vout.device_pointer)
        gbc.segmented_scan_raw(ctx, xb.device_pointer, yb.device_pointer, n, np.int32, ob.device_pointer,
                               off.size - 1, exclusive=True)

    batch()  # warms the pool: capture needs every temporary cached
    ctx.finish()
    g = gbc.capture(ctx, batch)
    ek, ev = orc.std_segmented_sort(keys, off, vals)
    ey = orc.std_segmented_scan(x, off, orc.OP_PLUS, 0, True)
    for _ in range(2):
        gbc.fill(ctx, kout, 0)
        gbc.fill(ctx, yb, 0)
        g.launch()
        assert np.array_equal(kout.to_host(), ek)
        assert np.array_equal(vout.to_host(), ev)
        assert np.array_equal(yb.to_host(), ey)
    g.release()
    # the plain sort is graph-capturable too
    k2 = gbc.DeviceBuffer.from_host(ctx, keys[:100000].astype(np.uint64))
    k2o = gbc.DeviceBuffer(ctx, 100000, np.uint64)
    f = lambda: gbc.sort_raw(ctx, k2.device_pointer, k2o.device_pointer, np.uint64, 100000)
    f()
    ctx.finish()
    g2 = gbc.capture(ctx, f)
    for _ in range(2):
        g2.launch()
        assert np.array_equal(k2o.to_host(), np.sort(keys[:100000]))
    g2.release()


@pytest.mark.parametrize("key_dtype", [np.uint64, np.uint32, np.float32])
@pytest.mark.parametrize("with_values", [True, False])
def test_msd_and_lsd_routes_mixed(ctx, gbc, orc, key_dtype, with_values):
    """Large segments go one of two ways: when the highest digit position
    that varies inside the segment splits it into buckets that one CTA can
    sort, one pass on that digit and a shared-memory sort per bucket (the MSD
    route); otherwise every digit pass (the LSD route). One call mixes both,
    plus segments whose varying digits lie low (small key ranges), a segment
    of equal keys and small segments, and checks the result bit for bit."""
    rng = np.random.default_rng(31)
    lens = [200000, 150000, 90000, 60000, 40000, 5000, 300, 17, 70000, 120000]
    off = offsets_from_lengths(lens)
    n = int(off[-1])
    bits = 64 if np.dtype(key_dtype).itemsize == 8 else 32
    keys = rng.integers(0, 2**63, size=n, dtype=np.uint64)
    if bits == 32:
        keys &= np.uint64(0xFFFFFFFF)
    b = [int(x) for x in off]
    # segment 1: one dominant value of the top digit (a bucket of ~90% -> LSD)
    seg = slice(b[1], b[2])
    keys[seg] = np.where(rng.random(lens[1]) < 0.9, keys[seg] & np.uint64((1 << (bits - 8)) - 1), keys[seg])
    # segment 2: keys below 2^20 (the top varying digit is low; buckets fit -> MSD there)
    keys[b[2]:b[3]] &= np.uint64((1 << 20) - 1)
    # segment 3: all keys equal (no digit varies -> LSD, every pass a copy)
    keys[b[3]:b[4]] = keys[b[3]]
    # segment 4: duplicates inside buckets (stability)
    keys[b[4]:b[5]:3] = keys[b[4]]
    # segment 9: two values only
    keys[b[9]:b[10]] = np.where(rng.random(lens[9]) < 0.5, 5, 7).astype(np.uint64)
    if np.dtype(key_dtype).kind == "f":
        k = rng.standard_normal(n).astype(np.float32)
        k[b[3]:b[4]] = 1.5
        k[b[1]:b[2]] = np.where(rng.random(lens[1]) < 0.9, np.float32(2.0) + k[b[1]:b[2]] * 1e-6, k[b[1]:b[2]])
        k[::97] = -0.0
        keys = k
    else:
        keys = keys.astype(key_dtype)
    vals = np.arange(n, dtype=np.uint32)
    for descending in (False, True):
        kb = gbc.DeviceBuffer.from_host(ctx, keys)
        vb = gbc.DeviceBuffer.from_host(ctx, vals) if with_values else None
        ob = gbc.DeviceBuffer.from_host(ctx, off)
        gbc.segmented_sort(ctx, kb, ob, vb, descending=descending)
        ek, ev = orc.std_segmented_sort(keys, off, vals if with_values else None, descending=descending)
        assert np.array_equal(kb.to_host().view(np.uint8), ek.view(np.uint8))
        if with_values:
            assert np.array_equal(vb.to_host(), ev)


def _size_class(v):
    k = 0
    while (1 << k) < v and k < 63:
        k += 1
    return f"2^{k}"


@pytest.mark.parametrize("form", [1, 3])
@pytest.mark.parametrize("key_dtype,with_values", [(np.uint64, True), (np.uint32, False), (np.float32, True)])
def test_one_persistent_launch(ctx, gbc, orc, form, key_dtype, with_values):
    """The whole batch in one cooperative launch (form 1: every CTA takes the
    small and the large segments in turn; form 3: a quarter of the CTAs sort
    the small and medium segments while the rest take the large ones),
    selected through the tuning table, directly and replayed from a CUDA
    graph: bit for bit the per-segment std::stable_sort."""
    off = orc.lognormal_segments(4000, 256, 2.0, 1, 1 << 17, seed=12)
    n = int(off[-1])
    rng = np.random.default_rng(13)
    if np.dtype(key_dtype).kind == "f":
        keys = rng.standard_normal(n).astype(key_dtype)
        keys[::17] = -0.0
    else:
        keys = rng.integers(0, 2**63, size=n, dtype=np.uint64).astype(key_dtype)
        keys[::9] = keys[0]
    vals = np.arange(n, dtype=np.uint32)
    tag = {np.dtype(np.uint64): "u64", np.dtype(np.uint32): "u32", np.dtype(np.float32): "u32"}[np.dtype(key_dtype)]
    key = f"segsort:{tag}{'kv' if with_values else 'k'}:{_size_class(n)}:avg{_size_class(n // (off.size - 1))}"
    ctx.tuning_set(key, 2048)
    ctx.tuning_set(key + ":batch", form)
    try:
        ek, ev = orc.std_segmented_sort(keys, off, vals if with_values else None)
        ob = gbc.DeviceBuffer.from_host(ctx, off)
        kin = gbc.DeviceBuffer.from_host(ctx, keys)
        vin = gbc.DeviceBuffer.from_host(ctx, vals)
        kout = gbc.DeviceBuffer(ctx, n, key_dtype)
        vout = gbc.DeviceBuffer(ctx, n, np.uint32)

        def call():
            gbc.segmented_sort_raw(ctx, kin.device_pointer, kout.device_pointer, key_dtype, n, ob.device_pointer,
                                   off.size - 1, vin.device_pointer if with_values else 0,
                                   vout.device_pointer if with_values else 0)

        call()
        assert np.array_equal(kout.to_host().view(np.uint8), ek.view(np.uint8))
        if with_values:
            assert np.array_equal(vout.to_host(), ev)
        # replayed from a graph, after the outputs are overwritten
        graph = gbc.capture(ctx, call)
        gbc.fill(ctx, kout, np.zeros(1, dtype=key_dtype)[0])
        graph.launch()
        ctx.finish()
        graph.release()
        assert np.array_equal(kout.to_host().view(np.uint8), ek.view(np.uint8))
        if with_values:
            assert np.array_equal(vout.to_host(), ev)
    finally:
        ctx.tuning_set(key + ":batch", 0)
