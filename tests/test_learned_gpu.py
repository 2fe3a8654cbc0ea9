"""Learned-CDF sort on the GPU: the network's gradients against the CPU
oracle, output bit-identical to the plain radix sort, the gain of the trained
network over bucketing without it, the second model level (oversized root
buckets split at sample quantiles), and the fallback to the plain radix sort
for a deliberately bad network."""
import numpy as np
import pytest
from helpers import learned_mixture

pytestmark = pytest.mark.gpu

H = 32


def network_case(rng, m):
    """Random parameters near the data-driven initialisation, so that most
    units sit inside their linear range, and m points."""
    keys = np.sort(rng.integers(0, 1 << 32, m, dtype=np.uint64)).astype(np.uint32)
    q = keys[np.minimum(np.arange(H + 1) * m // H, m - 1)].astype(np.int64)
    centres = (q[:-1] + (q[1:] - q[:-1]) // 2).astype(np.uint32)
    span = float(max(int(keys[-1]) - int(keys[0]), 1))
    width = np.maximum(q[1:] - q[:-1], 1).astype(np.float64)
    p = np.zeros(4 * H + H * H + 1, dtype=np.float32)
    p[0:H] = np.log(span / width) + rng.uniform(-1.0, 0.0, H)            # v1
    p[H:2 * H] = rng.uniform(0.3, 0.7, H)                                 # b1
    p[2 * H:2 * H + H * H] = np.log(rng.uniform(0.01, 0.05, H * H))       # v2
    p[2 * H + H * H:3 * H + H * H] = rng.uniform(-0.4, 0.0, H)            # b2
    p[3 * H + H * H:4 * H + H * H] = np.log(rng.uniform(0.5, 1.5, H) / H)  # v3
    p[-1] = 0.01
    ys = ((np.arange(m) + 0.5) / m).astype(np.float32)
    return p, centres, np.float32(1.0 / span), keys, ys


@pytest.mark.parametrize("m", [3000, 70001])
def test_mlp_gradients_match_oracle(ctx, gbc, orc, m):
    p, c, inv_span, keys, ys = network_case(np.random.default_rng(m), m)
    g_gpu, loss_gpu = gbc.learned_mlp_gradients(ctx, p, c, inv_span, keys, ys)
    g_cpu, loss_cpu = orc.mlp_grad(p, c, inv_span, keys, ys)
    assert np.count_nonzero(g_cpu) > 0.9 * g_cpu.size  # most units are active
    # fp32 on the GPU against double on the host: 1e-3 of the largest entry
    scale = np.max(np.abs(g_cpu))
    assert np.max(np.abs(g_gpu - g_cpu)) <= 1e-3 * scale
    assert abs(loss_gpu - loss_cpu) <= 1e-4 * max(loss_cpu, 1e-6)


def plain_sort(ctx, gbc, keys):
    kin = gbc.DeviceBuffer.from_host(ctx, keys)
    kout = gbc.DeviceBuffer(ctx, keys.size, keys.dtype)
    gbc.sort_raw(ctx, kin.device_pointer, kout.device_pointer, keys.dtype, keys.size)
    return kout.to_host()


def learned(ctx, gbc, keys, **kw):
    kin = gbc.DeviceBuffer.from_host(ctx, keys)
    kout = gbc.DeviceBuffer(ctx, keys.size, keys.dtype)
    st = gbc.sort_learned(ctx, kin.device_pointer, kout.device_pointer, keys.dtype, keys.size,
                          gbc.learned_options(**kw))
    assert np.array_equal(kin.to_host().view(np.uint32), keys.view(np.uint32))  # input untouched
    return kout.to_host(), st


@pytest.mark.parametrize("n", [1 << 22, 3_000_001])
def test_learned_sort_is_bit_identical_to_plain(ctx, gbc, n):
    keys = learned_mixture(n, seed=5)
    keys[:7] = np.array([-0.0, 0.0, np.inf, -np.inf, -0.0, 1e-45, -1e-45], dtype=np.float32)
    out, st = learned(ctx, gbc, keys, steps=32)
    ref = plain_sort(ctx, gbc, keys)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    assert st.violation == 0 and st.fallback == 0
    assert st.last_loss < st.first_loss


@pytest.mark.parametrize("group_threads,bucket_threads", [(256, 1024), (512, 512), (1024, 256)])
def test_partition_levels_at_every_cta_size(ctx, gbc, group_threads, bucket_threads):
    # The two partition levels with 1, 2 or 4 CTAs per SM (1024, 512 or 256
    # threads each, so 8,192, 4,096 or 2,048 keys per chunk): the same output.
    keys = learned_mixture(3_000_001, seed=9)
    ref = plain_sort(ctx, gbc, keys)
    try:
        ctx.tuning_set("learned:group_threads", group_threads)
        ctx.tuning_set("learned:bucket_threads", bucket_threads)
        out, st = learned(ctx, gbc, keys)
    finally:
        ctx.tuning_set("learned:group_threads", 512)
        ctx.tuning_set("learned:bucket_threads", 256)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    assert st.violation == 0 and st.fallback == 0


def test_trained_network_beats_bucketing_without_it(ctx, gbc):
    # Without the network the keys are bucketed by equal-width ranges of the
    # key domain; the mixture's narrow clusters then fill a few buckets far
    # beyond one CTA's shared-memory sort. The fitted CDF spreads them.
    keys = learned_mixture(1 << 22, seed=11)
    opts = dict(buckets=4096, refine=0)  # the root models alone
    out_l, st_l = learned(ctx, gbc, keys, steps=32, **opts)
    out_u, st_u = learned(ctx, gbc, keys, use_model=0, **opts)
    out_0, st_0 = learned(ctx, gbc, keys, steps=0, **opts)  # initialised, not trained
    ref = plain_sort(ctx, gbc, keys).view(np.uint32)
    for out in (out_l, out_u, out_0):
        assert np.array_equal(out.view(np.uint32), ref)
    assert st_l.fallback == 0
    # Without the network most keys would sit in oversized buckets: the sample
    # estimate predicts it and the plain radix sort takes over.
    assert st_u.estimated_oversized_keys > keys.size // 2 and st_u.fallback == 1
    assert st_l.estimated_oversized_keys * 3 < st_u.estimated_oversized_keys
    assert st_l.oversized_keys * 3 < keys.size
    assert st_l.nonempty_buckets > st_l.buckets // 2
    # training lowers the fit error of the initialised network
    assert st_l.last_loss < 0.5 * st_l.first_loss
    assert st_0.first_loss == 0.0 and st_0.fallback == 0


@pytest.mark.parametrize("dtype", [np.uint32, np.int32])
def test_learned_integer_keys_and_small_sizes(ctx, gbc, dtype):
    rng = np.random.default_rng(3)
    for n in (2, 5, 255, 4097, 300000):
        keys = rng.integers(np.iinfo(dtype).min, np.iinfo(dtype).max, size=n, dtype=np.int64).astype(dtype)
        keys[::9] = keys[0]
        out, st = learned(ctx, gbc, keys, sample=min(n, 1 << 16))
        assert np.array_equal(out, np.sort(keys))


def test_learned_constant_and_few_valued_keys(ctx, gbc):
    # a zero-width key range (every key equal), two values, and 5 values
    # with one holding most keys: buckets of one key value everywhere
    i = np.arange(300_001)
    cases = [np.full(100_000, 7.5, dtype=np.float32),
             np.where(i % 3 == 0, -1.0, 2.0).astype(np.float32),
             np.where(i % 10 < 7, 1e3, (i % 10).astype(np.float64)).astype(np.float32)]
    for keys in cases:
        out, st = learned(ctx, gbc, keys)
        assert np.array_equal(out.view(np.uint32), plain_sort(ctx, gbc, keys).view(np.uint32))
        assert st.violation == 0


def test_bad_network_falls_back_to_plain_sort(ctx, gbc):
    # Every weight ~ 0: the network's CDF is flat, every splitter lands past
    # the largest sampled key and all keys would share one bucket; the sample
    # estimate sends the input to the plain radix sort.
    keys = learned_mixture(1 << 20, seed=2)
    bad = np.zeros(gbc.learned_param_count(), dtype=np.float32)
    bad[0:H] = -30.0
    bad[2 * H:2 * H + H * H] = -30.0
    bad[3 * H + H * H:4 * H + H * H] = -30.0
    out, st = learned(ctx, gbc, keys, steps=0, params_in=bad.ctypes.data, refine=0)
    assert st.fallback == 1 and st.estimated_oversized_keys > keys.size // 2
    assert np.array_equal(out.view(np.uint32), plain_sort(ctx, gbc, keys).view(np.uint32))


def test_second_level_splits_oversized_buckets(ctx, gbc):
    # The mixture's narrow clusters fill root buckets far beyond one CTA's
    # shared-memory sort; the second level splits them at the sample's
    # quantiles, which also isolates the clusters' repeated values in buckets
    # of one key value (left unsorted). Output stays bit-identical.
    keys = learned_mixture(1 << 22, seed=11)
    ref = plain_sort(ctx, gbc, keys).view(np.uint32)
    out_0, st_0 = learned(ctx, gbc, keys, steps=0, refine=0)
    out_r, st_r = learned(ctx, gbc, keys, steps=0)
    for out in (out_0, out_r):
        assert np.array_equal(out.view(np.uint32), ref)
    assert st_0.refined_splitters == 0 and st_r.refined_splitters > 0
    assert st_r.refined_splitters <= st_r.buckets // 3
    assert st_r.fallback == 0 and st_r.violation == 0
    sorted_0 = st_0.oversized_keys - st_0.constant_keys  # keys the onesweep path sorts
    sorted_r = st_r.oversized_keys - st_r.constant_keys
    assert sorted_r * 2 < sorted_0


def test_second_level_rescues_a_flat_network_exactly(ctx, gbc):
    # With the root model flat (all keys in one root bucket) the second level
    # alone partitions the keys; the bucketing stays monotone and exact.
    keys = learned_mixture(1 << 20, seed=2)
    bad = np.zeros(gbc.learned_param_count(), dtype=np.float32)
    bad[0:H] = -30.0
    bad[2 * H:2 * H + H * H] = -30.0
    bad[3 * H + H * H:4 * H + H * H] = -30.0
    out, st = learned(ctx, gbc, keys, steps=0, params_in=bad.ctypes.data)
    assert np.array_equal(out.view(np.uint32), plain_sort(ctx, gbc, keys).view(np.uint32))
    assert st.violation == 0 and st.refined_splitters > 0


def ordered_u32(keys):
    k = keys.view(np.uint32)
    return np.where(k >> 31 == 1, ~k, k | np.uint32(0x80000000)).astype(np.uint32)


@pytest.mark.parametrize("reverse", [False, True])
def test_given_splitters_any_order_stays_exact(ctx, gbc, reverse):
    # The bucket of a key is a binary search over the splitters, monotone in
    # the key for any splitter array: even an unsorted one cannot break order.
    keys = learned_mixture(1 << 21, seed=9)
    B = 4096
    u = np.sort(ordered_u32(keys))
    sp = u[(np.arange(1, B) * u.size) // B].astype(np.uint32)
    if reverse:
        sp = sp[::-1].copy()
    out, st = learned(ctx, gbc, keys, buckets=B, splitters_in=sp.ctypes.data)
    assert np.array_equal(out.view(np.uint32), plain_sort(ctx, gbc, keys).view(np.uint32))
    assert st.violation == 0
    if not reverse:
        assert st.fallback == 0 and st.nonempty_buckets > B * 3 // 4


# ---- key-value form (64-bit keys for the sort -> reduce_by_key pipeline) ----

def splitmix64(x):
    with np.errstate(over="ignore"):
        z = x + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def pair_keys(case, n, rng):
    if case == "zipf_splitmix":
        return splitmix64((rng.zipf(1.1, n) % (1 << 24)).astype(np.uint64))
    if case == "raw_ranks":
        return (rng.zipf(1.1, n) % (1 << 24)).astype(np.uint64)
    if case == "uniform_i64":
        return rng.integers(-(1 << 63), (1 << 63) - 1, size=n, dtype=np.int64)
    return rng.integers(0, 1 << 64, size=n, dtype=np.uint64)


def plain_pairs(ctx, gbc, keys, vals):
    kin, vin = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    kout, vout = gbc.DeviceBuffer(ctx, keys.size, keys.dtype), gbc.DeviceBuffer(ctx, keys.size, np.uint32)
    gbc.sort_raw(ctx, kin.device_pointer, kout.device_pointer, keys.dtype, keys.size, vin.device_pointer,
                 vout.device_pointer)
    return kout.to_host(), vout.to_host()


def learned_pairs(ctx, gbc, keys, vals, **kw):
    kin, vin = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    kout, vout = gbc.DeviceBuffer(ctx, max(keys.size, 1), keys.dtype), gbc.DeviceBuffer(ctx, max(keys.size, 1), np.uint32)
    st = gbc.sort_learned_pairs(ctx, kin.device_pointer, kout.device_pointer, keys.dtype, vin.device_pointer,
                                vout.device_pointer, keys.size, gbc.learned_options(**kw))
    return kout.to_host()[: keys.size], vout.to_host()[: keys.size], st


@pytest.mark.parametrize("case", ["zipf_splitmix", "raw_ranks", "uniform_u64", "uniform_i64"])
def test_learned_pairs_64bit_bit_identical_to_plain(ctx, gbc, case):
    # the pipeline's keys: splitmix64 of Zipf(1.1) ranks over 2^24 values, the
    # raw ranks, and uniform 64-bit keys; values uniform in [0, 2^16) so that
    # equal keys check stability
    rng = np.random.default_rng(len(case))
    n = 3_000_001
    keys = pair_keys(case, n, rng)
    vals = rng.integers(0, 1 << 16, size=n, dtype=np.uint32)
    k, v, st = learned_pairs(ctx, gbc, keys, vals)
    rk, rv = plain_pairs(ctx, gbc, keys, vals)
    assert np.array_equal(k, rk) and np.array_equal(v, rv)
    assert st.violation == 0


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32, np.uint64, np.int64])
def test_learned_pairs_key_types_and_small_sizes(ctx, gbc, dtype):
    rng = np.random.default_rng(7)
    for n in (0, 1, 2, 5, 255, 4097, 300_001):
        if np.dtype(dtype).kind == "f":
            keys = learned_mixture(max(n, 1), seed=n)[:n]
        else:
            info = np.iinfo(dtype)
            keys = rng.integers(info.min, info.max, size=n, dtype=dtype, endpoint=True)
            if n:
                keys[::7] = keys[0]  # duplicates: stability
        vals = np.arange(n, dtype=np.uint32)
        k, v, st = learned_pairs(ctx, gbc, keys, vals, sample=min(max(n, 1), 1 << 16))
        rk, rv = plain_pairs(ctx, gbc, keys, vals) if n else (keys, vals)
        assert np.array_equal(k.view(np.uint8), rk.view(np.uint8)) and np.array_equal(v, rv)


def test_learned_pairs_mixture_trains_and_partitions(ctx, gbc):
    keys = learned_mixture(1 << 22, seed=13)
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v, st = learned_pairs(ctx, gbc, keys, vals, steps=32)
    rk, rv = plain_pairs(ctx, gbc, keys, vals)
    assert np.array_equal(k.view(np.uint32), rk.view(np.uint32)) and np.array_equal(v, rv)
    assert st.fallback == 0 and st.violation == 0 and st.last_loss < st.first_loss
    assert st.nonempty_buckets > st.buckets // 2


def test_learned_pairs_bad_network_falls_back(ctx, gbc):
    keys = pair_keys("zipf_splitmix", 1 << 20, np.random.default_rng(2))
    vals = np.arange(keys.size, dtype=np.uint32)
    bad = np.zeros(gbc.learned_param_count(), dtype=np.float32)
    bad[0:H] = -30.0
    bad[2 * H:2 * H + H * H] = -30.0
    bad[3 * H + H * H:4 * H + H * H] = -30.0
    k, v, st = learned_pairs(ctx, gbc, keys, vals, steps=0, params_in=bad.ctypes.data, refine=0)
    rk, rv = plain_pairs(ctx, gbc, keys, vals)
    assert st.fallback == 1
    assert np.array_equal(k, rk) and np.array_equal(v, rv)


def test_learned_pairs_zipf_heads_need_no_sort(ctx, gbc):
    # Zipf(1.1): the most frequent keys fill whole buckets with one key value;
    # those buckets are left as the stable partition leaves them, so the model
    # is used rather than the plain sort
    rng = np.random.default_rng(21)
    keys = pair_keys("zipf_splitmix", 1 << 22, rng)
    vals = rng.integers(0, 1 << 16, size=keys.size, dtype=np.uint32)
    k, v, st = learned_pairs(ctx, gbc, keys, vals)
    rk, rv = plain_pairs(ctx, gbc, keys, vals)
    assert np.array_equal(k, rk) and np.array_equal(v, rv)
    assert st.fallback == 0 and st.violation == 0
    assert st.constant_keys > keys.size // 10  # the heads (14% of the keys at this seed)
