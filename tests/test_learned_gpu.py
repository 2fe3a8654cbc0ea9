"""Learned-CDF sort on the GPU: the network's gradients against the CPU
oracle, output bit-identical to the plain radix sort, the gain of the trained
network over bucketing without it, and the fallback on a monotonicity
violation."""
import numpy as np
import pytest
from helpers import learned_mixture

pytestmark = pytest.mark.gpu


def test_mlp_gradients_match_oracle(ctx, gbc, orc):
    rng = np.random.default_rng(1)
    npar = gbc.learned_param_count()
    params = rng.uniform(0.05, 0.6, npar).astype(np.float32)
    params[32:64] = rng.uniform(-1, 0, 32)  # b1: ramps inside [0, 1]
    xs = rng.uniform(0, 1, 3000).astype(np.float32)
    ys = np.sort(rng.uniform(0, 1, 3000)).astype(np.float32)
    g_gpu, loss_gpu = gbc.learned_mlp_gradients(ctx, params, xs, ys)
    g_cpu, loss_cpu = orc.mlp_grad(params, xs, ys)
    # fp32 on the GPU against double on the host: relative 1e-3 of the largest
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
    out, st = learned(ctx, gbc, keys)
    ref = plain_sort(ctx, gbc, keys)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    assert st.violation == 0 and st.fallback == 0
    assert st.last_loss < st.first_loss


def test_trained_network_beats_bucketing_without_it(ctx, gbc):
    # The method without the network buckets by the normalised key alone; the
    # fitted CDF spreads the mixture's keys far more evenly, so fewer keys
    # land in buckets too large for one CTA's shared-memory sort.
    keys = learned_mixture(1 << 22, seed=11)
    opts = dict(buckets=4096, grid=4096)
    out_l, st_l = learned(ctx, gbc, keys, **opts)
    out_u, st_u = learned(ctx, gbc, keys, use_model=0, **opts)
    assert np.array_equal(out_l.view(np.uint32), out_u.view(np.uint32))
    assert st_l.largest_bucket < st_u.largest_bucket
    assert st_l.oversized_keys < st_u.oversized_keys
    assert st_l.nonempty_buckets > st_u.nonempty_buckets


@pytest.mark.parametrize("dtype", [np.uint32, np.int32])
def test_learned_integer_keys_and_small_sizes(ctx, gbc, dtype):
    rng = np.random.default_rng(3)
    for n in (2, 5, 4097, 300000):
        keys = rng.integers(np.iinfo(dtype).min, np.iinfo(dtype).max, size=n, dtype=np.int64).astype(dtype)
        keys[::9] = keys[0]
        out, st = learned(ctx, gbc, keys, sample=min(n, 1 << 16))
        assert np.array_equal(out, np.sort(keys))


def test_monotonicity_violation_falls_back(ctx, gbc):
    keys = learned_mixture(1 << 20, seed=2)
    grid = 1024
    bad = np.linspace(1.0, 0.0, grid + 1).astype(np.float32)  # a decreasing CDF
    out, st = learned(ctx, gbc, keys, grid=grid, table_in=bad.ctypes.data)
    assert st.violation == 1 and st.fallback == 1
    assert np.array_equal(out.view(np.uint32), plain_sort(ctx, gbc, keys).view(np.uint32))
