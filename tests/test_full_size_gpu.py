"""The configurations at their full sizes, through the library's public calls,
checked bit for bit against the oracle (the restated reference algorithms on
every host thread): the 2^28 uniform key-value and keys-only sorts, the
key-value sort of keys that are the AND of 4 uniform words (its lowest
entropy), 2^27 64-bit key-value pairs, the exclusive scan of 2^30 int32 with
its exact int64 total, the 256-bin histogram of 2^30 bytes, the learned-CDF
sort of 2^26 mixture floats, and bitpack compression of 2^28 timestamps
(words equal to the oracle's, and the round trip). Inputs are seeded."""
import numpy as np
import pytest
from helpers import learned_mixture

pytestmark = pytest.mark.gpu


def _kv_sort_against_oracle(gbc, ctx, orc, keys):
    vals = np.arange(keys.size, dtype=np.uint32)
    kb, vb = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    if keys.dtype.itemsize == 4:
        gbc.sort_by_key(ctx, kb, vb)
    else:
        gbc.sort_ex(ctx, kb, vb)
    rk, rv = orc.ref_radix_sort(keys, vals)
    assert np.array_equal(kb.to_host(), rk)
    assert np.array_equal(vb.to_host(), rv)


def test_kv_sort_2e28_uniform(gbc, ctx, orc):
    keys = np.random.default_rng(1).integers(0, 2**32, size=1 << 28, dtype=np.uint32)
    _kv_sort_against_oracle(gbc, ctx, orc, keys)


def test_keys_sort_2e28_uniform(gbc, ctx, orc):
    # keys only: the tile-offset form of the digit pass, the default at this size
    keys = np.random.default_rng(4).integers(0, 2**32, size=1 << 28, dtype=np.uint32)
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    gbc.sort(ctx, kb)
    orc.ref_radix_sort_inplace(keys)
    assert np.array_equal(kb.to_host(), keys)


def test_kv_sort_2e28_and_of_4_words(gbc, ctx, orc):
    rng = np.random.default_rng(2)
    keys = rng.integers(0, 2**32, size=1 << 28, dtype=np.uint32)
    for _ in range(3):
        keys &= rng.integers(0, 2**32, size=keys.size, dtype=np.uint32)
    _kv_sort_against_oracle(gbc, ctx, orc, keys)


def test_kv_sort_2e27_u64_keys(gbc, ctx, orc):
    keys = np.random.default_rng(3).integers(0, 2**64, size=1 << 27, dtype=np.uint64)
    _kv_sort_against_oracle(gbc, ctx, orc, keys)


def test_exclusive_scan_2e30_with_total(gbc, ctx, orc):
    x = np.random.default_rng(4).integers(-1000, 1001, size=1 << 30, dtype=np.int32)
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    yb = gbc.DeviceBuffer(ctx, x.size, np.int32)
    total = gbc.exclusive_scan(ctx, xb, yb, total=True)
    assert int(total) == int(x.sum(dtype=np.int64))
    assert np.array_equal(yb.to_host(), orc.ref_scan(x, exclusive=True))


def test_histogram_2e30_bytes(gbc, ctx, orc):
    u8 = np.random.default_rng(5).integers(0, 256, size=1 << 30, dtype=np.uint8)
    ub = gbc.DeviceBuffer.from_host(ctx, u8)
    hb = gbc.DeviceBuffer(ctx, 256, np.uint32)
    gbc.histogram_even(ctx, ub, hb, 0.0, 256.0)
    assert np.array_equal(hb.to_host(), orc.histogram_even(u8, 256, 0.0, 256.0))


def test_learned_sort_2e26_mixture(gbc, ctx, orc):
    keys = learned_mixture(1 << 26, seed=6)
    kin = gbc.DeviceBuffer.from_host(ctx, keys)
    kout = gbc.DeviceBuffer(ctx, keys.size, np.float32)
    st = gbc.sort_learned(ctx, kin.device_pointer, kout.device_pointer, np.float32, keys.size)
    ref, _ = orc.ref_radix_sort(keys)
    assert np.array_equal(kout.to_host().view(np.uint32), ref.view(np.uint32))
    assert st.violation == 0 and st.fallback == 0


def test_bitpack_2e28_timestamps(gbc, ctx, orc):
    rng = np.random.default_rng(7)
    n = 1 << 28
    ts = ((1700000000 + np.cumsum(rng.integers(0, 50, size=n, dtype=np.uint64))) & 0xFFFFFFFF).astype(np.uint32)
    inb = gbc.DeviceBuffer.from_host(ctx, ts)
    comp = gbc.compress_bitpack(ctx, inb, delta=True, chunk_size=2048)
    assert np.array_equal(comp.data.to_host(), orc.bitpack_compress(ts, 2048, True))
    out = gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.decompress_bitpack(ctx, comp, out)
    assert np.array_equal(out.to_host(), ts)
