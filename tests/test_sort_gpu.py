"""Radix sort parity on the GPU, through the C ABI: the reference's test
recipes (lib/test/Compute/main.cpp:246-312) against the golden fixtures and
the CPU oracle, bit for bit, plus 64-bit keys, pass skipping, out-of-place
sorts and full-size properties."""
import numpy as np
import pytest
from helpers import GOLDEN, SIZES, digest, ordered_u32

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", SIZES)
def test_sort_by_key_reference_recipe(ctx, gbc, orc, n):
    keys = orc.random_uints(n, 0xFFFFFFFF, n + 2)
    assert digest(keys) == GOLDEN["sort_by_key"][str(n)]["keys_in"]
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    vb = gbc.DeviceBuffer.from_host(ctx, np.arange(n, dtype=np.uint32))
    gbc.sort_by_key(ctx, kb, vb)
    k, v = kb.to_host(), vb.to_host()
    assert digest(k) == GOLDEN["sort_by_key"][str(n)]["keys"]
    assert digest(v) == GOLDEN["sort_by_key"][str(n)]["values"]


@pytest.mark.parametrize("n", [2, 31, 4095, 4096, 4097, 12289, 100003])
def test_keys_only_matches_oracle(ctx, gbc, orc, n):
    keys = orc.random_uints(n, 0xFFFFFFFF, 1000 + n)
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    gbc.sort(ctx, kb)
    assert np.array_equal(kb.to_host(), orc.std_sort(keys)[0])


def test_stability_many_duplicates(ctx, gbc, orc):
    dup = orc.random_uints(50000, 15, 99)
    kb = gbc.DeviceBuffer.from_host(ctx, dup)
    vb = gbc.DeviceBuffer.from_host(ctx, np.arange(dup.size, dtype=np.uint32))
    gbc.sort_by_key(ctx, kb, vb)
    assert digest(kb.to_host()) == GOLDEN["stability"]["keys"]
    assert digest(vb.to_host()) == GOLDEN["stability"]["values"]


def test_signed_keys(ctx, gbc):
    ints = np.array(GOLDEN["signed"]["keys_in"], dtype=np.int32)
    ib = gbc.DeviceBuffer.from_host(ctx, ints)
    gbc.sort(ctx, ib)
    assert ib.to_host().tolist() == GOLDEN["signed"]["sorted"]


def test_float_keys_descending_bit_exact(ctx, gbc, orc):
    f = orc.random_floats(3000, -1e6, 1e6, 5)
    f[0], f[1], f[2] = np.float32(-0.0), np.float32(np.inf), np.float32(-np.inf)
    assert digest(f) == GOLDEN["floats_desc"]["keys_in"]  # same generator output on every host
    fb = gbc.DeviceBuffer.from_host(ctx, f)
    gbc.sort(ctx, fb, True)
    got = fb.to_host()
    assert digest(got.view(np.uint32)) == GOLDEN["floats_desc"]["sorted_bits"]
    assert np.array_equal(got, np.sort(f)[::-1])


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32])
@pytest.mark.parametrize("descending", [False, True])
def test_pairs_all_key_types(ctx, gbc, orc, dtype, descending):
    rng = np.random.default_rng(11)
    n = 70001
    raw = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    raw[::5] = raw[7]  # duplicates exercise stability
    if dtype == np.float32:
        raw[::97] = 0x80000000  # -0.0
        raw[1::97] = 0x00000000  # +0.0
        raw[2::991] = 0x7FC00000  # a NaN pattern sorts by its bits
    keys = raw.view(dtype)
    vals = np.arange(n, dtype=np.uint32)
    kb, vb = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    gbc.sort_by_key(ctx, kb, vb, descending)
    ek, ev = orc.std_sort(keys, vals, descending)
    assert np.array_equal(kb.to_host().view(np.uint32), ek.view(np.uint32))
    assert np.array_equal(vb.to_host(), ev)
    order = np.argsort(ordered_u32(keys, descending), kind="stable")
    assert np.array_equal(ev, vals[order])


@pytest.mark.parametrize("dtype", [np.uint64, np.int64, np.float64])
@pytest.mark.parametrize("with_values", [False, True])
def test_64bit_keys(ctx, gbc, orc, dtype, with_values):
    rng = np.random.default_rng(12)
    n = 50003
    raw = rng.integers(0, 2**64, size=n, dtype=np.uint64)
    raw[::3] = raw[5]
    keys = raw.view(dtype)
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    vals = np.arange(n, dtype=np.uint32)
    vb = gbc.DeviceBuffer.from_host(ctx, vals) if with_values else None
    gbc.sort_ex(ctx, kb, vb)
    ek, ev = orc.std_sort(keys, vals if with_values else None)
    assert np.array_equal(kb.to_host().view(np.uint64), ek.view(np.uint64))
    if with_values:
        assert np.array_equal(vb.to_host(), ev)


@pytest.mark.parametrize("mask", [0x000000FF, 0x0000FF00, 0x00FF00FF, 0xFF000000, 0x0])
@pytest.mark.parametrize("with_values", [False, True])
def test_pass_skipping(ctx, gbc, orc, mask, with_values):
    # Digit positions on which all keys agree are skipped on the device; an odd
    # number of remaining passes takes the copy path of the in-place sort.
    rng = np.random.default_rng(mask)
    n = 30011
    keys = (rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32) & np.uint32(mask)) | np.uint32(
        0x12345678 & ~mask)
    vals = np.arange(n, dtype=np.uint32)
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    vb = gbc.DeviceBuffer.from_host(ctx, vals) if with_values else None
    if with_values:
        gbc.sort_by_key(ctx, kb, vb)
    else:
        gbc.sort(ctx, kb)
    ek, ev = orc.std_sort(keys, vals)
    assert np.array_equal(kb.to_host(), ek)
    if with_values:
        assert np.array_equal(vb.to_host(), ev)


@pytest.mark.parametrize("mask", [0x000000FF, 0x00FFFFFF, 0xFFFFFFFF, 0x0])
def test_out_of_place_keeps_input(ctx, gbc, orc, mask):
    rng = np.random.default_rng(3)
    n = 40000
    keys = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32) & np.uint32(mask)
    vals = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    kin, vin = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    kout, vout = gbc.DeviceBuffer(ctx, n, np.uint32), gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.sort_raw(ctx, kin.device_pointer, kout.device_pointer, np.uint32, n, vin.device_pointer, vout.device_pointer)
    ek, ev = orc.std_sort(keys, vals)
    assert np.array_equal(kout.to_host(), ek) and np.array_equal(vout.to_host(), ev)
    assert np.array_equal(kin.to_host(), keys) and np.array_equal(vin.to_host(), vals)


@pytest.mark.parametrize("k", [0, 1, 2, 4])
def test_entropy_and_keys(ctx, gbc, orc, k):
    # keys = AND of k uniform words (k = 0: the empty AND, all ones)
    rng = np.random.default_rng(100 + k)
    n = 1 << 20
    keys = np.full(n, 0xFFFFFFFF, dtype=np.uint32)
    for _ in range(k):
        keys &= rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    kb, vb = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    gbc.sort_by_key(ctx, kb, vb)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(kb.to_host(), keys[order])
    assert np.array_equal(vb.to_host(), order.astype(np.uint32))


def test_full_size_properties(ctx, gbc):
    # 2^24 uniform keys (the reference's CPU-runnable configuration): sorted,
    # a permutation of the input, stable.
    rng = np.random.default_rng(1)
    n = 1 << 24
    keys = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    kb, vb = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)
    gbc.sort_by_key(ctx, kb, vb)
    k, v = kb.to_host(), vb.to_host()
    assert np.all(k[1:] >= k[:-1])
    assert np.array_equal(keys[v], k)
    assert np.array_equal(np.sort(v), vals)
    same = k[1:] == k[:-1]
    assert np.all(v[1:][same] > v[:-1][same])


def test_repeated_calls_and_memory_reuse(ctx, gbc, orc):
    keys = orc.random_uints(300000, 0xFFFFFFFF, 42)
    exp = orc.std_sort(keys)[0]
    before = ctx.memory_stats().total_allocations
    for _ in range(3):
        kb = gbc.DeviceBuffer.from_host(ctx, keys)
        gbc.sort(ctx, kb)
        assert np.array_equal(kb.to_host(), exp)
        kb.release()
    s = ctx.memory_stats()
    assert s.current_allocations == 0
    assert s.total_allocations > before


# The tile-offset variants of the 32-bit keys-only list (PAD 1, PAD 0): every
# tile's output offsets are counted before the pass instead of looked back.
TILE_OFFSET_VARIANTS = (11, 12)


@pytest.mark.parametrize("dtype", [np.uint32, np.int32, np.float32])
@pytest.mark.parametrize("descending", [False, True])
def test_tile_offset_form_multi_tile_chunks(ctx, gbc, orc, dtype, descending):
    # The tile-offset form (the default for keys without values from 2^27
    # keys) forced at 5,000,003 keys: 814 tiles in chunks of 3, so the chunk
    # scan carries offsets across chunks, the last chunk holds one tile and
    # the last tile is partial; every 32-bit key transform, both directions,
    # and one case whose constant top byte leaves an odd number of passes.
    assert gbc.tuning_sort_variants(4, False) == 13
    n = 5_000_003
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    cases = [bits, (bits & np.uint32(0x00FFFFFF)) | np.uint32(0x3F000000)]
    key = gbc.tuning_sort_key(4, False, n)
    try:
        for var in TILE_OFFSET_VARIANTS:
            ctx.tuning_set(key, var)
            for raw in cases:
                keys = raw.view(dtype)
                exp = orc.ref_radix_sort(keys, None, descending)[0]
                kb = gbc.DeviceBuffer.from_host(ctx, keys)
                gbc.sort(ctx, kb, descending)
                assert np.array_equal(kb.to_host().view(np.uint32), exp.view(np.uint32)), (var, dtype, descending)
    finally:
        ctx.tuning_set(key, 0)


@pytest.mark.parametrize("key_dtype", [np.uint32, np.uint64])
@pytest.mark.parametrize("with_values", [False, True])
def test_every_compiled_variant(ctx, gbc, orc, key_dtype, with_values):
    # Each launch shape the tuning table can select (plain loads, bulk-copy
    # staging, match or ballot ranking) sorts identically, including partial
    # last tiles and arrays whose address rules out bulk copies.
    kb_ = np.dtype(key_dtype).itemsize
    rng = np.random.default_rng(21)
    for n in (1, 3, 4096, 4097, 12288 * 3 + 5, 200003):
        raw = rng.integers(0, 2**63, size=n, dtype=np.uint64).astype(key_dtype)
        raw[::11] = raw[0]
        vals = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
        ek, ev = orc.std_sort(raw, vals if with_values else None)
        key = gbc.tuning_sort_key(kb_, with_values, n)
        try:
            for var in range(gbc.tuning_sort_variants(kb_, with_values)):
                ctx.tuning_set(key, var)
                for shift in (0, 1):  # element offset 1: not 16-byte aligned
                    kin = gbc.DeviceBuffer.from_host(ctx, np.concatenate([raw[:shift], raw]))
                    vin = gbc.DeviceBuffer.from_host(ctx, np.concatenate([vals[:shift], vals]))
                    kout = gbc.DeviceBuffer(ctx, n + shift, key_dtype)
                    vout = gbc.DeviceBuffer(ctx, n + shift, np.uint32)
                    kp = lambda b: b.device_pointer + shift * b.dtype.itemsize
                    gbc.sort_raw(ctx, kp(kin), kp(kout), key_dtype, n, kp(vin) if with_values else 0,
                                 kp(vout) if with_values else 0)
                    assert np.array_equal(kout.to_host()[shift:], ek), (var, n, shift)
                    if with_values:
                        assert np.array_equal(vout.to_host()[shift:], ev), (var, n, shift)
        finally:
            ctx.tuning_set(key, 0)
