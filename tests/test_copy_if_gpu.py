"""copy_if against the reference's own test recipes and numpy (C integer
semantics: % truncates toward zero, mixed signed/unsigned operands convert
to unsigned), with the predicate grammar's limits."""
import numpy as np
import pytest
from helpers import SIZES

pytestmark = pytest.mark.gpu


def run(ctx, gbc, x, pred):
    a = gbc.DeviceBuffer.from_host(ctx, x)
    o = gbc.DeviceBuffer(ctx, max(x.size, 1), x.dtype)
    count = gbc.copy_if(ctx, a, o, pred)
    return o.to_host()[:count], count


@pytest.mark.parametrize("n", SIZES)
def test_reference_recipe_mod3(ctx, gbc, orc, n):
    # main.cpp:314-327: random_uints(n, 1000, n + 3), "(x % 3u) == 0u"
    host = orc.random_uints(n, 1000, n + 3)
    got, count = run(ctx, gbc, host, "(x % 3u) == 0u")
    ref = host[host % 3 == 0]
    assert count == ref.size and np.array_equal(got, ref)


def test_reference_recipe_positive_int32(ctx, gbc):
    # capi.c:130: "x > 0" on int32 data
    rng = np.random.default_rng(11)
    x = rng.integers(-1000, 1000, size=100003, dtype=np.int32)
    got, count = run(ctx, gbc, x, "x > 0")
    assert count == int((x > 0).sum()) and np.array_equal(got, x[x > 0])


@pytest.mark.parametrize("dtype,pred,ref", [
    (np.int32, "(x % 7) != 0", lambda x: np.fmod(x, 7) != 0),
    (np.int32, "(x % 7u) == 1u", lambda x: (x.astype(np.uint32) % 7) == 1),   # int converts to unsigned
    (np.int64, "x >= -5 && x < 17", lambda x: (x >= -5) & (x < 17)),
    (np.uint64, "(x & 0xFF) == 0x10 || x < 100", lambda x: ((x & 0xFF) == 0x10) | (x < 100)),
    (np.uint8, "x > 200", lambda x: x > 200),
    (np.int16, "x <= -3", lambda x: x <= -3),
    (np.float32, "x < 0.25f", lambda x: x < np.float32(0.25)),
    (np.float64, "x > 0.5 && x != 0.75", lambda x: (x > 0.5) & (x != 0.75)),
])
def test_types_and_grammar(ctx, gbc, dtype, pred, ref):
    rng = np.random.default_rng(5)
    n = 1_000_003
    if np.dtype(dtype).kind == "f":
        x = rng.random(n).astype(dtype)
        x[::97] = 0.75
    elif np.dtype(dtype).kind == "u":
        x = rng.integers(0, np.iinfo(dtype).max, size=n, dtype=np.uint64).astype(dtype)
        x[::13] = 0x10
    else:
        lo = max(np.iinfo(dtype).min, -(1 << 40))
        hi = min(np.iinfo(dtype).max, 1 << 40)
        x = rng.integers(lo, hi, size=n, dtype=np.int64).astype(dtype)
        x[::11] = rng.integers(-20, 20, size=x[::11].size)
    got, count = run(ctx, gbc, x, pred)
    want = x[ref(x)]
    assert count == want.size and np.array_equal(got, want)


def test_edge_sizes_and_all_or_nothing(ctx, gbc):
    for n in (1, 2, 4095, 4096, 4097, 65537):
        x = np.arange(n, dtype=np.uint32)
        got, count = run(ctx, gbc, x, "x >= 0u")
        assert count == n and np.array_equal(got, x)
        got, count = run(ctx, gbc, x, "x > 4294967295u")
        assert count == 0


@pytest.mark.parametrize("pred", ["x*2 > 3", "foo > 1", "(x % 0) == 0", "(x % 2.0) == 0", "x > 1 && x < 5 || x == 9",
                                  "y > 0", "x >"])
def test_outside_grammar_is_unsupported(ctx, gbc, pred):
    x = np.arange(100, dtype=np.int32)
    with pytest.raises(gbc.UnsupportedError):
        run(ctx, gbc, x, pred)
