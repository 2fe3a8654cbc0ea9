"""copy_if against the reference's own test recipes and numpy (C integer
semantics: % truncates toward zero, mixed signed/unsigned operands convert
to unsigned), general OpenCL C predicates against the oracle's truth value,
and the BUILD / UNSUPPORTED classification of the rest."""
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


PREDICATES = [
    # the reference's own and general OpenCL C predicates, checked against the
    # oracle's truth value of the same expression
    (np.int32, "x*2 > 3"),
    (np.int32, "(x % 0) == 0"),                 # x % 0 is defined as 0 here
    (np.int32, "x > 1 && x < 5 || x == 9"),
    (np.int32, "x"),                            # truthiness: nonzero
    (np.int32, "abs(x) < 100 ? x & 1 : x > 0"),
    (np.uint32, "x >= 700u"),                   # compute-pipeline main.cpp:160
    (np.uint32, "(x & 1u) == 0u"),              # lib/Compute.md:51
    (np.float32, "x * 0.5f > 0.25f"),
    (np.float32, "x"),                          # NaN is nonzero: kept
    (np.float32, "x != x"),
    (np.float64, "(x > 0.5) == (x < 0.75)"),
    (np.int64, "x % 3 == -1"),
    (np.uint64, "(x >> 40) > 100"),
    (np.uint8, "x - 100"),                      # int arithmetic after promotion
    (np.int16, "(x ^ 0x5555) < 0"),
    (np.int32, "(x+1) * ((x+2) * (x+3)) > 0"),  # uses the temporaries
    # `x OP literal` on 4-byte elements: the inlined-comparison count pass
    (np.int32, "x < -5"),
    (np.int32, "x <= 7"),
    (np.int32, "x >= -2147483647 - 1"),
    (np.int32, "x == 0"),
    (np.int32, "x != 3"),
    (np.uint32, "x > 4000000000u"),
    (np.uint32, "x == 5u"),
    (np.float32, "x < 0.0f"),                   # NaN and -0.0 not kept
    (np.float32, "x >= -0.0f"),
    (np.float32, "x != 1.5f"),                  # NaN kept
    (np.float32, "x == 0.0f"),                  # -0.0 kept
]


def sample(dtype, n, rng):
    dt = np.dtype(dtype)
    if dt.kind == "f":
        v = (rng.standard_normal(n) * 2).astype(dt)
        v[::37] = np.nan
        v[::41] = 0.0
        v[::43] = -0.0
        v[::47] = 1.5
        return v
    info = np.iinfo(dt)
    v = rng.integers(info.min, info.max, size=n, dtype=dt, endpoint=True)
    v[::13] = rng.integers(-20, 20, size=v[::13].size).astype(dt)
    return v


@pytest.mark.parametrize("dtype,pred", PREDICATES, ids=[f"{np.dtype(d)}|{p}" for d, p in PREDICATES])
def test_general_predicates(ctx, gbc, dtype, pred):
    import transform_oracle as T

    rng = np.random.default_rng(len(pred) * 7 + np.dtype(dtype).itemsize)
    for n in (1, 4097, 300_001):
        x = sample(dtype, n, rng)
        got, count = run(ctx, gbc, x, pred)
        want = x[T.truth(pred, x)]
        assert count == want.size
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8))  # bit-exact, NaN included


@pytest.mark.parametrize("pred", ["foo > 1", "(x % 2.0) == 0", "y > 0", "x >", "x +* nonsense"])
def test_malformed_predicate_is_a_build_error(ctx, gbc, pred):
    x = np.arange(100, dtype=np.int32)
    with pytest.raises(gbc.BuildError) as e:
        run(ctx, gbc, x, pred)
    assert "build log" in str(e.value)


@pytest.mark.parametrize("pred", ["sqrt(x) > 1", "(float4)x", "mad(x, x, x) > 0"])
def test_outside_the_subset_is_unsupported(ctx, gbc, pred):
    x = np.arange(100, dtype=np.int32)
    with pytest.raises(gbc.UnsupportedError):
        run(ctx, gbc, x, pred)
