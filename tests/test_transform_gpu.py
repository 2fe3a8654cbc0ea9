"""transform / transform2 on the GPU, bit-exact against the independent CPU
oracle (transform_oracle): the reference's own recipes (main.cpp:155-178,
capi.c:103-128 and 153-157, compute-pipeline main.cpp:149-164), then every
operator, conversion and operand form over random data with planted edge
values (zero divisors, INT_MIN / -1, NaN, infinities, out-of-range floats),
both interpreter widths, ragged sizes, unaligned pointers and in-place use."""
import zlib

import numpy as np
import pytest
from helpers import SIZES

import transform_oracle as T

pytestmark = pytest.mark.gpu


def gpu_transform(ctx, gbc, expr, x, out_dtype, y=None, out_alias=None):
    bx = gbc.DeviceBuffer.from_host(ctx, x)
    by = gbc.DeviceBuffer.from_host(ctx, y) if y is not None else None
    if out_alias == "x":
        bo = bx
    else:
        bo = gbc.DeviceBuffer(ctx, max(x.size, 1), out_dtype)
    if y is None:
        gbc.transform(ctx, bx, bo, expr)
    else:
        gbc.transform(ctx, bx, by, bo, expr)
    return bo.to_host()[: x.size]


def same(got, want):
    """Bit-exact, except that any NaN matches any NaN (payloads are not
    specified by C)."""
    assert got.dtype == want.dtype and got.shape == want.shape
    if got.dtype.kind == "f":
        u = np.dtype(f"u{got.dtype.itemsize}")
        ok = (got.view(u) == want.view(u)) | (np.isnan(got) & np.isnan(want))
    else:
        ok = got == want
    bad = np.flatnonzero(~ok)
    assert bad.size == 0, f"{bad.size} mismatches, first at {bad[:5]}: got {got[bad[:5]]} want {want[bad[:5]]}"


@pytest.mark.parametrize("n", SIZES)
def test_reference_sequence_recipes(ctx, gbc, n):
    # main.cpp:155-178
    seq = gbc.DeviceBuffer(ctx, n, np.int32)
    if n == 0:  # empty buffers are valid and nothing runs
        gbc.transform(ctx, seq, gbc.DeviceBuffer(ctx, 0, np.float32), "(float)x * 0.5f")
        return
    gbc.sequence(ctx, seq, 5, 3)
    expected = (5 + 3 * np.arange(n, dtype=np.int64)).astype(np.int32)
    out = gbc.DeviceBuffer(ctx, n, np.float32)
    gbc.transform(ctx, seq, out, "(float)x * 0.5f")
    same(out.to_host(), expected.astype(np.float32) * np.float32(0.5))
    prod = gbc.DeviceBuffer(ctx, n, np.int32)
    gbc.transform(ctx, seq, seq, prod, "x * y - 1")
    with np.errstate(over="ignore"):
        same(prod.to_host(), (expected.astype(np.int64) ** 2 - 1).astype(np.int32))


def test_reference_capi_recipe(ctx, gbc):
    # capi.c:103-128 and 153-157 through the C ABI
    N = 10007
    host = ((np.arange(N, dtype=np.uint64) * 7919) % 1000).astype(np.int32) - 500
    fout = gpu_transform(ctx, gbc, "(float)x * 0.5f", host, np.float32)
    assert fout[3] == np.float32(host[3]) * np.float32(0.5)
    same(fout, T.transform("(float)x * 0.5f", host, np.float32))
    with pytest.raises(gbc.BuildError) as e:
        gpu_transform(ctx, gbc, "x +* nonsense", host, np.int32)
    assert "build log" in str(e.value)


def test_reference_pipeline_recipe_in_place(ctx, gbc):
    # compute-pipeline main.cpp:149 and 164: calibrate in place ("x + y" into
    # the first input), then convert to Fahrenheit.
    rng = np.random.default_rng(42)
    n = 1 << 20
    readings = (150 + rng.integers(0, 300, n) + np.where(rng.integers(0, 1000, n) == 0, 600, 0)).astype(np.uint32)
    offsets = (rng.integers(0, 1000, n) % 7).astype(np.uint32)
    d_r = gbc.DeviceBuffer.from_host(ctx, readings)
    d_o = gbc.DeviceBuffer.from_host(ctx, offsets)
    gbc.transform(ctx, d_r, d_o, d_r, "x + y")
    cal = readings + offsets
    same(d_r.to_host(), cal)
    d_f = gbc.DeviceBuffer(ctx, n, np.float32)
    gbc.transform(ctx, d_r, d_f, "x * 0.18f + 32.0f")
    same(d_f.to_host(), cal.astype(np.float32) * np.float32(0.18) + np.float32(32.0))


def sample(dtype, n, rng, divisor=False):
    dt = np.dtype(dtype)
    if dt.kind == "f":
        v = (rng.standard_normal(n) * 10.0 ** rng.integers(-3, 12, n)).astype(dt)
        specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 0.5, 2.0**31, -2.0**31, 2.0**32,
                             2.0**63, 2.0**64, -2.0**63, 255.5, -0.75, 1e-40], dtype=np.float64).astype(dt)
        v[rng.integers(0, n, n // 20)] = specials[rng.integers(0, specials.size, n // 20)]
        return v
    info = np.iinfo(dt)
    v = rng.integers(info.min, info.max, size=n, dtype=dt, endpoint=True)
    specials = np.array([0, 1, info.max, info.min] + ([-1] if dt.kind == "i" else []), dtype=dt)
    k = n // (5 if divisor else 20)
    v[rng.integers(0, n, k)] = specials[rng.integers(0, specials.size, k)]
    return v


I8, U8, I16, U16, I32, U32, I64, U64, F32, F64 = (np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32,
                                                  np.int64, np.uint64, np.float32, np.float64)

CASES = [
    # 32-bit interpreter
    ("x * 0.18f + 32.0f", U32, None, F32),
    ("(float)x * 0.5f", I32, None, F32),
    ("x + y", U32, U32, U32),
    ("x * y - 1", I32, I32, I32),
    ("x / y", I32, I32, I32),
    ("x % y", I32, I32, I32),
    ("x / y + x % y", U32, U32, U32),
    ("(x << y) ^ (x >> (y + 3))", I32, I32, I32),
    ("(x << y) | (x >> y)", U32, U32, U32),
    ("x < y ? y - x : x - y", F32, F32, F32),
    ("min(x, y) + max(x, y) * 2.0f", F32, F32, F32),
    ("fmin(x, 0.0f) - fmax(y, -1.0f)", F32, F32, F32),
    ("x / y", F32, F32, F32),
    ("clamp(x, -100, 100)", I32, None, I8),
    ("abs(x) >> 1", I32, None, U32),
    ("fabs(x) / (y + 1.0f)", F32, F32, F32),
    ("as_float(as_uint(x) ^ 0x80000000u)", F32, None, F32),
    ("(int)x", F32, None, I32),
    ("(uint)x", F32, None, U32),
    ("x", F32, None, U8),
    ("x * 3 + y", U8, I16, I16),
    ("(char)x + (uchar)y", I32, U32, I32),
    ("!x + (x && y) * 2 + (x || y) * 4", I32, U32, I32),
    ("~x & 0xFF00FF", U32, None, U32),
    ("-x", U32, None, U32),
    ("x == y", F32, F32, I32),
    ("x != x", F32, None, U8),
    ("((x + 1) * (y - 2)) / ((x - 3) + (y * 5) + 1)", I32, I32, I32),
    ("(x+1) * ((y+2) * ((x+3) * ((y+4) * (x+5))))", I32, I32, I32),
    ("x ? y : 7", I32, I32, I32),
    ("x > 0.5f ? x : y", F32, F32, F32),
    ("convert_int(x) + as_int(y)", F32, F32, I32),
    ("INT_MAX + x", I32, None, I32),
    ("abs((char)x) - 200", I32, None, I32),
    ("min((uchar)x, (uchar)y) * 3", U32, U32, U16),
    ("x >= 700u", U32, None, U32),
    ("clamp(x, 0.0f, 1.0f) * 255.0f", F32, None, U8),
    ("x", U16, None, F32),
    ("(short)x", F32, None, I32),
    # 64-bit interpreter
    ("x - 2147483648", I32, None, I64),
    ("x + y", I64, I64, I64),
    ("x * y", U64, U64, U64),
    ("x / y", I64, I64, I64),
    ("x % y", U64, U64, U64),
    ("x % y", I64, I64, I64),
    ("x * 0.5 + y", F64, F64, F64),
    ("x / y", F64, F64, F64),
    ("(double)x * 1e-3", I64, None, F64),
    ("(float)x", U64, None, F32),
    ("(float)x", I64, None, F32),
    ("(double)x", U64, None, F64),
    ("(long)x", F64, None, I64),
    ("(ulong)x", F64, None, U64),
    ("(long)x", F32, None, I64),
    ("(float)x", F64, None, F32),
    ("x", F64, None, I16),
    ("x << y", I64, U8, I64),
    ("x >> y", I64, I32, I64),
    ("x >> y", U64, U64, U64),
    ("min(x, y)", I64, U32, I64),
    ("x + y", I32, U64, U64),
    ("x * 2.5", F32, None, F64),
    ("abs(x)", I64, None, U64),
    ("x > y ? x : y", U64, I64, U64),
    ("x + 1", U64, None, U8),
    ("x", I32, None, F64),
    ("as_double(x)", U64, None, F64),
    ("-x * (y + 0.25)", F64, F32, F64),
    ("max(x, y) - min(x, y)", F64, F64, F64),
    ("(x & 0xFFFFFFFF00000000UL) | (y & 0xFFFFu)", U64, U32, U64),
    ("x ? (double)y : -1.0", I64, F32, F64),
    # division by integer literals (multiply-high), every sign and width
    ("x / 3 + x % 3", I32, None, I32),
    ("x / -7 * 100 + x % -7", I32, None, I32),
    ("x / 1000000007", I32, None, I32),
    ("x % 65536 + x / 2", I32, None, I32),
    ("x / 3u + x % 10u", U32, None, U32),
    ("x / 4294967295u + x % 641u", U32, None, U32),
    ("x / 7 + x % 2147483647", U32, None, U32),
    ("x / 3 - x % 5", I64, None, I64),
    ("x / -1000000000000 + x % 97", I64, None, I64),
    ("x / 3ul + x % 1000000000039ul", U64, None, U64),
    ("x / 18446744073709551615ul", U64, None, U64),
    ("(x % 3u) == 0u", U32, None, U8),
    ("x / 9 + x % 9", I16, None, I32),
    ("100 / (x | 1)", I32, None, I32),
]


@pytest.mark.parametrize("expr,tx,ty,to", CASES, ids=[f"{c[0]}|{np.dtype(c[1])}|{c[2] and np.dtype(c[2])}|"
                                                        f"{np.dtype(c[3])}" for c in CASES])
def test_parity_random(ctx, gbc, expr, tx, ty, to):
    rng = np.random.default_rng(zlib.crc32(expr.encode()))
    n = 1_000_003  # not a multiple of the chunk: ragged tail
    divides = "/" in expr or "%" in expr
    x = sample(tx, n, rng)
    y = sample(ty, n, rng, divisor=divides) if ty is not None else None
    got = gpu_transform(ctx, gbc, expr, x, to, y)
    want = T.transform(expr, x, to, y)
    same(got, np.asarray(want, dtype=np.dtype(to)))


@pytest.mark.parametrize("n", [1, 2, 3, 7, 8, 9, 255, 256, 257, 2047, 2048, 2049, 4097, 100003])
@pytest.mark.parametrize("expr,tx,to", [("x * 3u + 1u", U32, U32), ("(double)x / 7.0", I64, F64),
                                        ("x + 1", U8, U8)])
def test_ragged_sizes(ctx, gbc, n, expr, tx, to):
    rng = np.random.default_rng(n)
    x = sample(tx, n, rng)
    same(gpu_transform(ctx, gbc, expr, x, to), T.transform(expr, x, to))


@pytest.mark.parametrize("offset", [1, 2, 3])
def test_unaligned_pointers(ctx, gbc, offset):
    # device pointers off the 16-byte boundary take the element-wise path
    rng = np.random.default_rng(offset)
    n = 50_001
    x = sample(U32, n + 4, rng)
    y = sample(U32, n + 4, rng)
    bx = gbc.DeviceBuffer.from_host(ctx, x)
    by = gbc.DeviceBuffer.from_host(ctx, y)
    bo = gbc.DeviceBuffer(ctx, n + 4, np.uint32)
    wx = gbc.DeviceBuffer.wrap(ctx, bx.device_pointer + 4 * offset, n, np.uint32)
    wy = gbc.DeviceBuffer.wrap(ctx, by.device_pointer + 4 * offset, n, np.uint32)
    wo = gbc.DeviceBuffer.wrap(ctx, bo.device_pointer + 4 * offset, n, np.uint32)
    gbc.transform(ctx, wx, wy, wo, "x * y + (x >> 3)")
    got = bo.to_host()[offset: offset + n]
    same(got, T.transform("x * y + (x >> 3)", x[offset: offset + n], np.uint32, y[offset: offset + n]))


def test_in_place_unary(ctx, gbc):
    rng = np.random.default_rng(3)
    x = sample(F32, 300_001, rng)
    got = gpu_transform(ctx, gbc, "x * x - 1.0f", x, F32, out_alias="x")
    same(got, T.transform("x * x - 1.0f", x, F32))


def test_errors(ctx, gbc):
    x = np.arange(16, dtype=np.int32)
    with pytest.raises(gbc.UnsupportedError):
        gpu_transform(ctx, gbc, "sqrt(x)", x, np.float32)
    with pytest.raises(gbc.BuildError):
        gpu_transform(ctx, gbc, "x + z", x, np.int32)
    a = gbc.DeviceBuffer.from_host(ctx, x)
    small = gbc.DeviceBuffer(ctx, 8, np.int32)
    with pytest.raises(ValueError):
        gbc.transform(ctx, a, small, "x + 1")
