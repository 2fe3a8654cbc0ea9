"""Scan and reduce parity on the GPU (lib/test/Compute/main.cpp:182-244 and
capi.c:114-123): integer results bit-exact against the golden fixtures and
the oracle; floating-point sums within a stated tolerance."""
import numpy as np
import pytest
from helpers import GOLDEN, SIZES, digest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", SIZES)
def test_scan_reference_recipe(ctx, gbc, orc, n):
    host = orc.random_uints(n, 100, n + 1)
    inp = gbc.DeviceBuffer.from_host(ctx, host)
    out = gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.inclusive_scan(ctx, inp, out)
    assert digest(out.to_host()) == GOLDEN["scan"][str(n)]["inclusive"]
    gbc.exclusive_scan(ctx, inp, out)
    assert digest(out.to_host()) == GOLDEN["scan"][str(n)]["exclusive"]
    gbc.inclusive_scan(ctx, inp, inp)  # in place
    assert digest(inp.to_host()) == GOLDEN["scan"][str(n)]["inclusive"]


def test_scan_non_commutative_and_max(ctx, gbc):
    v = (np.arange(5000, dtype=np.int64) * 7 % 101).astype(np.int32)
    vb = gbc.DeviceBuffer.from_host(ctx, v)
    vo = gbc.DeviceBuffer(ctx, v.size, np.int32)
    gbc.inclusive_scan(ctx, vb, vo, gbc.binary_op("b", "0"))
    assert np.array_equal(vo.to_host(), v)
    gbc.inclusive_scan(ctx, vb, vo, gbc.ops.maximum(np.int32))
    assert digest(vo.to_host()) == GOLDEN["scan_max"]["inclusive"]
    gbc.exclusive_scan(ctx, vb, vo, gbc.binary_op("b", "0"))
    got = vo.to_host()
    assert got[0] == 0 and np.array_equal(got[1:], v[:-1])


@pytest.mark.parametrize("dtype", [np.int32, np.uint32, np.int64, np.uint64])
@pytest.mark.parametrize("opname", ["plus", "multiplies", "bit_and", "bit_or", "bit_xor", "minimum", "maximum"])
def test_scan_ops_types(ctx, gbc, orc, dtype, opname):
    rng = np.random.default_rng(5)
    n = 123457
    info = np.iinfo(dtype)
    x = rng.integers(max(info.min, -(2**40)), min(info.max, 2**40), size=n, dtype=np.int64).astype(dtype)
    if opname == "multiplies":
        x = (x & dtype(3)) | dtype(1)
    op = getattr(gbc.ops, opname)(dtype) if opname in ("minimum", "maximum") else getattr(gbc.ops, opname)()
    code = orc.OPS[op.expression]
    ident = {"0": 0, "1": 1, "(~0)": -1 if info.min < 0 else info.max}.get(op.identity)
    if ident is None:
        ident = info.max if opname == "minimum" else info.min
    inp = gbc.DeviceBuffer.from_host(ctx, x)
    out = gbc.DeviceBuffer(ctx, n, dtype)
    for exclusive in (False, True):
        (gbc.exclusive_scan if exclusive else gbc.inclusive_scan)(ctx, inp, out, op)
        assert np.array_equal(out.to_host(), orc.std_scan(x, code, ident, exclusive)), (opname, exclusive)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_scan_float(ctx, gbc, orc, dtype):
    rng = np.random.default_rng(6)
    n = 200003
    x = rng.uniform(-1, 1, size=n).astype(dtype)
    inp = gbc.DeviceBuffer.from_host(ctx, x)
    out = gbc.DeviceBuffer(ctx, n, dtype)
    gbc.inclusive_scan(ctx, inp, out, gbc.ops.maximum(dtype))
    assert np.array_equal(out.to_host(), np.maximum.accumulate(x))  # exact
    gbc.inclusive_scan(ctx, inp, out)
    ref = np.cumsum(x.astype(np.float64))
    # Sums associate differently from a sequential loop: |err| <= n * eps * sum|x|
    tol = (4e-7 if dtype == np.float32 else 1e-15) * np.cumsum(np.abs(x.astype(np.float64))) * 64
    assert np.all(np.abs(out.to_host().astype(np.float64) - ref) <= tol + 1e-6)


def test_scan_int32_wide_total(ctx, gbc, orc):
    # config shape at reduced n: int32 in [-1000, 1000], exclusive, int64 total
    rng = np.random.default_rng(2)
    n = (1 << 22) + 123
    x = rng.integers(-1000, 1001, size=n, dtype=np.int64).astype(np.int32)
    inp = gbc.DeviceBuffer.from_host(ctx, x)
    out = gbc.DeviceBuffer(ctx, n, np.int32)
    total = gbc.exclusive_scan(ctx, inp, out, total=True)
    assert int(total) == orc.sum_i32(x)
    assert np.array_equal(out.to_host(), orc.std_scan(x, exclusive=True))
    # wrap-around is mod 2^32, the total is not
    big = np.full(4096 * 3 + 5, 2**30, dtype=np.int32)
    bb = gbc.DeviceBuffer.from_host(ctx, big)
    bo = gbc.DeviceBuffer(ctx, big.size, np.int32)
    total = gbc.inclusive_scan(ctx, bb, bo, total=True)
    assert int(total) == big.size * 2**30
    assert np.array_equal(bo.to_host(), orc.std_scan(big))


@pytest.mark.parametrize("n", SIZES)
def test_reduce_reference_recipe(ctx, gbc, orc, n):
    host = orc.random_uints(n, 1000, n)
    buf = gbc.DeviceBuffer.from_host(ctx, host)
    g = GOLDEN["reduce"][str(n)]
    assert int(gbc.reduce(ctx, buf, gbc.ops.plus(), 7)) == g["sum_init7"]
    if n:
        assert int(gbc.reduce(ctx, buf, gbc.ops.maximum(np.uint32), 0)) == g["max"]
        assert int(gbc.reduce(ctx, buf, gbc.ops.minimum(np.uint32), 0xFFFFFFFF)) == g["min"]


def test_reduce_floats_and_wide(ctx, gbc, orc):
    f = (np.arange(10000) % 17).astype(np.float32) - 8.0  # main.cpp:200-204
    fb = gbc.DeviceBuffer.from_host(ctx, f)
    assert gbc.reduce(ctx, fb, gbc.ops.maximum(np.float32), -np.inf) == 8.0
    assert gbc.reduce(ctx, fb, gbc.ops.minimum(np.float32), np.inf) == -8.0
    rng = np.random.default_rng(9)
    d = rng.uniform(-1e3, 1e3, size=1000003)
    db = gbc.DeviceBuffer.from_host(ctx, d)
    s = gbc.reduce(ctx, db, gbc.ops.plus(), 0.0)
    assert abs(s - d.sum()) <= 1e-9 * np.abs(d).sum()
    x = rng.integers(-2**62, 2**62, size=777777, dtype=np.int64)
    xb = gbc.DeviceBuffer.from_host(ctx, x)
    assert int(gbc.reduce(ctx, xb, gbc.ops.bit_xor(), 0)) == int(np.bitwise_xor.reduce(x))
    assert int(gbc.reduce(ctx, xb, gbc.ops.plus(), 0)) == int(orc.std_reduce(x, orc.OP_PLUS, 0, 0))
