"""transform / transform2 without a GPU: the oracle against the reference's
own transform recipes, and the library's expression compiler (typing,
operand forms, BUILD vs UNSUPPORTED classification) through
clc_transform_compile."""
import numpy as np
import pytest
from helpers import SIZES

import transform_oracle as T


@pytest.fixture(scope="module")
def gbc():
    import gbcompute

    return gbcompute


@pytest.mark.parametrize("n", SIZES)
def test_oracle_reference_sequence_recipes(n):
    # lib/test/Compute/main.cpp:155-178: seq = 5 + 3 i; "(float)x * 0.5f"
    # into floats; "x * y - 1" with x = y = seq; fill 2.5f.
    seq = (5 + 3 * np.arange(n, dtype=np.int64)).astype(np.int32)
    half = np.array([np.float32(float(v)) * np.float32(0.5) for v in seq[:1000]], dtype=np.float32)
    got = T.transform("(float)x * 0.5f", seq, np.float32)
    assert np.array_equal(got[:1000], half)
    with np.errstate(over="ignore"):
        squares = (seq.astype(np.int64) * seq.astype(np.int64) - 1).astype(np.int32)  # wraps like cl_int
    assert np.array_equal(T.transform("x * y - 1", seq, np.int32, seq), squares)


def test_oracle_capi_recipe():
    # lib/test/Compute/capi.c:103-128: host[i] = (i * 7919) % 1000 - 500,
    # "(float)x * 0.5f" from I32 to F32, fout[3] == (float)host[3] * 0.5f.
    N = 10007
    host = ((np.arange(N, dtype=np.uint64) * 7919) % 1000).astype(np.int32) - 500
    out = T.transform("(float)x * 0.5f", host, np.float32)
    assert out[3] == np.float32(host[3]) * np.float32(0.5)
    assert np.array_equal(out, host.astype(np.float32) * np.float32(0.5))


def test_oracle_pipeline_recipe():
    # samples/core/compute-pipeline/main.cpp:97-164: readings 150 + rng % 300
    # (+600 now and then), offsets = sensor % 7; "x + y" then
    # "x * 0.18f + 32.0f" to Fahrenheit.
    rng = np.random.default_rng(42)
    n = 100_000
    readings = (150 + rng.integers(0, 300, n) + np.where(rng.integers(0, 1000, n) == 0, 600, 0)).astype(np.uint32)
    offsets = (rng.integers(0, 1000, n) % 7).astype(np.uint32)
    cal = T.transform("x + y", readings, np.uint32, offsets)
    assert np.array_equal(cal, readings + offsets)
    f = T.transform("x * 0.18f + 32.0f", cal, np.float32)
    want = (cal.astype(np.float32) * np.float32(0.18)) + np.float32(32.0)
    assert np.array_equal(f, want)


def test_oracle_c_semantics():
    x = np.array([0, 1, -3, 7, -2**31, 2**31 - 1], dtype=np.int32)
    assert list(T.transform("x / -1", x, np.int32)) == [0, -1, 3, -7, -2**31, -(2**31 - 1)]
    assert list(T.transform("x % 3", x, np.int32)) == [0, 1, 0, 1, -2, 1]       # truncating
    assert list(T.transform("x / 0", x, np.int32)) == [0] * 6                     # defined as 0
    assert list(T.transform("x << 33", x, np.int32)) == [0, 2, -6, 14, 0, -2]    # count & 31
    assert list(T.transform("abs(x)", x, np.uint32)) == [0, 1, 3, 7, 2**31, 2**31 - 1]
    assert list(T.transform("x < 0u", x, np.int32)) == [0] * 6                    # int -> uint
    assert list(T.transform("x < 0L", x, np.int32)) == [0, 0, 1, 0, 1, 0]         # int -> long
    f = np.array([np.nan, -1.5, 3e9, -3e9, 0.9, 255.7, 300.2], dtype=np.float32)
    assert list(T.transform("x", f, np.int32)) == [0, -1, 2**31 - 1, -2**31, 0, 255, 300]
    assert list(T.transform("x", f, np.uint32)) == [0, 0, 3000000000, 0, 0, 255, 300]
    assert list(T.transform("x", f, np.uint8)) == [0, 255, 255, 0, 0, 255, 44]
    y = np.array([1.0, np.nan, -2.0, 0.0, np.nan, 1.0, 2.0], dtype=np.float32)
    m = T.transform("min(x, y)", f, np.float32, y)
    assert np.isnan(m[0]) is np.False_ and m[0] == 1.0 and m[1] == -1.5 and m[4] == np.float32(0.9)


def listing(gbc, expr, tx, tout, ty=None):
    return gbc.transform_compile(expr, tx, tout, ty).split("\n")[:-1]


def test_compiler_reference_expressions(gbc):
    assert listing(gbc, "(float)x * 0.5f", np.int32, np.float32) == [
        "load.i32 x", "cvt.i32->f32", "mul.f32 #0x3f000000"]
    assert listing(gbc, "x * y - 1", np.int32, np.int32, np.int32) == ["load.i32 x", "mul.i32 y", "sub.i32 #0x1"]
    assert listing(gbc, "x + y", np.uint32, np.uint32, np.uint32) == ["load.u32 x", "add.u32 y"]
    assert listing(gbc, "x * 0.18f + 32.0f", np.uint32, np.float32) == [
        "load.u32 x", "cvt.u32->f32", "mul.f32 #0x3e3851ec", "add.f32 #0x42000000"]


def test_compiler_typing(gbc):
    # int literal vs uint data: the usual arithmetic conversions give uint
    assert listing(gbc, "x - 1", np.uint32, np.uint32) == ["load.u32 x", "sub.u32 #0x1"]
    # a decimal literal above INT_MAX is long: the operation widens
    assert listing(gbc, "x + 3000000000", np.int32, np.int64) == ["load.i32 x", "cvt.i32->i64", "add.i64 #0xb2d05e00"]
    # double literal: the float operand converts to double, the result back
    assert listing(gbc, "x * 0.5", np.float32, np.float32) == [
        "load.f32 x", "cvt.f32->f64", "mul.f64 #0x3fe0000000000000", "cvt.f64->f32"]
    # char data promotes to int; narrow result re-extended
    assert listing(gbc, "(uchar)(x + 1)", np.int8, np.int32) == ["load.i32 x", "add.i32 #0x1", "ext8u.i32"]
    # a literal on the left becomes a reversed operation
    assert listing(gbc, "100 - x * 3", np.int32, np.int32) == ["load.i32 x", "mul.i32 #0x3", "rsub.i32 #0x64"]
    # abs of int is uint: the following shift is logical
    assert listing(gbc, "abs(x) >> 1", np.int32, np.uint32) == ["load.i32 x", "abs.i32", "shr.u32 #0x1"]
    # two non-leaf operands use a stack slot
    assert listing(gbc, "(x + 1) * (y - 2)", np.int32, np.int32, np.int32) == [
        "load.i32 x", "add.i32 #0x1", "push.i32 st0", "load.i32 y", "sub.i32 #0x2", "mul.i32 st0"]


@pytest.mark.parametrize("expr", ["x +* nonsense", "foo(x)", "y + 1", "x % 1.5f", "", "x = 3", "x++", "1e",
                                  "0x", "08", "(x", "x)", "abs(1.5f)", "fmin(x, 1)", "as_long(x)", "x << 1.0f",
                                  "max(x)", "~1.0f", "x $ 2"])
def test_compiler_build_errors(gbc, expr):
    with pytest.raises(gbc.BuildError) as e:
        gbc.transform_compile(expr, np.int32, np.int32)
    assert "build log" in str(e.value)  # capi.c:153-157


@pytest.mark.parametrize("expr", ["sqrt(x)", "(float4)x", "x, 1", "(half)x", "convert_int_sat(x)", "M_PI_F * x",
                                  "0x1p3f", "mad(x, x, x)",
                                  "(x+1) * ((x+2) * ((x+3) * ((x+4) * ((x+5) * (x+6)))))"])
def test_compiler_unsupported(gbc, expr):
    with pytest.raises(gbc.UnsupportedError):
        gbc.transform_compile(expr, np.int32, np.int32)


@pytest.mark.parametrize("expr", ["x +* nonsense", "foo(x)", "x % 1.5f", "abs(1.5f)", "x << 1.0f"])
def test_oracle_agrees_on_build_errors(expr):
    with pytest.raises(SyntaxError):
        T.transform(expr, np.arange(4, dtype=np.int32), np.int32)


HOSTILE = {
    "parentheses": lambda k: "(" * k + "x" + ")" * k,
    "prefix_operators": lambda k: "!" * k + "x",
    "casts": lambda k: "(int)" * k + "x",
    "ternaries": lambda k: "x ? " * k + "x" + " : x" * k,
    "operator_chain": lambda k: "x" + " + x" * k,
    "call_arguments": lambda k: "min(" * k + "x" + ", 1)" * k,
}


@pytest.mark.parametrize("form", sorted(HOSTILE))
def test_compiler_refuses_hostile_nesting(form):
    # 100,000 levels must come back as an error status, not a stack
    # overflow of the caller's process: run in a child process so that a
    # crash fails this test instead of the test run.
    import os
    import subprocess
    import sys

    text = HOSTILE[form](100_000)
    here = os.path.dirname(os.path.abspath(__file__))
    code = (
        "import sys, numpy as np\n"
        f"sys.path.insert(0, {os.path.join(os.path.dirname(here), 'opencl-sdk_gb300')!r})\n"
        "import gbcompute as gbc\n"
        "text = sys.stdin.read()\n"
        "try:\n"
        "    gbc.transform_compile(text, np.int32, np.int32)\n"
        "    print('compiled')\n"
        "except (gbc.UnsupportedError, gbc.BuildError) as e:\n"
        "    print(type(e).__name__)\n"
    )
    r = subprocess.run([sys.executable, "-c", code], input=text, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr[-500:])
    assert r.stdout.strip() in ("UnsupportedError", "BuildError"), r.stdout


def test_compiler_and_oracle_agree_on_generated_expressions(gbc):
    # Seeded random expressions of the subset (interp_replay.random_expression)
    # over random element types: the library's compiler and the oracle's
    # independent parser must accept and reject the same texts (the compiler
    # may also refuse programs beyond its 48 operations or 4 temporaries as
    # UNSUPPORTED).
    import random

    import interp_replay as R

    rng = random.Random(2024)
    types = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64, np.float32,
             np.float64]
    seen = {"ok": 0, "build": 0}
    for _ in range(20000):
        has_y = rng.random() < 0.5
        tx, to = rng.choice(types), rng.choice(types)
        ty = rng.choice(types) if has_y else None
        expr = R.random_expression(rng, rng.randint(1, 5), has_y)
        try:
            gbc.transform_compile(expr, tx, to, ty)
            lib = "ok"
        except gbc.BuildError:
            lib = "build"
        except gbc.UnsupportedError:
            continue
        try:
            T.transform(expr, np.zeros(2, dtype=tx), to, np.zeros(2, dtype=ty) if has_y else None)
            orc = "ok"
        except SyntaxError:
            orc = "build"
        assert lib == orc, (expr, np.dtype(tx).name, np.dtype(ty).name if ty else None, np.dtype(to).name)
        seen[lib] += 1
    assert seen["ok"] > 8000 and seen["build"] > 4000


def test_compiler_refuses_oversized_text_quickly(gbc):
    # 10 MB of text is refused before lexing, and the message quotes only
    # the start of it
    import time

    text = "x+" * 5_000_000 + "x"
    t0 = time.perf_counter()
    with pytest.raises(gbc.UnsupportedError) as e:
        gbc.transform_compile(text, np.int32, np.int32)
    assert time.perf_counter() - t0 < 2.0
    assert len(str(e.value)) < 1000
