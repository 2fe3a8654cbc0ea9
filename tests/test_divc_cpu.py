"""Division and remainder by an integer literal, without a GPU: the
transform compiler turns `x / d` and `x % d` (|d| >= 2) into a multiply-high
sequence whose magic number m and shift l it prints in the listing
(Granlund & Montgomery 1994, figures 4.1 unsigned and 5.2 signed). Here the
kernel's sequence is replayed in exact integer arithmetic for many divisors
of every integer width and checked against C's truncating division over
boundary and random dividends."""
import re

import numpy as np
import pytest


@pytest.fixture(scope="module")
def gbc():
    import gbcompute

    return gbcompute


TYPES = {  # numpy type: (bits, signed)
    np.uint32: (32, False),
    np.int32: (32, True),
    np.uint64: (64, False),
    np.int64: (64, True),
}


def wrap(v, bits, signed):
    v &= (1 << bits) - 1
    if signed and v >> (bits - 1):
        v -= 1 << bits
    return v


def c_div(n, d):  # C: truncation toward zero
    q = abs(n) // abs(d)
    return q if (n >= 0) == (d >= 0) else -q


def replay(n, d, m, l, bits, signed):
    """The kernel's quotient for dividend n (interp.cuh exec_divc)."""
    if not signed:
        t1 = (m * n) >> bits
        sh1, sh2 = (1, l - 1) if l > 0 else (0, 0)
        return ((t1 + ((n - t1) >> sh1)) >> sh2) & ((1 << bits) - 1)
    ms = wrap(m, bits, True)
    q = wrap(n + ((ms * n) >> bits), bits, True)  # MULSH: high half of the signed product
    q = (q >> (l - 1)) - (-1 if n < 0 else 0)
    ds = -1 if d < 0 else 0
    return wrap((q ^ ds) - ds, bits, True)


def divisors(bits, signed):
    top = (1 << (bits - 1)) - 1 if signed else (1 << bits) - 1
    ds = set(range(2, 130)) | {1000, 1000000007, 641, 6700417, 274177}
    for k in range(2, bits - (1 if signed else 0)):
        ds |= {(1 << k) - 1, 1 << k, (1 << k) + 1}
    ds |= {top, top - 1, top // 3, top // 7 + 1}
    ds = {d for d in ds if 2 <= d <= top}
    if signed:  # the most negative value is not a literal (C writes it as an expression)
        ds |= {-d for d in list(ds)}
    return sorted(ds)


def literal(d, bits, signed):
    # suffixes keep the literal in the operand's type (an unsuffixed decimal
    # above INT_MAX is a long, which would widen a uint division to long)
    if not signed:
        return f"{d}ul" if bits == 64 else f"{d}u"
    return f"({d})" if d < 0 else str(d)


def dividends(d, bits, signed, rng):
    lo, hi = (-(1 << (bits - 1)), (1 << (bits - 1)) - 1) if signed else (0, (1 << bits) - 1)
    base = {0, 1, 2, lo, lo + 1, hi, hi - 1}
    for k in (1, 2, 3):
        base |= {k * d - 1, k * d, k * d + 1, -k * d - 1, -k * d, -k * d + 1}
    vals = [v for v in base if lo <= v <= hi]
    vals += [int(v) for v in rng.integers(lo, hi, size=200, dtype=np.int64 if signed else np.uint64, endpoint=True)]
    return vals


@pytest.mark.parametrize("ty", list(TYPES), ids=lambda t: np.dtype(t).name)
@pytest.mark.parametrize("op", ["/", "%"])
def test_literal_division_magic(gbc, ty, op):
    bits, signed = TYPES[ty]
    rng = np.random.default_rng(bits * 2 + signed)
    checked = 0
    for d in divisors(bits, signed):
        text = gbc.transform_compile(f"x {op} {literal(d, bits, signed)}", ty, ty)
        mo = re.search(r"(divc|remc)\.(\w+) #0x([0-9a-f]+) m=0x([0-9a-f]+) l=(\d+)", text)
        assert mo is not None, text
        assert mo.group(1) == ("divc" if op == "/" else "remc")
        assert mo.group(2) == ("i" if signed else "u") + str(bits), text  # no widening
        assert wrap(int(mo.group(3), 16), bits, signed) == d
        m, l = int(mo.group(4), 16), int(mo.group(5))
        for n in dividends(d, bits, signed, rng):
            q = replay(n, d, m, l, bits, signed)
            q_ref = wrap(c_div(n, d), bits, signed) if signed else n // d
            if op == "/":
                assert q == q_ref, (d, n, m, l)
            else:
                r = wrap(n - q * d, bits, signed)
                assert r == wrap(n - q_ref * d, bits, signed), (d, n, m, l)
            checked += 1
    assert checked > 10000


@pytest.mark.parametrize("expr", ["x / 1", "x / 0", "x % 1"])
def test_small_divisors_are_not_magic(gbc, expr):
    # |d| < 2 keeps the plain operation (x / 0 is defined as 0 by the kernel)
    text = gbc.transform_compile(expr, np.int32, np.int32)
    assert "divc" not in text and "remc" not in text
