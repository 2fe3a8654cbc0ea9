"""Test infrastructure: replays a compiled transform program (the listing that
clc_transform_compile prints) element by element in exact arithmetic, with
the device interpreter's rules, so that the compiler's code generation
(operand order, reversed operations, stack slots, conversions, selects) can
be checked on the CPU against the expression oracle.

The interpreter's rules (opencl-sdk_gb300/csrc/interp.cuh):
- values travel as raw bits; a 32-bit type uses the low 32 bits, and a 32-bit
  result is stored zero-extended;
- `x` / `y` are the element promoted to at least 32 bits (narrow signed types
  sign-extended to int, narrow unsigned ones zero-extended), and an `x`/`y`
  operand is reinterpreted in the operation's type, never converted;
- integer arithmetic wraps; `/ 0` and `% 0` give 0, a divisor of -1 negates
  (wrapping) and gives remainder 0; shift counts are masked to the width;
  `>>` is arithmetic for signed types;
- float arithmetic is IEEE round to nearest in the operation's type; `min` /
  `max` of a NaN give the other operand;
- comparisons give an int 0/1;
- `cvt.A->B` converts (float to integer: truncating, saturating, NaN -> 0);
- `ext8s` / `ext8u` / `ext16s` / `ext16u` re-extend the low bits to int;
- `sel stN` keeps the accumulator unless the low 32 bits of slot N are
  nonzero, then takes slot N+1;
- `divc` / `remc` divide by the immediate with the printed magic number;
- the store writes the low bytes of the result for the output element.
"""
from __future__ import annotations

import re

import numpy as np

import transform_oracle as T

TY = {"i32": np.int32, "u32": np.uint32, "i64": np.int64, "u64": np.uint64, "f32": np.float32, "f64": np.float64}
BITS = {"i32": 32, "u32": 32, "i64": 64, "u64": 64, "f32": 32, "f64": 64}
_LINE = re.compile(r"^(?P<kind>\w+)\.(?P<t>\w+?)(?:->(?P<t2>\w+))?(?: (?P<opd>#0x[0-9a-f]+|x|y|st\d+))?"
                   r"(?: m=0x(?P<m>[0-9a-f]+) l=(?P<l>\d+))?$")
_MASK = {32: (1 << 32) - 1, 64: (1 << 64) - 1}


def parse(listing: str):
    ops = []
    for line in listing.strip().split("\n"):
        mo = _LINE.match(line.strip())
        if mo is None:
            raise ValueError(f"unparsed listing line {line!r}")
        ops.append(mo.groupdict())
    return ops


def get(t: str, raw: int):
    """The value of type t held in raw bits."""
    b = BITS[t]
    r = raw & _MASK[b]
    if t in ("f32", "f64"):
        return np.array([r], dtype=np.uint32 if b == 32 else np.uint64).view(TY[t])[0]
    if t[0] == "i" and r >> (b - 1):
        r -= 1 << b
    return r


def put(t: str, v) -> int:
    """Raw bits (zero-extended) of value v of type t."""
    b = BITS[t]
    if t in ("f32", "f64"):
        return int(np.array([v], dtype=TY[t]).view(np.uint32 if b == 32 else np.uint64)[0])
    return int(v) & _MASK[b]


def promote_raw(v) -> int:
    """An element's raw register value (promoted to at least 32 bits)."""
    dt = np.asarray(v).dtype
    if dt.kind == "f":
        return int(np.array([v], dtype=dt).view(np.uint32 if dt.itemsize == 4 else np.uint64)[0])
    iv = int(v)
    if dt.itemsize < 4 and dt.kind == "i":
        return iv & _MASK[32]
    return iv & _MASK[64 if dt.itemsize == 8 else 32]


def _int_op(kind, t, a, b):
    bits, signed = BITS[t], t[0] == "i"
    wrap = lambda v: get(t, v & _MASK[bits])  # noqa: E731
    if kind in ("add", "sub", "mul", "and", "or", "xor"):
        return wrap({"add": a + b, "sub": a - b, "mul": a * b, "and": a & b, "or": a | b, "xor": a ^ b}[kind])
    if kind == "div":
        if b == 0:
            return 0
        if signed and b == -1:
            return wrap(-a)
        q = abs(a) // abs(b)
        return wrap(q if (a >= 0) == (b >= 0) else -q)
    if kind == "rem":
        if b == 0 or (signed and b == -1):
            return 0
        q = abs(a) // abs(b)
        q = q if (a >= 0) == (b >= 0) else -q
        return wrap(a - q * b)
    if kind in ("shl", "shr"):
        s = (b & _MASK[bits]) & (bits - 1)
        return wrap(a << s) if kind == "shl" else wrap(a >> s)  # Python >> on a signed value is arithmetic
    if kind in ("min", "max"):
        return (b if b < a else a) if kind == "min" else (b if a < b else a)
    raise ValueError(kind)


def _fp_op(kind, t, a, b):
    with np.errstate(all="ignore"):
        if kind == "add":
            return a + b
        if kind == "sub":
            return a - b
        if kind == "mul":
            return a * b
        if kind == "div":
            return a / b
    if kind == "min":
        return b if np.isnan(a) else (a if np.isnan(b) else (b if b < a else a))
    if kind == "max":
        return b if np.isnan(a) else (a if np.isnan(b) else (b if a < b else a))
    raise ValueError(kind)


_CMP = {"lt": lambda a, b: a < b, "le": lambda a, b: a <= b, "gt": lambda a, b: a > b, "ge": lambda a, b: a >= b,
        "eq": lambda a, b: a == b, "ne": lambda a, b: a != b}
_REVERSED = {"rsub": "sub", "rdiv": "div", "rrem": "rem", "rshl": "shl", "rshr": "shr"}


def _divc(t, n, d, m, l):
    bits, signed = BITS[t], t[0] == "i"
    if not signed:
        t1 = (m * n) >> bits
        sh1, sh2 = (1, l - 1) if l > 0 else (0, 0)
        return ((t1 + ((n - t1) >> sh1)) >> sh2) & _MASK[bits]
    ms = get(t, m)
    q = get(t, (n + ((ms * n) >> bits)) & _MASK[bits])
    q = (q >> (l - 1)) - (-1 if n < 0 else 0)
    ds = -1 if d < 0 else 0
    return get(t, ((q ^ ds) - ds) & _MASK[bits])


def run(ops, xr: int, yr: int | None) -> int:
    """The program's raw result for one element (raw promoted x and y)."""
    acc = 0
    slots = {}

    def operand(o, t):
        s = o["opd"]
        if s == "x":
            return get(t, xr)
        if s == "y":
            return get(t, yr)
        if s.startswith("#"):
            return get(t, int(s[3:], 16))
        return get(t, slots[int(s[2:])])

    for o in ops:
        kind, t = o["kind"], o["t"]
        if kind == "load":
            acc = {"x": xr, "y": yr}.get(o["opd"]) if o["opd"] in ("x", "y") else int(o["opd"][3:], 16)
            continue
        if kind == "push":
            slots[int(o["opd"][2:])] = acc
            continue
        if kind == "sel":
            k = int(o["opd"][2:])
            if slots[k] & _MASK[32]:
                acc = slots[k + 1]
            continue
        if kind == "cvt":
            src = np.array([get(t, acc)], dtype=TY[t])
            acc = put(o["t2"], T.convert(src, np.dtype(TY[o["t2"]]))[0])
            continue
        if kind.startswith("ext"):
            v = acc & (0xFF if kind.startswith("ext8") else 0xFFFF)
            w = 8 if kind.startswith("ext8") else 16
            if kind.endswith("s") and v >> (w - 1):
                v -= 1 << w
            acc = put("i32", v)
            continue
        a = get(t, acc)
        if kind in ("divc", "remc"):
            d = get(t, int(o["opd"][3:], 16))
            q = _divc(t, a, d, int(o["m"], 16), int(o["l"]))
            acc = put(t, q if kind == "divc" else get(t, (a - q * d) & _MASK[BITS[t]]))
            continue
        fp = t in ("f32", "f64")
        if kind in ("neg", "not", "abs"):
            if fp:
                acc = put(t, -a if kind == "neg" else np.abs(a))
            elif kind == "neg":
                acc = put(t, -a)
            elif kind == "not":
                acc = put(t, ~a)
            else:
                acc = put(t, -a if a < 0 else a)
            continue
        b = operand(o, t)
        if kind in _REVERSED:
            kind, a, b = _REVERSED[kind], b, a
        if kind in _CMP:
            acc = put("i32", 1 if _CMP[kind](a, b) else 0)
        elif fp:
            acc = put(t, _fp_op(kind, t, a, b))
        else:
            acc = put(t, _int_op(kind, t, a, b))
    return acc


def evaluate(listing: str, x: np.ndarray, out_dtype, y: np.ndarray | None = None) -> np.ndarray:
    """The kernel's output array for inputs x (and y)."""
    ops = parse(listing)
    out = np.dtype(out_dtype)
    raws = [run(ops, promote_raw(x[i]), promote_raw(y[i]) if y is not None else None) for i in range(x.size)]
    width = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[out.itemsize]
    mask = (1 << (8 * out.itemsize)) - 1
    return np.array([r & mask for r in raws], dtype=width).view(out)


# ---- seeded random expressions of the supported subset ----

CASTS = ["char", "uchar", "short", "ushort", "int", "uint", "long", "ulong", "float", "double"]
LITERALS = ["0", "1", "3", "7u", "255", "1000000", "3000000000", "5L", "2ul", "0x7f", "0xffffffffu", "1.5f", "0.5",
            "2.0f", "-1", "INT_MAX", "UINT_MAX", "FLT_MAX", "NAN", "INFINITY"]
BINOPS = ["+", "-", "*", "/", "%", "&", "|", "^", "<<", ">>", "<", ">", "<=", ">=", "==", "!=", "&&", "||"]


def random_expression(rng, depth: int, has_y: bool) -> str:
    """A random expression over x (and y) with literals of every kind,
    binary and unary operators, casts, ternaries, as_T / convert_T and
    min/max/clamp/abs/fabs/fmin/fmax calls (not all well typed: some must be
    refused)."""
    def gen(d):
        if d <= 0 or rng.random() < 0.25:
            return rng.choice(["x", "y"] if has_y else ["x"]) if rng.random() < 0.6 else rng.choice(LITERALS)
        r = rng.random()
        if r < 0.45:
            return f"({gen(d - 1)} {rng.choice(BINOPS)} {gen(d - 1)})"
        if r < 0.55:
            return rng.choice(["-", "~", "!", "+"]) + f"({gen(d - 1)})"
        if r < 0.65:
            return f"({rng.choice(CASTS)})({gen(d - 1)})"
        if r < 0.72:
            return f"({gen(d - 1)} ? {gen(d - 1)} : {gen(d - 1)})"
        if r < 0.78:
            return f"{rng.choice(['as_', 'convert_'])}{rng.choice(CASTS)}({gen(d - 1)})"
        f = rng.choice(["min", "max", "abs", "fabs", "fmin", "fmax", "clamp"])
        if f in ("abs", "fabs"):
            return f"{f}({gen(d - 1)})"
        if f == "clamp":
            return f"clamp({gen(d - 1)}, {gen(d - 1)}, {gen(d - 1)})"
        return f"{f}({gen(d - 1)}, {gen(d - 1)})"

    return gen(depth)


def sample_values(rng, dtype, n: int) -> np.ndarray:
    """n values of dtype: random ones and the type's edge values."""
    dt = np.dtype(dtype)
    if dt.kind == "f":
        specials = [0.0, -0.0, 1.0, -1.0, 1.5, -2.5, 255.7, 3e9, -3e9, 1e30, -1e30, np.inf, -np.inf, np.nan]
        v = [rng.choice([rng.uniform(-1e3, 1e3), rng.uniform(-1e10, 1e10), float(rng.randint(-300, 300))])
             for _ in range(n)]
    else:
        info = np.iinfo(dt)
        specials = [0, 1, info.max, info.min] + ([-1, info.min + 1] if dt.kind == "i" else [info.max - 1])
        v = [rng.randint(int(info.min), int(info.max)) if rng.random() < 0.7 else rng.randint(-20, 20) % (int(info.max) + 1)
             if dt.kind == "u" else rng.randint(-20, 20) for _ in range(n)]
    out = np.array(v[: n - len(specials)] + specials, dtype=np.float64 if dt.kind == "f" else object)
    return out.astype(dt)
