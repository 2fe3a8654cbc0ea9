"""CPU ORACLE for transform / transform2 — test infrastructure only.

Evaluates an OpenCL C element-wise expression over numpy arrays the way the
reference's kernels clc_transform / clc_transform2 do
(lib/src/Compute/Algorithm.cpp:30-56: `const T_IN x = in[i]; out[i] =
(T_OUT)(EXPR)`, host side 361-398; x and y per lib/Compute.md:39-41), with
OpenCL C's typing: integer promotion of char/short, the usual arithmetic
conversions, int 0/1 results of comparisons and logic, shift counts masked to
the left operand's width, abs of an integer giving its unsigned type. Where
OpenCL C leaves a result undefined this oracle fixes it the same way the
library documents: integer x / 0 and x % 0 give 0, INT_MIN / -1 wraps,
float -> integer conversion truncates and saturates (NaN -> 0), min/max/fmin/
fmax of a NaN give the other operand. Float arithmetic is numpy's IEEE
float32 / float64 (round to nearest, no fused multiply-add).

A second, independent implementation of the expression language (its own
tokenizer, parser and typing) used only by tests/ to check results. Float
literals with an f suffix are read through a double (the literals the tests
use are exact or far from a rounding tie). Raises SyntaxError for malformed
text and NotImplementedError for constructs outside the supported subset.
"""
from __future__ import annotations

import re

import numpy as np

I8, U8, I16, U16, I32, U32, I64, U64, F32, F64 = (np.dtype(t) for t in (
    np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64, np.float32, np.float64))

_TYPE_NAMES = {
    "char": I8, "uchar": U8, "short": I16, "ushort": U16, "int": I32, "uint": U32, "long": I64, "ulong": U64,
    "float": F32, "double": F64, "size_t": U64,
    "unsigned char": U8, "unsigned short": U16, "unsigned int": U32, "unsigned long": U64, "unsigned": U32,
    "signed char": I8, "signed short": I16, "signed int": I32, "signed long": I64, "signed": I32,
}


def _promote(t):
    return I32 if t.itemsize < 4 else t


def _usual(a, b):
    """C99 6.3.1.8 with 32-bit int and 64-bit long."""
    if F64 in (a, b):
        return F64
    if F32 in (a, b):
        return F32
    a, b = _promote(a), _promote(b)
    if a == b:
        return a
    ua, ub = a.kind == "u", b.kind == "u"
    if ua == ub:
        return a if a.itemsize >= b.itemsize else b
    u, s = (a, b) if ua else (b, a)
    if u.itemsize >= s.itemsize:
        return u
    return s  # the signed type is wider: it holds every value of the unsigned one


def convert(v: np.ndarray, to: np.dtype) -> np.ndarray:
    """C conversion of array v to type `to` (floats to integers: truncation,
    saturating, NaN -> 0)."""
    to = np.dtype(to)
    if v.dtype == to:
        return v
    with np.errstate(all="ignore"):
        if to.kind == "f":
            return v.astype(to)
        if v.dtype.kind == "f":
            info = np.iinfo(to)
            hi = float(2 ** (info.bits - 1)) if to.kind == "i" else float(2 ** info.bits)
            lo = -hi if to.kind == "i" else 0.0
            nan = np.isnan(v)
            over = v >= hi
            under = v < lo if to.kind == "i" else v <= -1.0
            safe = np.where(nan | over | under, 0, np.trunc(v)).astype(to)
            safe = np.where(over, info.max, safe).astype(to)
            if to.kind == "i":
                safe = np.where(under, info.min, safe).astype(to)
            return safe
        if to.kind in "iu" and v.dtype.kind in "iu":
            # modular: reinterpret through the unsigned view of the wider type
            wide = v.astype(np.int64) if v.dtype.kind == "i" else v.astype(np.uint64)
            return wide.astype(to)
    raise TypeError(f"cannot convert {v.dtype} to {to}")


class _Val:
    """A typed array (C type `t`); narrow types are stored in their own dtype."""

    def __init__(self, a, t, boolean=False):
        self.t = np.dtype(t)
        self.a = np.asarray(a, dtype=self.t)
        self.boolean = boolean

    def as_(self, t):
        return convert(self.a, t)


_TOKEN = re.compile(r"\s*(?:(?P<num>(?:0[xX][0-9a-fA-F]+|\d+\.?\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)"
                    r"[uUlLfF]*)|(?P<id>[A-Za-z_]\w*)|(?P<op><<|>>|<=|>=|==|!=|&&|\|\||[-+*/%&|^~!<>()?:,]))")


def _tokens(text):
    pos, out = 0, []
    text = text.rstrip()
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            raise SyntaxError(f"build log: unexpected character at {pos} in {text!r}")
        kind = m.lastgroup
        out.append((kind, m.group(kind)))
        pos = m.end()
    out.append(("end", ""))
    return out


class _Parser:
    LEVELS = [["||"], ["&&"], ["|"], ["^"], ["&"], ["==", "!="], ["<", ">", "<=", ">="], ["<<", ">>"],
              ["+", "-"], ["*", "/", "%"]]

    def __init__(self, text, x, y):
        self.toks = _tokens(text)
        self.i = 0
        self.x, self.y = x, y
        self.n = x.a.shape[0]

    def peek(self, k=0):
        return self.toks[min(self.i + k, len(self.toks) - 1)]

    def take(self, s=None):
        t = self.peek()
        if s is not None and t[1] != s:
            raise SyntaxError(f"build log: expected {s!r}, got {t[1]!r}")
        self.i += 1
        return t

    def full(self, value, t):
        return _Val(np.full(self.n, value, dtype=np.dtype(t)), t)

    # ---- grammar ----
    def parse(self):
        if self.peek()[0] == "end":
            raise SyntaxError("build log: empty expression")
        v = self.cond()
        if self.peek()[0] != "end":
            raise SyntaxError(f"build log: trailing {self.peek()[1]!r}")
        return v

    def cond(self):
        c = self.binary(0)
        if self.peek()[1] != "?":
            return c
        self.take("?")
        a = self.cond()
        self.take(":")
        b = self.cond()
        t = _usual(a.t, b.t)
        truth = self._truth(c)
        return _Val(np.where(truth != 0, a.as_(t), b.as_(t)), t)

    def binary(self, level):
        if level == len(self.LEVELS):
            return self.unary()
        v = self.binary(level + 1)
        while self.peek()[0] == "op" and self.peek()[1] in self.LEVELS[level]:
            op = self.take()[1]
            w = self.binary(level + 1)
            v = self.apply(op, v, w)
        return v

    def _truth(self, v):
        return (v.a != 0).astype(np.int32)

    def apply(self, op, v, w):
        with np.errstate(all="ignore"):
            if op in ("&&", "||"):
                a, b = self._truth(v), self._truth(w)
                return _Val((a & b) if op == "&&" else (a | b), I32, True)
            if op in ("<<", ">>"):
                if v.t.kind == "f" or w.t.kind == "f":
                    raise SyntaxError("build log: shift of a floating-point operand")
                t = _promote(v.t)
                a = v.as_(t)
                bits = t.itemsize * 8
                count = convert(w.a, t).astype(np.uint64) & np.uint64(bits - 1)
                ut = np.dtype(f"u{t.itemsize}")
                if op == "<<":
                    r = (a.view(ut).astype(np.uint64) << count).astype(ut).view(t)
                else:
                    r = (a >> count.astype(t)) if t.kind == "i" else (a.astype(np.uint64) >> count).astype(t)
                return _Val(r, t)
            t = _usual(v.t, w.t)
            a, b = v.as_(t), w.as_(t)
            if op in ("==", "!=", "<", ">", "<=", ">="):
                r = {"==": a == b, "!=": a != b, "<": a < b, ">": a > b, "<=": a <= b, ">=": a >= b}[op]
                return _Val(r.astype(np.int32), I32, True)
            if op in ("%", "&", "|", "^") and t.kind == "f":
                raise SyntaxError(f"build log: invalid operands to {op}")
            if op == "+":
                return _Val(a + b, t)
            if op == "-":
                return _Val(a - b, t)
            if op == "*":
                return _Val(a * b, t)
            if op == "&":
                return _Val(a & b, t)
            if op == "|":
                return _Val(a | b, t)
            if op == "^":
                return _Val(a ^ b, t)
            if op in ("/", "%"):
                if t.kind == "f":
                    return _Val(a / b, t)
                return _Val(self._divmod(a, b, t, op == "/"), t)
        raise SyntaxError(f"build log: operator {op}")

    @staticmethod
    def _divmod(a, b, t, want_quotient):
        """C division truncating toward zero; x/0 -> 0, x%0 -> 0, MIN/-1 wraps."""
        zero = b == 0
        if t.kind == "u":
            bs = np.where(zero, 1, b).astype(t)
            q = (a // bs).astype(t)
            r = (a % bs).astype(t)
        else:
            neg1 = b == -1
            bs = np.where(zero | neg1, 1, b).astype(t)
            ua = np.abs(a.astype(np.int64)).astype(np.uint64) if t.itemsize < 8 else \
                np.where(a < 0, (~a.view(np.uint64)) + np.uint64(1), a.view(np.uint64))
            ub = np.abs(bs.astype(np.int64)).astype(np.uint64) if t.itemsize < 8 else \
                np.where(bs < 0, (~bs.view(np.uint64)) + np.uint64(1), bs.view(np.uint64))
            uq = ua // ub
            ur = ua % ub
            sign_q = (a < 0) != (bs < 0)
            q = np.where(sign_q, (~uq) + np.uint64(1), uq).astype(t)  # modular negate, then narrow
            r = np.where(a < 0, (~ur) + np.uint64(1), ur).astype(t)
            q = np.where(neg1, (np.zeros_like(a) - a).astype(t), q).astype(t)
            r = np.where(neg1, 0, r).astype(t)
        q = np.where(zero, 0, q).astype(t)
        r = np.where(zero, 0, r).astype(t)
        return q if want_quotient else r

    def type_name(self):
        k, s = self.peek()
        if k != "id":
            return None
        if s in ("unsigned", "signed"):
            k2, s2 = self.peek(1)
            if k2 == "id" and s2 in ("char", "short", "int", "long"):
                return s + " " + s2, 2
            return s, 1
        if s in _TYPE_NAMES:
            return s, 1
        return None

    def unary(self):
        k, s = self.peek()
        if k == "op" and s in ("+", "-", "~", "!"):
            self.take()
            v = self.unary()
            with np.errstate(all="ignore"):
                if s == "!":
                    return _Val((v.a == 0).astype(np.int32), I32, True)
                t = _promote(v.t)
                a = v.as_(t)
                if s == "+":
                    return _Val(a, t)
                if s == "-":
                    return _Val(-a if t.kind == "f" else (np.zeros_like(a) - a).astype(t), t)
                if t.kind == "f":
                    raise SyntaxError("build log: ~ of a floating-point operand")
                return _Val(~a, t)
        if k == "op" and s == "(":
            save = self.i
            self.take("(")
            tn = self.type_name()
            if tn is not None and self.peek(tn[1])[1] == ")":
                for _ in range(tn[1]):
                    self.take()
                self.take(")")
                v = self.unary()
                return self.cast(v, _TYPE_NAMES[tn[0]])
            self.i = save
        return self.primary()

    def cast(self, v, t):
        t = np.dtype(t)
        if t.itemsize < 4 and v.t.kind == "f":
            return _Val(convert(v.as_(I32), t), t)  # through int (saturating), then modulo
        return _Val(v.as_(t), t)

    def args(self, count, name):
        self.take("(")
        out = []
        if self.peek()[1] != ")":
            out.append(self.cond())
            while self.peek()[1] == ",":
                self.take(",")
                out.append(self.cond())
        self.take(")")
        if len(out) != count:
            raise SyntaxError(f"build log: {name} takes {count} arguments")
        return out

    @staticmethod
    def _minmax(a, b, t, is_min):
        if t.kind == "f":
            pick = (b < a) if is_min else (a < b)
            r = np.where(pick, b, a)
            r = np.where(np.isnan(b), a, r)
            return np.where(np.isnan(a), b, r).astype(t)
        return (np.minimum(a, b) if is_min else np.maximum(a, b)).astype(t)

    def call(self, name):
        if name in ("min", "max", "fmin", "fmax"):
            a, b = self.args(2, name)
            if name[0] == "f" and (a.t.kind != "f" or b.t.kind != "f"):
                raise SyntaxError("build log: ambiguous call")
            t = a.t if a.t == b.t else _usual(a.t, b.t)
            at = _promote(t)
            r = self._minmax(a.as_(at), b.as_(at), at, name.endswith("min"))
            return _Val(convert(r, t), t)
        if name == "clamp":
            v, lo, hi = self.args(3, name)
            t = v.t if (lo.t == v.t and hi.t == v.t) else _usual(_usual(v.t, lo.t), hi.t)
            at = _promote(t)
            r = self._minmax(v.as_(at), lo.as_(at), at, False)
            r = self._minmax(r, hi.as_(at), at, True)
            return _Val(convert(r, t), t)
        if name in ("abs", "fabs"):
            (v,) = self.args(1, name)
            if (name == "abs") != (v.t.kind in "iu"):
                raise SyntaxError(f"build log: no {name} for {v.t}")
            if name == "fabs":
                return _Val(np.abs(v.a), v.t)
            ut = np.dtype(f"u{v.t.itemsize}")
            with np.errstate(all="ignore"):
                if v.t.kind == "i":
                    r = np.where(v.a < 0, (np.zeros_like(v.a) - v.a), v.a).astype(v.t).view(ut)
                else:
                    r = v.a
            return _Val(r, ut)
        m = re.fullmatch(r"(as|convert)_(char|uchar|short|ushort|int|uint|long|ulong|float|double)", name)
        if m:
            (v,) = self.args(1, name)
            t = _TYPE_NAMES[m.group(2)]
            if m.group(1) == "convert":
                return self.cast(v, t)
            if v.t.itemsize != t.itemsize:
                raise SyntaxError("build log: as_ of a different size")
            return _Val(v.a.view(t), t)
        if name in ("sqrt", "exp", "log", "sin", "cos", "pow", "mad", "fma", "select"):
            raise NotImplementedError(name)
        raise SyntaxError(f"build log: implicit declaration of {name}")

    def literal(self, s):
        is_hex = s[:2].lower() == "0x"
        m = re.fullmatch(r"(0[xX][0-9a-fA-F]+)([uUlL]*)" if is_hex else r"(.*?)([uUlLfF]*)", s)
        digits, suf = m.group(1), m.group(2).lower()
        if not is_hex and (any(c in digits for c in ".eE") or "f" in suf):
            if "f" in suf:
                return self.full(np.float32(float(digits)), F32)
            return self.full(float(digits), F64)
        v = int(digits, 16) if is_hex else (int(digits, 8) if len(digits) > 1 and digits[0] == "0" else int(digits))
        u, l_ = "u" in suf, "l" in suf
        decimal = not (len(digits) > 1 and digits[0] == "0")
        if not u and not l_ and v <= 0x7FFFFFFF:
            t = I32
        elif not l_ and (u or not decimal) and v <= 0xFFFFFFFF:
            t = U32
        elif not u and v <= 0x7FFFFFFFFFFFFFFF:
            t = I64
        else:
            t = U64
        return self.full(v, t)

    CONSTANTS = {
        "INT_MAX": (2**31 - 1, I32), "INT_MIN": (-2**31, I32), "UINT_MAX": (2**32 - 1, U32),
        "LONG_MAX": (2**63 - 1, I64), "LONG_MIN": (-2**63, I64), "ULONG_MAX": (2**64 - 1, U64),
        "CHAR_MAX": (127, I32), "CHAR_MIN": (-128, I32), "UCHAR_MAX": (255, I32), "SHRT_MAX": (32767, I32),
        "SHRT_MIN": (-32768, I32), "USHRT_MAX": (65535, I32), "CHAR_BIT": (8, I32),
        "FLT_MAX": (np.finfo(np.float32).max, F32), "MAXFLOAT": (np.finfo(np.float32).max, F32),
        "FLT_MIN": (np.finfo(np.float32).tiny, F32), "FLT_EPSILON": (np.finfo(np.float32).eps, F32),
        "DBL_MAX": (np.finfo(np.float64).max, F64), "DBL_MIN": (np.finfo(np.float64).tiny, F64),
        "DBL_EPSILON": (np.finfo(np.float64).eps, F64), "INFINITY": (np.inf, F32), "HUGE_VALF": (np.inf, F32),
        "HUGE_VAL": (np.inf, F64), "NAN": (np.nan, F32),
    }

    def primary(self):
        k, s = self.take()
        if k == "num":
            return self.literal(s)
        if k == "id":
            if self.peek()[1] == "(":
                return self.call(s)
            if s == "x":
                return self.x
            if s == "y" and self.y is not None:
                return self.y
            if s in self.CONSTANTS:
                v, t = self.CONSTANTS[s]
                return self.full(v, t)
            raise SyntaxError(f"build log: undeclared identifier {s}")
        if s == "(":
            v = self.cond()
            self.take(")")
            return v
        raise SyntaxError(f"build log: unexpected {s!r}")


def transform(expression: str, x: np.ndarray, out_dtype, y: np.ndarray | None = None) -> np.ndarray:
    """out[i] = (out_dtype)(expression) with x = x[i] (and y = y[i])."""
    xv = _Val(x, x.dtype)
    yv = _Val(y, y.dtype) if y is not None else None
    v = _Parser(expression, xv, yv).parse()
    out = np.dtype(out_dtype)
    if out.itemsize < 4 and v.t.kind == "f":
        return convert(convert(v.a, I32), out)
    return convert(v.a, out)


def truth(expression: str, x: np.ndarray) -> np.ndarray:
    """The reference's copy_if flag `(PRED) ? 1u : 0u`: the expression over
    x = x[i] is nonzero in its own type (NaN counts as nonzero)."""
    v = _Parser(expression, _Val(x, x.dtype), None).parse()
    return v.a != 0
