"""CPU ORACLE loader — test infrastructure only.

ctypes access to oracle/_build/liboracle.so (built from oracle.cpp by
oracle/Makefile). Used by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg to check results against; never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

T_I8, T_U8, T_I16, T_U16, T_I32, T_U32, T_I64, T_U64, T_F32, T_F64 = range(10)
OP_PLUS, OP_MUL, OP_AND, OP_OR, OP_XOR, OP_MIN, OP_MAX, OP_RIGHT = range(8)

_TYPES = {
    np.dtype(np.int8): T_I8, np.dtype(np.uint8): T_U8, np.dtype(np.int16): T_I16,
    np.dtype(np.uint16): T_U16, np.dtype(np.int32): T_I32, np.dtype(np.uint32): T_U32,
    np.dtype(np.int64): T_I64, np.dtype(np.uint64): T_U64, np.dtype(np.float32): T_F32,
    np.dtype(np.float64): T_F64,
}

# Operator expressions (as the C ABI spells them) -> oracle op codes.
OPS = {
    "(a + b)": OP_PLUS, "(a * b)": OP_MUL, "(a & b)": OP_AND, "(a | b)": OP_OR,
    "(a ^ b)": OP_XOR, "((b < a) ? b : a)": OP_MIN, "((a < b) ? b : a)": OP_MAX, "b": OP_RIGHT,
}


def build() -> str:
    newest = max(os.path.getmtime(os.path.join(HERE, f)) for f in ("oracle.cpp", "Makefile"))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, sz, i = C.c_void_p, C.c_size_t, C.c_int
        L.orc_random_uints.argtypes = [vp, sz, C.c_uint32, C.c_uint]
        L.orc_random_floats.argtypes = [vp, sz, C.c_float, C.c_float, C.c_uint]
        L.orc_std_sort.argtypes = [vp, vp, sz, i, i, i]
        L.orc_std_scan.argtypes = [vp, vp, sz, i, i, vp, i]
        L.orc_std_reduce.argtypes = [vp, sz, i, i, vp, vp, vp]
        L.orc_sum_i32.argtypes = [vp, sz]
        L.orc_sum_i32.restype = C.c_longlong
        L.orc_histogram_even.argtypes = [vp, sz, i, vp, sz, C.c_double, C.c_double, i]
        L.orc_ref_radix_sort.argtypes = [vp, vp, sz, i, i, i, i]
        L.orc_ref_scan.argtypes = [vp, vp, sz, i, i, vp, i, i]
        L.orc_ref_reduce.argtypes = [vp, sz, i, i, vp, vp, vp, i]
        L.orc_hardware_threads.restype = i
        L.orc_std_segmented_sort.argtypes = [vp, vp, sz, i, i, i, vp, sz, i]
        L.orc_std_segmented_scan.argtypes = [vp, vp, sz, i, i, vp, i, vp, sz]
        L.orc_mlp_grad.argtypes = [vp, vp, C.c_float, vp, vp, sz, i, vp, C.POINTER(C.c_double)]
        L.orc_std_reduce_by_key.argtypes = [vp, i, vp, sz, vp, vp, vp, vp]
        L.orc_std_reduce_by_key.restype = sz
        L.orc_bitpack_compress.argtypes = [vp, sz, sz, i, vp]
        L.orc_bitpack_compress.restype = sz
        L.orc_bitpack_decompress.argtypes = [vp, sz, sz, sz, i, vp]
        L.orc_bitpack_decompress.restype = i
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def key_kind(dtype) -> int:
    k = np.dtype(dtype).kind
    return {"u": 0, "i": 1, "f": 2}[k]


# ---- generators ---------------------------------------------------------------

def random_uints(n: int, maximum: int, seed: int) -> np.ndarray:
    """std::mt19937(seed) + uniform_int_distribution<uint32>(0, maximum)."""
    out = np.empty(n, dtype=np.uint32)
    lib().orc_random_uints(_p(out), n, maximum, seed)
    return out


def random_floats(n: int, lo: float, hi: float, seed: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    lib().orc_random_floats(_p(out), n, lo, hi, seed)
    return out


# ---- ground truth ---------------------------------------------------------------

def std_sort(keys: np.ndarray, values: np.ndarray | None = None, descending: bool = False):
    k = np.ascontiguousarray(keys).copy()
    v = None if values is None else np.ascontiguousarray(values, dtype=np.uint32).copy()
    lib().orc_std_sort(_p(k), None if v is None else _p(v), k.size, k.dtype.itemsize, key_kind(k.dtype),
                       int(descending))
    return k, v


def ref_radix_sort(keys: np.ndarray, values: np.ndarray | None = None, descending: bool = False,
                   threads: int = 0):
    k = np.ascontiguousarray(keys).copy()
    v = None if values is None else np.ascontiguousarray(values, dtype=np.uint32).copy()
    lib().orc_ref_radix_sort(_p(k), None if v is None else _p(v), k.size, k.dtype.itemsize, key_kind(k.dtype),
                             int(descending), threads)
    return k, v


def ref_radix_sort_inplace(keys: np.ndarray, values: np.ndarray | None = None, threads: int = 0) -> None:
    """The restated reference sort on the caller's own (contiguous) arrays,
    ascending: no copies, so a caller can time the sort alone."""
    assert keys.flags.c_contiguous and (values is None or (values.flags.c_contiguous and values.dtype == np.uint32))
    lib().orc_ref_radix_sort(_p(keys), None if values is None else _p(values), keys.size, keys.dtype.itemsize,
                             key_kind(keys.dtype), 0, threads)


def std_sort_inplace(keys: np.ndarray, values: np.ndarray | None = None) -> None:
    """std::stable_sort (one thread) on the caller's own arrays, ascending."""
    assert keys.flags.c_contiguous and (values is None or (values.flags.c_contiguous and values.dtype == np.uint32))
    lib().orc_std_sort(_p(keys), None if values is None else _p(values), keys.size, keys.dtype.itemsize,
                       key_kind(keys.dtype), 0)


def _ident(dtype, identity) -> np.ndarray:
    return np.array([identity], dtype=dtype)


def std_scan(x: np.ndarray, op: int = OP_PLUS, identity=0, exclusive: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    lib().orc_std_scan(_p(x), _p(out), x.size, _TYPES[x.dtype], op, _p(_ident(x.dtype, identity)), int(exclusive))
    return out


def ref_scan(x: np.ndarray, op: int = OP_PLUS, identity=0, exclusive: bool = False, threads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    lib().orc_ref_scan(_p(x), _p(out), x.size, _TYPES[x.dtype], op, _p(_ident(x.dtype, identity)), int(exclusive),
                       threads)
    return out


def std_reduce(x: np.ndarray, op: int = OP_PLUS, identity=0, init=0):
    x = np.ascontiguousarray(x)
    r = np.zeros(1, dtype=x.dtype)
    lib().orc_std_reduce(_p(x), x.size, _TYPES[x.dtype], op, _p(_ident(x.dtype, identity)),
                         _p(_ident(x.dtype, init)), _p(r))
    return r[0]


def ref_reduce(x: np.ndarray, op: int = OP_PLUS, identity=0, init=0, threads: int = 0):
    x = np.ascontiguousarray(x)
    r = np.zeros(1, dtype=x.dtype)
    lib().orc_ref_reduce(_p(x), x.size, _TYPES[x.dtype], op, _p(_ident(x.dtype, identity)),
                         _p(_ident(x.dtype, init)), _p(r), threads)
    return r[0]


def sum_i32(x: np.ndarray) -> int:
    x = np.ascontiguousarray(x, dtype=np.int32)
    return int(lib().orc_sum_i32(_p(x), x.size))


def histogram_even(x: np.ndarray, bins: int, lower: float, upper: float, threads: int = 0) -> np.ndarray:
    x = np.ascontiguousarray(x)
    h = np.zeros(bins, dtype=np.uint32)
    lib().orc_histogram_even(_p(x), x.size, _TYPES[x.dtype], _p(h), bins, lower, upper, threads)
    return h


def hardware_threads() -> int:
    return lib().orc_hardware_threads()


# ---- batched forms ----------------------------------------------------------

def std_segmented_sort(keys: np.ndarray, offsets: np.ndarray, values: np.ndarray | None = None,
                       descending: bool = False, threads: int = 0):
    k = np.ascontiguousarray(keys).copy()
    off = np.ascontiguousarray(offsets, dtype=np.uint32)
    v = None if values is None else np.ascontiguousarray(values, dtype=np.uint32).copy()
    lib().orc_std_segmented_sort(_p(k), None if v is None else _p(v), k.size, k.dtype.itemsize, key_kind(k.dtype),
                                 int(descending), _p(off), off.size - 1, threads)
    return k, v


def std_segmented_scan(x: np.ndarray, offsets: np.ndarray, op: int = OP_PLUS, identity=0,
                       exclusive: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x)
    off = np.ascontiguousarray(offsets, dtype=np.uint32)
    out = np.empty_like(x)
    lib().orc_std_segmented_scan(_p(x), _p(out), x.size, _TYPES[x.dtype], op, _p(_ident(x.dtype, identity)),
                                 int(exclusive), _p(off), off.size - 1)
    return out


def lognormal_segments(num_segments: int, median: float, sigma: float, lo: int, hi: int, seed: int) -> np.ndarray:
    """Offsets of segments whose lengths are round(lognormal(ln median, sigma)) clipped to [lo, hi]."""
    rng = np.random.default_rng(seed)
    lens = np.clip(np.rint(rng.lognormal(np.log(median), sigma, size=num_segments)), lo, hi).astype(np.int64)
    off = np.zeros(num_segments + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    return off.astype(np.uint32)


def mlp_grad(params: np.ndarray, centres: np.ndarray, inv_span: float, keys: np.ndarray, ys: np.ndarray,
             hidden: int = 32):
    """Gradient (raw parameters) and loss of the learned-CDF network, in double."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    c = np.ascontiguousarray(centres, dtype=np.uint32)
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    y = np.ascontiguousarray(ys, dtype=np.float32)
    g = np.zeros_like(p)
    loss = C.c_double(0)
    lib().orc_mlp_grad(_p(p), _p(c), C.c_float(inv_span), _p(k), _p(y), k.size, hidden, _p(g), C.byref(loss))
    return g, loss.value


def std_reduce_by_key(keys: np.ndarray, vals: np.ndarray):
    """(unique keys, uint64 sums, run lengths, 65536-bin histogram of key & 0xFFFF)."""
    k = np.ascontiguousarray(keys)
    v = np.ascontiguousarray(vals, dtype=np.uint32)
    ko = np.empty_like(k)
    sums = np.empty(k.size, dtype=np.uint64)
    counts = np.empty(k.size, dtype=np.uint32)
    hist = np.zeros(65536, dtype=np.uint32)
    r = lib().orc_std_reduce_by_key(_p(k), k.dtype.itemsize, _p(v), k.size, _p(ko), _p(sums), _p(counts), _p(hist))
    return ko[:r], sums[:r], counts[:r], hist


def zipf_keys(n: int, s: float, distinct: int, seed: int) -> np.ndarray:
    """Zipf(s) ranks over `distinct` values (inverse CDF), mapped to 64-bit keys by splitmix64 (a bijection)."""
    rng = np.random.default_rng(seed)
    w = 1.0 / np.arange(1, distinct + 1, dtype=np.float64) ** s
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    ranks = np.searchsorted(cdf, rng.random(n)).astype(np.uint64)
    z = ranks + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


# ---- bitpack compression (the reference's chunk format) ---------------------

def bitpack_compress(x: np.ndarray, chunk: int = 2048, delta: bool = False) -> np.ndarray:
    """The compressed words (3 header words per chunk, then the packed area)."""
    x = np.ascontiguousarray(x, dtype=np.uint32)
    words = lib().orc_bitpack_compress(_p(x), x.size, chunk, int(delta), None)
    out = np.zeros(words, dtype=np.uint32)
    if words:
        lib().orc_bitpack_compress(_p(x), x.size, chunk, int(delta), _p(out))
    return out


def bitpack_decompress(words: np.ndarray, n: int, chunk: int = 2048, delta: bool = False) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = np.zeros(n, dtype=np.uint32)
    if lib().orc_bitpack_decompress(_p(w), w.size, n, chunk, int(delta), _p(out)) != 0:
        raise ValueError("bitpack: corrupt chunk header")
    return out


def bitpack_recipes():
    """The reference's compression test inputs (lib/test/Compute/main.cpp:
    392-402) for every size of main.cpp:54, in its order: slowly increasing
    timestamps (one mt19937(11) shared across the sizes: t += rng() % 50 from
    1,700,000,000), small-range values (uniform [0, 300] + 5,000,000, seed
    n + 4) and incompressible noise (uniform 32-bit, seed n + 5)."""
    sizes = [0, 1, 7, 255, 256, 1000, 4097, 100003, 1 << 20]
    ts_all = mt19937_words(11, sum(sizes))
    out, used = [], 0
    for n in sizes:
        steps = (ts_all[used:used + n] % 50).astype(np.uint64)
        used += n
        ts = ((1700000000 + np.cumsum(steps)) & 0xFFFFFFFF).astype(np.uint32)
        small = (random_uints(n, 300, n + 4).astype(np.uint64) + 5000000).astype(np.uint32)
        noise = random_uints(n, 0xFFFFFFFF, n + 5)
        out.append((n, ts, small, noise))
    return out


def mt19937_words(seed: int, count: int) -> np.ndarray:
    """The first `count` raw outputs of std::mt19937(seed)."""
    return random_uints(count, 0xFFFFFFFF, seed)


# ---- static_map -----------------------------------------------------------------

def murmur_fmix32(k: np.ndarray) -> np.ndarray:
    """The MurmurHash3 32-bit finalizer (the hash of the reference's
    static_map, DeviceHeaders.cpp:136-145)."""
    k = np.asarray(k, dtype=np.uint64) & 0xFFFFFFFF
    k ^= k >> 16
    k = (k * 0x85EBCA6B) & 0xFFFFFFFF
    k ^= k >> 13
    k = (k * 0xC2B2AE35) & 0xFFFFFFFF
    k ^= k >> 16
    return k.astype(np.uint32)


def linear_probe_table_ok(slot_keys: np.ndarray, empty_key: int) -> bool:
    """True when every stored key is reachable by the linear-probing walk the
    reference's find makes (HashMap.cpp:45-58): from slot hash(key) & mask
    forward, no empty slot before the key's slot."""
    cap = slot_keys.size
    mask = cap - 1
    occupied = slot_keys != empty_key
    idx = np.nonzero(occupied)[0]
    home = murmur_fmix32(slot_keys[idx]).astype(np.int64) & mask
    # an empty slot on the cyclic walk home .. idx breaks the chain
    empty_pos = np.nonzero(~occupied)[0]
    if empty_pos.size == 0:
        return True
    dist = (idx - home) % cap
    # nearest empty slot at or after home, cyclically
    nxt = np.searchsorted(empty_pos, home)
    nearest = np.where(nxt < empty_pos.size, empty_pos[np.minimum(nxt, empty_pos.size - 1)], empty_pos[0] + cap)
    gap = nearest - home
    return bool(np.all(dist < gap))
