"""Generates tests/golden/reference_recipes.json from the CPU oracle.

The fixtures restate the reference's own test recipes (lib/test/Compute/
main.cpp and capi.c) — inputs from std::mt19937 + uniform distributions with
the same sizes and seeds — and record the expected outputs, computed by the
oracle's std:: layer, as SHA-256 digests (large arrays) or literal values
(small ones). GPU tests compare libgbcompute's outputs against these records;
tests/test_oracle.py checks that both oracle layers reproduce them.

Run: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

SIZES = [0, 1, 7, 255, 256, 1000, 4097, 100003, 1 << 20]  # main.cpp:54


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def capi_host(n: int = 10007) -> np.ndarray:
    # capi.c:103-108: host[i] = (int32_t)((i * 7919u) % 1000u) - 500
    i = np.arange(n, dtype=np.uint64)
    return (((i * 7919) % 1000).astype(np.int64) - 500).astype(np.int32)


def make() -> dict:
    out: dict = {"sizes": SIZES}

    # std::mt19937 default-seed property from the C++ standard: the 10000th
    # output of mt19937(5489) is 4123659995; with the full uint32 range
    # libstdc++'s uniform_int_distribution passes engine output through.
    out["mt19937_5489_10000th"] = int(oracle.random_uints(10000, 0xFFFFFFFF, 5489)[9999])

    sort = {}
    for n in SIZES:  # main.cpp:248-272: sort_by_key, values = index, seed n + 2
        keys = oracle.random_uints(n, 0xFFFFFFFF, n + 2)
        k, v = oracle.std_sort(keys, np.arange(n, dtype=np.uint32))
        sort[str(n)] = {"keys_in": digest(keys), "keys": digest(k), "values": digest(v)}
    out["sort_by_key"] = sort

    dup = oracle.random_uints(50000, 15, 99)  # main.cpp:274-287
    k, v = oracle.std_sort(dup, np.arange(dup.size, dtype=np.uint32))
    out["stability"] = {"keys_in": digest(dup), "keys": digest(k), "values": digest(v)}

    ints = np.array([5, -3, 0, -(2**31), 7, -1, 2**31 - 1, 2], dtype=np.int32)  # main.cpp:290-295
    out["signed"] = {"keys_in": ints.tolist(), "sorted": sorted(ints.tolist())}

    floats = oracle.random_floats(3000, -1e6, 1e6, 5)  # main.cpp:297-311
    floats[0], floats[1], floats[2] = np.float32(-0.0), np.float32(np.inf), np.float32(-np.inf)
    fk, _ = oracle.std_sort(floats, None, descending=True)
    out["floats_desc"] = {"keys_in": digest(floats), "sorted_bits": digest(fk.view(np.uint32)),
                          "head": [float(x) for x in fk[:3]], "tail": [float(x) for x in fk[-3:]]}

    scan = {}
    for n in SIZES:  # main.cpp:209-229: seed n + 1, values <= 100
        x = oracle.random_uints(n, 100, n + 1)
        scan[str(n)] = {"in": digest(x), "inclusive": digest(oracle.std_scan(x)),
                        "exclusive": digest(oracle.std_scan(x, exclusive=True))}
    out["scan"] = scan
    v = (np.arange(5000, dtype=np.int64) * 7 % 101).astype(np.int32)  # main.cpp:233-243
    out["scan_right_projection"] = {"in": digest(v), "inclusive": digest(oracle.std_scan(v, oracle.OP_RIGHT, 0))}
    out["scan_max"] = {"inclusive": digest(oracle.std_scan(v, oracle.OP_MAX, -(2**31)))}

    red = {}
    for n in SIZES:  # main.cpp:184-199: seed n, values <= 1000, init 7
        x = oracle.random_uints(n, 1000, n)
        entry = {"sum_init7": int(oracle.std_reduce(x, oracle.OP_PLUS, 0, 7))}
        if n:
            entry["max"] = int(x.max())
            entry["min"] = int(x.min())
        red[str(n)] = entry
    out["reduce"] = red

    hist = {}
    for n in SIZES:  # main.cpp:314-336: seed n + 3, 10 bins over [0, 1000)
        x = oracle.random_uints(n, 1000, n + 3)
        hist[str(n)] = oracle.histogram_even(x, 10, 0.0, 1000.0).tolist()
    out["histogram10"] = hist

    h = capi_host()  # capi.c:103-141
    s = int(h.astype(np.int64).sum())
    out["capi"] = {"n": int(h.size), "sum_i64": s, "sum_i32": ((s + 2**31) % 2**32) - 2**31,
                   "max": int(h.max()), "positives": int((h > 0).sum())}
    return out


if __name__ == "__main__":
    data = make()
    path = os.path.join(HERE, "reference_recipes.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print("wrote", path, os.path.getsize(path), "bytes")
