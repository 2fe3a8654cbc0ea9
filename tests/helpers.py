"""Small helpers shared by the test modules."""
import hashlib
import json
import os

import numpy as np

with open(os.path.join(os.path.dirname(__file__), "golden", "reference_recipes.json")) as _f:
    GOLDEN = json.load(_f)
SIZES = GOLDEN["sizes"]  # lib/test/Compute/main.cpp:54


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def stable_order(keys_t: np.ndarray) -> np.ndarray:
    """Stable argsort of already-transformed (unsigned) keys."""
    return np.argsort(keys_t, kind="stable")


def ordered_u32(keys: np.ndarray, descending: bool = False) -> np.ndarray:
    """The order-preserving bijection of the reference (Algorithm.cpp:459-469)."""
    k = keys.view(np.uint32) if keys.dtype != np.uint32 else keys
    if keys.dtype == np.int32:
        t = k ^ np.uint32(0x80000000)
    elif keys.dtype == np.float32:
        t = np.where(k & np.uint32(0x80000000), ~k, k | np.uint32(0x80000000)).astype(np.uint32)
    else:
        t = k.copy()
    return ~t if descending else t


def learned_mixture(n: int, seed: int = 5) -> np.ndarray:
    """The learned-CDF configuration's key distribution at any n (float32):
    75% from 8 Gaussians (means uniform in [-1e3, 1e3], sigmas log-uniform in
    [1e-2, 1e2]), 20% lognormal(0, 2), 5% exact copies of 1,000 values taken
    from the preceding keys; shuffled."""
    rng = np.random.default_rng(seed)
    n75, n20 = int(0.75 * n), int(0.20 * n)
    n5 = n - n75 - n20
    means = rng.uniform(-1e3, 1e3, 8)
    sig = np.exp(rng.uniform(np.log(1e-2), np.log(1e2), 8))
    comp = rng.integers(0, 8, n75)
    a = means[comp] + sig[comp] * rng.standard_normal(n75)
    b = rng.lognormal(0.0, 2.0, n20)
    pool = np.concatenate([a, b])[:1000]
    c = pool[rng.integers(0, pool.size, n5)] if pool.size else np.zeros(n5)
    keys = np.concatenate([a, b, c]).astype(np.float32)
    rng.shuffle(keys)
    return keys
