"""Small helpers shared by the test modules."""
import hashlib
import json
import os

import numpy as np

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_recipes.json")))
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
