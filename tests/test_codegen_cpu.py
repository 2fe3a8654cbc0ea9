"""The transform compiler's code generation, without a GPU: seeded random
expressions are compiled by the library (clc_transform_compile) and the
program it emits is replayed with the device interpreter's rules
(interp_replay), element by element, on random and edge-value inputs of
random element types; every result must equal the expression oracle's
evaluation of the source text, bit for bit (NaN payloads aside). This checks
operand order, reversed operations, stack slots, conversions and selects for
programs far more varied than the GPU cases."""
import random

import numpy as np
import pytest

import interp_replay as R
import transform_oracle as T

TYPES = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64, np.float32, np.float64]


@pytest.fixture(scope="module")
def gbc():
    import gbcompute

    return gbcompute


def same(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    if a.dtype.kind == "f":
        return (np.isnan(a) & np.isnan(b)) | (a.view(np.uint32 if a.itemsize == 4 else np.uint64) ==
                                              b.view(np.uint32 if b.itemsize == 4 else np.uint64))
    return a == b


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_emitted_programs_match_the_oracle(gbc, seed):
    rng = random.Random(seed)
    compared = 0
    for _ in range(2500):
        has_y = rng.random() < 0.5
        tx, to = rng.choice(TYPES), rng.choice(TYPES)
        ty = rng.choice(TYPES) if has_y else None
        expr = R.random_expression(rng, rng.randint(1, 5), has_y)
        try:
            listing = gbc.transform_compile(expr, tx, to, ty)
        except (gbc.BuildError, gbc.UnsupportedError):
            continue
        x = R.sample_values(rng, tx, 24)
        y = R.sample_values(rng, ty, 24) if has_y else None
        want = T.transform(expr, x, to, y)
        got = R.evaluate(listing, x, to, y)
        ok = same(got, want)
        assert ok.all(), (expr, np.dtype(tx).name, np.dtype(ty).name if ty else None, np.dtype(to).name,
                          x[~ok][:3], (y[~ok][:3] if y is not None else None), got[~ok][:3], want[~ok][:3], listing)
        compared += 1
    assert compared > 1000
