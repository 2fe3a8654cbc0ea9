"""Pins the CPU oracle (both layers) to the reference's own test recipes and
known answers, and checks the restated reference algorithms against the
std:: layer. CPU only."""
import hashlib
import json
import os

import numpy as np
import pytest

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_recipes.json")))
SMALL = [0, 1, 7, 255, 256, 1000, 4097, 100003]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_generator_matches_cxx_standard(orc):
    # [rand.predef]: the 10000th consecutive output of a default-constructed
    # mt19937 is 4123659995.
    assert orc.random_uints(10000, 0xFFFFFFFF, 5489)[9999] == 4123659995
    assert GOLDEN["mt19937_5489_10000th"] == 4123659995


def test_fixtures_reproduce(orc):
    # The committed fixtures are what the oracle computes here and on the GPU host.
    import importlib.util

    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    assert json.loads(json.dumps(mg.make(), sort_keys=True)) == GOLDEN


def test_capi_known_answers():
    # capi.c:103-141: N = 10007, host[i] = (i * 7919 % 1000) - 500; max is 499.
    i = np.arange(10007, dtype=np.int64)
    h = (i * 7919 % 1000 - 500).astype(np.int32)
    assert GOLDEN["capi"]["max"] == 499 == int(h.max())
    assert GOLDEN["capi"]["sum_i64"] == int(h.astype(np.int64).sum())


@pytest.mark.parametrize("n", SMALL)
def test_ref_radix_sort_matches_std(orc, n):
    keys = orc.random_uints(n, 0xFFFFFFFF, n + 2)
    idx = np.arange(n, dtype=np.uint32)
    k1, v1 = orc.std_sort(keys, idx)
    k2, v2 = orc.ref_radix_sort(keys, idx)
    assert np.array_equal(k1, k2) and np.array_equal(v1, v2)
    assert digest(k1) == GOLDEN["sort_by_key"][str(n)]["keys"]
    assert digest(v1) == GOLDEN["sort_by_key"][str(n)]["values"]
    assert np.array_equal(k1, np.sort(keys, kind="stable"))


def test_stability_signed_float(orc):
    dup = orc.random_uints(50000, 15, 99)
    k, v = orc.ref_radix_sort(dup, np.arange(dup.size, dtype=np.uint32))
    assert digest(v) == GOLDEN["stability"]["values"]
    assert np.all((np.diff(k.astype(np.int64)) > 0) | ((np.diff(k.astype(np.int64)) == 0) & (np.diff(v.astype(np.int64)) > 0)))

    ints = np.array(GOLDEN["signed"]["keys_in"], dtype=np.int32)
    assert orc.ref_radix_sort(ints)[0].tolist() == GOLDEN["signed"]["sorted"]

    f = orc.random_floats(3000, -1e6, 1e6, 5)
    f[0], f[1], f[2] = np.float32(-0.0), np.float32(np.inf), np.float32(-np.inf)
    fk, _ = orc.ref_radix_sort(f, None, descending=True)
    assert digest(fk.view(np.uint32)) == GOLDEN["floats_desc"]["sorted_bits"]
    # the reference test's own check: equal as floats to std::sort(greater)
    assert np.array_equal(fk, np.sort(f)[::-1])
    # and the bit-exact order puts +0.0 before -0.0 when descending
    zeros = fk[(fk == 0)]
    assert np.signbit(zeros[-1])


def test_u64_and_descending(orc):
    rng = np.random.default_rng(7)
    k = rng.integers(0, 2**64, size=5000, dtype=np.uint64)
    k[::7] = k[3]
    v = np.arange(k.size, dtype=np.uint32)
    a = orc.std_sort(k, v, descending=True)
    b = orc.ref_radix_sort(k, v, descending=True)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    order = np.lexsort((v, ~k))
    assert np.array_equal(a[1], v[order])


@pytest.mark.parametrize("n", SMALL)
def test_ref_scan_matches_std(orc, n):
    x = orc.random_uints(n, 100, n + 1)
    assert digest(orc.std_scan(x)) == GOLDEN["scan"][str(n)]["inclusive"]
    assert digest(orc.std_scan(x, exclusive=True)) == GOLDEN["scan"][str(n)]["exclusive"]
    assert np.array_equal(orc.ref_scan(x), orc.std_scan(x))
    assert np.array_equal(orc.ref_scan(x, exclusive=True), orc.std_scan(x, exclusive=True))


def test_scan_non_commutative_and_max(orc):
    v = (np.arange(5000, dtype=np.int64) * 7 % 101).astype(np.int32)
    r = orc.ref_scan(v, orc.OP_RIGHT, 0)
    assert np.array_equal(r, v)
    assert digest(orc.std_scan(v, orc.OP_MAX, -(2**31))) == GOLDEN["scan_max"]["inclusive"]
    assert np.array_equal(orc.ref_scan(v, orc.OP_MAX, -(2**31)), np.maximum.accumulate(v))


def test_int32_scan_wraps(orc):
    x = np.full(10, 2**30, dtype=np.int32)
    s = orc.std_scan(x)
    assert s[3] == np.int32(-(2**32) + 4 * 2**30) and s[2] == -(2**30)


@pytest.mark.parametrize("n", SMALL)
def test_reduce(orc, n):
    x = orc.random_uints(n, 1000, n)
    g = GOLDEN["reduce"][str(n)]
    assert int(orc.std_reduce(x, orc.OP_PLUS, 0, 7)) == g["sum_init7"]
    assert int(orc.ref_reduce(x, orc.OP_PLUS, 0, 7)) == g["sum_init7"]
    if n:
        assert int(orc.ref_reduce(x, orc.OP_MAX, 0, 0)) == g["max"]
        assert int(orc.ref_reduce(x, orc.OP_MIN, 0xFFFFFFFF, 0xFFFFFFFF)) == g["min"]


@pytest.mark.parametrize("n", SMALL)
def test_histogram(orc, n):
    x = orc.random_uints(n, 1000, n + 3)
    h = orc.histogram_even(x, 10, 0.0, 1000.0)
    # the reference test's host reference (main.cpp:332-334)
    href = np.bincount(x[x < 1000] // 100, minlength=10)
    assert h.tolist() == href.tolist() == GOLDEN["histogram10"][str(n)]


def test_histogram_float_rule(orc):
    # bins computed in float: values near an edge follow (x - lower) * scale
    x = np.array([0.0, 0.1, 0.2999999, 0.3, 0.9999999, 1.0, -0.0, np.nan], dtype=np.float32)
    h = orc.histogram_even(x, 10, 0.0, 1.0)
    scale = np.float32(10) / (np.float32(1.0) - np.float32(0.0))
    exp = np.zeros(10, dtype=np.uint32)
    for v in x:
        if v >= 0 and v < 1:
            b = min(int(np.float32(v - np.float32(0)) * scale), 9)
            exp[b] += 1
    assert h.tolist() == exp.tolist()


def test_network_gradient_matches_finite_differences(orc):
    # The oracle's analytic gradient of the learned-CDF network against
    # central differences of its own loss (parameters in float, loss in double).
    H = 32
    rng = np.random.default_rng(4)
    m = 400
    keys = np.sort(rng.integers(0, 1 << 32, m, dtype=np.uint64)).astype(np.uint32)
    q = keys[np.minimum(np.arange(H + 1) * m // H, m - 1)].astype(np.int64)
    centres = (q[:-1] + (q[1:] - q[:-1]) // 2).astype(np.uint32)
    span = float(int(keys[-1]) - int(keys[0]))
    p = np.zeros(4 * H + H * H + 1, dtype=np.float32)
    p[0:H] = np.log(span / np.maximum(q[1:] - q[:-1], 1)) - 0.5
    p[H:2 * H] = rng.uniform(0.3, 0.7, H)
    p[2 * H:2 * H + H * H] = np.log(rng.uniform(0.01, 0.05, H * H))
    p[2 * H + H * H:3 * H + H * H] = rng.uniform(-0.4, 0.0, H)
    p[3 * H + H * H:4 * H + H * H] = np.log(np.full(H, 1.0 / H))
    ys = ((np.arange(m) + 0.5) / m).astype(np.float32)
    g, _ = orc.mlp_grad(p, centres, np.float32(1.0 / span), keys, ys)
    picks = [0, 5, H + 3, 2 * H + 7, 2 * H + 33 * 5, 2 * H + H * H + 2, 3 * H + H * H + 9, 4 * H + H * H]
    for i in picks:
        eps = np.float32(1e-2)
        up, dn = p.copy(), p.copy()
        up[i] += eps
        dn[i] -= eps
        _, lu = orc.mlp_grad(up, centres, np.float32(1.0 / span), keys, ys)
        _, ld = orc.mlp_grad(dn, centres, np.float32(1.0 / span), keys, ys)
        fd = (lu - ld) / (float(up[i]) - float(dn[i]))
        assert abs(fd - g[i]) <= 2e-2 * max(abs(g[i]), 1e-3 * np.max(np.abs(g))), (i, fd, g[i])
