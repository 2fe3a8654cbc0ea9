"""Two contexts on one device, each driven by its own host thread (a context
is not thread-safe, so one per thread; compute_c.h): sorts, scans and
reductions run concurrently on the two contexts' streams. Every result must
equal the one-context result, bit for bit. This is the double-buffered use
that the end-to-end benchmark makes."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def work(gbc, c, keys_host, vals_host, x_host, rounds, out):
    """Per round: sort_by_key of a copy of the keys, an exclusive scan with
    its wide total and a reduction, all on context c; the last round's
    results go to out."""
    for _ in range(rounds):
        k = gbc.DeviceBuffer.from_host(c, keys_host)
        v = gbc.DeviceBuffer.from_host(c, vals_host)
        gbc.sort_by_key(c, k, v)
        x = gbc.DeviceBuffer.from_host(c, x_host)
        y = gbc.DeviceBuffer(c, x_host.size, np.int32)
        total = gbc.exclusive_scan(c, x, y, total=True)
        red = gbc.reduce(c, x)
        out["keys"], out["vals"], out["scan"] = k.to_host(), v.to_host(), y.to_host()
        out["total"], out["reduce"] = int(total), int(red)


@pytest.mark.parametrize("n", [1 << 16, 3_000_001])
def test_two_contexts_two_threads(gbc, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.uint32)
    x = rng.integers(-1000, 1001, n).astype(np.int32)
    order = np.argsort(keys, kind="stable")
    want_scan = (np.cumsum(x, dtype=np.int64) - x).astype(np.int32)  # wraps like int32
    ctxs = [gbc.Context(), gbc.Context()]
    try:
        outs = [{}, {}]
        errors = []

        def run(i):
            try:
                work(gbc, ctxs[i], keys, vals, x, 3, outs[i])
            except Exception as exc:  # re-raised after the join
                errors.append(exc)

        threads = [threading.Thread(target=run, args=(i,)) for i in range(2)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        for out in outs:
            assert np.array_equal(out["keys"], keys[order])
            assert np.array_equal(out["vals"], vals[order])
            assert np.array_equal(out["scan"], want_scan)
            assert out["total"] == int(x.astype(np.int64).sum())
            assert out["reduce"] == int(x.astype(np.int64).sum())  # no int32 wrap at these sizes
    finally:
        for c in ctxs:
            c.close()
