"""static_map through the C ABI, on the reference's test recipe
(lib/test/Compute/main.cpp:337-386): 200,000 distinct keys i * 2654435761 mod
0xFFFFFFF0 with values i in a table of 400,000 slots, every key inserted once
(re-inserting counts nothing and keeps the first value), finds of present
and absent keys, contains, and the overflow of a 4-slot table; plus the
table's structure checked against the linear-probing rule of the oracle, the
first-value rule, custom empty markers, clear() and the limits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_reference_recipe(gbc, ctx, orc):
    n = 200000
    keys = ((np.arange(n, dtype=np.uint64) * 2654435761) % 0xFFFFFFF0).astype(np.uint32)
    assert np.unique(keys).size == n
    values = np.arange(n, dtype=np.uint32)
    m = gbc.StaticMap(ctx, 2 * n)
    assert m.capacity() == 1 << 19
    kb, vb = gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, values)
    assert m.insert(kb, vb) == n
    assert m.size() == n
    assert m.insert(kb, vb) == 0
    queries = np.concatenate([keys[:1000], (0xFFFFFFF1 + np.arange(1000) % 14).astype(np.uint32)])
    qb = gbc.DeviceBuffer.from_host(ctx, queries)
    found = gbc.DeviceBuffer(ctx, queries.size, np.uint32)
    m.find(qb, found)
    fv = found.to_host()
    assert np.array_equal(fv[:1000], values[:1000])
    assert np.all(fv[1000:] == m.empty_value())
    present = gbc.DeviceBuffer(ctx, queries.size, np.uint8)
    m.contains(qb, present)
    pv = present.to_host()
    assert int(pv.sum()) == 1000 and np.all(pv[:1000] == 1)
    sk, sv = m.slots()
    assert orc.linear_probe_table_ok(sk, 0xFFFFFFFF)
    occ = sk != 0xFFFFFFFF
    assert occ.sum() == n
    order = np.argsort(sk[occ])
    assert np.array_equal(sk[occ][order], np.sort(keys))
    assert np.array_equal(sv[occ][order], values[np.argsort(keys)])

    tiny = gbc.StaticMap(ctx, 4)
    with pytest.raises(gbc.OutOfMemoryError, match="table is full"):
        tiny.insert(kb, vb, 10)
    assert tiny.size() == 4
    tiny.clear()
    assert tiny.size() == 0
    assert tiny.insert(kb, vb, 3) == 3


def test_first_value_wins_and_empty_key(gbc, ctx):
    m = gbc.StaticMap(ctx, 64, empty_key=0, empty_value=7)
    keys = np.array([5, 9, 0, 5, 12], dtype=np.uint32)  # 0 is the empty marker: skipped
    vals = np.array([50, 90, 1, 51, 120], dtype=np.uint32)
    assert m.insert(gbc.DeviceBuffer.from_host(ctx, keys[:3]), gbc.DeviceBuffer.from_host(ctx, vals[:3])) == 2
    # a later insert of a present key keeps the first value
    assert m.insert(gbc.DeviceBuffer.from_host(ctx, keys[3:]), gbc.DeviceBuffer.from_host(ctx, vals[3:])) == 1
    q = np.array([5, 9, 12, 0, 1], dtype=np.uint32)
    out = gbc.DeviceBuffer(ctx, 5, np.uint32)
    m.find(gbc.DeviceBuffer.from_host(ctx, q), out)
    assert list(out.to_host()) == [50, 90, 120, 7, 7]


def test_duplicates_in_one_insert(gbc, ctx, orc):
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 5000, size=200000, dtype=np.uint32)  # many duplicates per key
    vals = rng.integers(0, 1 << 30, size=keys.size, dtype=np.uint32)
    m = gbc.StaticMap(ctx, 16384)
    distinct = np.unique(keys)
    assert m.insert(gbc.DeviceBuffer.from_host(ctx, keys), gbc.DeviceBuffer.from_host(ctx, vals)) == distinct.size
    out = gbc.DeviceBuffer(ctx, distinct.size, np.uint32)
    m.find(gbc.DeviceBuffer.from_host(ctx, distinct), out)
    got = out.to_host()
    # the stored value is one of that key's values (which one is not specified
    # for keys repeated inside one insert)
    pairs = set(zip(keys.tolist(), vals.tolist()))
    assert all((int(k), int(v)) in pairs for k, v in zip(distinct, got))
    sk, _ = m.slots()
    assert orc.linear_probe_table_ok(sk, 0xFFFFFFFF)


def test_full_table_and_limits(gbc, ctx, orc):
    # exactly full: every slot used, absent keys still terminate their walk
    m = gbc.StaticMap(ctx, 1024)
    keys = np.arange(1, 1025, dtype=np.uint32) * 7919
    kb = gbc.DeviceBuffer.from_host(ctx, keys)
    assert m.insert(kb, kb) == 1024
    q = gbc.DeviceBuffer.from_host(ctx, np.array([3, keys[10]], dtype=np.uint32))
    out = gbc.DeviceBuffer(ctx, 2, np.uint32)
    m.find(q, out)
    assert list(out.to_host()) == [0xFFFFFFFF, keys[10]]
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.StaticMap(ctx, (1 << 31) + 1)
    with pytest.raises(gbc.InvalidArgumentError):
        m.insert(kb, kb, 2000)  # n beyond the buffers
