"""The bitpack oracle (the reference's chunk format, lib/src/Compute/
Compression.cpp) on the reference's own test inputs (lib/test/Compute/
main.cpp:388-438): every recipe round-trips for both chunk sizes the
reference tests, with and without delta coding; the timestamps compress by
more than 4x in delta mode as the reference asserts; and the format's
details (header triples, widths, zigzag, wrap-around) match hand-computed
cases."""
import numpy as np
import pytest


def test_recipes_round_trip(orc):
    for n, ts, small, noise in orc.bitpack_recipes():
        for x in (ts, small, noise):
            for delta in (False, True):
                for chunk in (256, 2048):
                    words = orc.bitpack_compress(x, chunk, delta)
                    assert np.array_equal(orc.bitpack_decompress(words, n, chunk, delta), x)


def test_timestamps_delta_ratio(orc):
    n, ts, _, _ = orc.bitpack_recipes()[-1]
    words = orc.bitpack_compress(ts, 2048, True)
    assert 4 * n / (4 * words.size) > 4.0


def test_hand_computed_chunks(orc):
    # one chunk: values 10..13 -> base 10, width 2, packed 0b11100100 = 0xE4
    w = orc.bitpack_compress(np.array([10, 11, 12, 13], dtype=np.uint32), 256, False)
    assert list(w) == [10, 2, 0, 0xE4]
    # all equal: width 0, no packed words
    w = orc.bitpack_compress(np.full(300, 7, dtype=np.uint32), 256, False)
    assert list(w) == [7, 0, 0, 7, 0, 0]
    # full range: width 32, values stored verbatim
    x = np.array([0, 0xFFFFFFFF, 5], dtype=np.uint32)
    w = orc.bitpack_compress(x, 256, False)
    assert list(w[:3]) == [0, 32, 0] and list(w[3:]) == [0, 0xFFFFFFFF, 5]
    # delta + zigzag: 5, 3, 3 -> d = 5, -2, 0 -> zigzag 10, 3, 0
    w = orc.bitpack_compress(np.array([5, 3, 3], dtype=np.uint32), 256, True)
    assert list(w[:2]) == [0, 4]
    assert w[3] == (10 | (3 << 4) | (0 << 8))
    # wrap-around deltas decode exactly
    x = np.array([0xFFFFFFFF, 0, 0x80000000, 1], dtype=np.uint32)
    assert np.array_equal(orc.bitpack_decompress(orc.bitpack_compress(x, 256, True), 4, 256, True), x)


def test_corrupt_header_rejected(orc):
    w = orc.bitpack_compress(np.arange(1000, dtype=np.uint32), 256, False)
    bad = w.copy()
    bad[3 * 1 + 2] = 10 ** 6  # chunk 1's offset points past the data
    with pytest.raises(ValueError):
        orc.bitpack_decompress(bad, 1000, 256, False)
