"""Bitpack compression on the GPU through the C ABI against the oracle
(the reference's chunk format): the compressed words must equal the oracle's
word for word, decompression must restore the input exactly, and the
serialized blob must round-trip, on the reference's test recipes
(lib/test/Compute/main.cpp:388-451) at every size of main.cpp:54, both chunk
sizes it tests and every chunk size the format allows, plus unaligned
pointers, sizes that are not a multiple of 4 and the corrupt-blob
rejections."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _roundtrip(gbc, ctx, orc, x, chunk, delta):
    n = x.size
    inb = gbc.DeviceBuffer.from_host(ctx, x)
    comp = gbc.compress_bitpack(ctx, inb, delta=delta, chunk_size=chunk)
    want = orc.bitpack_compress(x, chunk, delta)
    got = comp.data.to_host() if comp.data.size else np.zeros(0, np.uint32)
    assert np.array_equal(got, want), (n, chunk, delta)
    out = gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.decompress_bitpack(ctx, comp, out)
    assert np.array_equal(out.to_host(), x)
    blob = comp.serialize()
    back = gbc.CompressedBuffer.deserialize(ctx, blob)
    assert (back.num_elements, back.chunk_size, back.delta) == (n, chunk, delta)
    out2 = gbc.DeviceBuffer(ctx, n, np.uint32)
    gbc.decompress_bitpack(ctx, back, out2)
    assert np.array_equal(out2.to_host(), x)
    return comp


def test_reference_recipes(gbc, ctx, orc):
    for n, ts, small, noise in orc.bitpack_recipes():
        for x in (ts, small, noise):
            for delta in (False, True):
                for chunk in (256, 2048):
                    _roundtrip(gbc, ctx, orc, x, chunk, delta)
    n, ts, _, _ = orc.bitpack_recipes()[-1]
    comp = _roundtrip(gbc, ctx, orc, ts, 2048, True)
    assert comp.uncompressed_bytes() / comp.compressed_bytes() > 4.0


@pytest.mark.parametrize("chunk", [256, 512, 1024, 2048, 4096, 16384, 65536])
def test_every_chunk_size_and_width(gbc, ctx, orc, chunk):
    rng = np.random.default_rng(chunk)
    n = 3 * chunk + 1237
    # chunks of every bit width 0..32 side by side
    widths = np.arange(n) // chunk
    x = np.zeros(n, dtype=np.uint64)
    for c in range((n + chunk - 1) // chunk):
        wbits = (7 * c + 3) % 33
        sl = slice(c * chunk, min(n, (c + 1) * chunk))
        hi = (1 << wbits) if wbits else 1
        x[sl] = 1000 + rng.integers(0, hi, size=sl.stop - sl.start, dtype=np.uint64)
    x = (x & 0xFFFFFFFF).astype(np.uint32)
    del widths
    for delta in (False, True):
        _roundtrip(gbc, ctx, orc, x, chunk, delta)


def test_odd_sizes_and_unaligned_pointers(gbc, ctx, orc):
    rng = np.random.default_rng(9)
    for n in (1, 2, 3, 5, 255, 257, 2047, 2049, 4099, 70001):
        x = rng.integers(0, 1 << 20, size=n, dtype=np.uint32)
        for delta in (False, True):
            _roundtrip(gbc, ctx, orc, x, 256, delta)
    # raw forms on pointers one element past a 16-byte boundary
    n = 100003
    x = rng.integers(0, 1 << 12, size=n + 1, dtype=np.uint32)
    inb = gbc.DeviceBuffer.from_host(ctx, x)
    cap = gbc.bitpack_words_bound(n, 2048)
    outw = gbc.DeviceBuffer(ctx, cap + 1, np.uint32)
    words = gbc.compress_bitpack_raw(ctx, inb.device_pointer + 4, n, outw.device_pointer + 4, cap, delta=True)
    want = orc.bitpack_compress(x[1:], 2048, True)
    assert words == want.size and np.array_equal(outw.to_host()[1:1 + words], want)
    dec = gbc.DeviceBuffer(ctx, n + 1, np.uint32)
    gbc.decompress_bitpack_raw(ctx, outw.device_pointer + 4, words, n, dec.device_pointer + 4, delta=True)
    assert np.array_equal(dec.to_host()[1:], x[1:])


def test_rejections(gbc, ctx, orc):
    x = np.arange(5000, dtype=np.uint32)
    inb = gbc.DeviceBuffer.from_host(ctx, x)
    for bad_chunk in (128, 300, 131072):
        with pytest.raises(gbc.InvalidArgumentError):
            gbc.compress_bitpack(ctx, inb, chunk_size=bad_chunk)
    # capacity below the compressed size
    outw = gbc.DeviceBuffer(ctx, 10, np.uint32)
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.compress_bitpack_raw(ctx, inb.device_pointer, x.size, outw.device_pointer, 10)
    # blobs: all zeros, truncated, corrupt chunk header
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.CompressedBuffer.deserialize(ctx, bytes(64))
    blob = gbc.compress_bitpack(ctx, inb, chunk_size=256).serialize()
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.CompressedBuffer.deserialize(ctx, blob[:-4])
    words = np.frombuffer(blob, dtype=np.uint32).copy()
    words[8 + 3 * 2 + 2] = 1 << 30  # chunk 2's packed offset past the data
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.CompressedBuffer.deserialize(ctx, words.tobytes())
    words = np.frombuffer(blob, dtype=np.uint32).copy()
    words[8 + 3 * 1 + 1] = 33  # a width above 32
    with pytest.raises(gbc.InvalidArgumentError):
        gbc.CompressedBuffer.deserialize(ctx, words.tobytes())
    # empty input: nothing to pack, still a valid (empty) stream
    e = gbc.DeviceBuffer(ctx, 0, np.uint32)
    comp = gbc.compress_bitpack(ctx, e)
    assert comp.num_elements == 0 and comp.compressed_bytes() == 0
    back = gbc.CompressedBuffer.deserialize(ctx, comp.serialize())
    assert back.num_elements == 0


@pytest.mark.parametrize("form", [0, 1])
def test_both_decoders_every_width(gbc, ctx, orc, form):
    # The one-pass decoder (lane-private whole words, the delta prefix sum
    # by look-back) and the two-pass one (4-element groups, then a scan), each
    # forced through the tuning table: chunks of every width 0..32, sizes that
    # end inside a chunk and inside a lane's 32 elements, both modes.
    rng = np.random.default_rng(40 + form)
    ctx.tuning_set("bitpack:unpack", form)
    try:
        for chunk in (256, 2048, 65536):
            for n in (5, 1000, 8192 * 3 + 33, 3 * chunk + 1237):
                x = np.zeros(n, dtype=np.uint64)
                for c in range((n + chunk - 1) // chunk):
                    wbits = (5 * c + 1) % 33
                    sl = slice(c * chunk, min(n, (c + 1) * chunk))
                    hi = (1 << wbits) if wbits else 1
                    x[sl] = 77 + rng.integers(0, hi, size=sl.stop - sl.start, dtype=np.uint64)
                x = (x & 0xFFFFFFFF).astype(np.uint32)
                steps = rng.integers(0, 50, n).astype(np.uint64)
                ts = ((1700000000 + np.cumsum(steps)) & 0xFFFFFFFF).astype(np.uint32)
                for data in (x, ts):
                    for delta in (False, True):
                        _roundtrip(gbc, ctx, orc, data, chunk, delta)
    finally:
        ctx.tuning_set("bitpack:unpack", -1)
