"""histogram_even parity on the GPU (lib/test/Compute/main.cpp:314-336 and
the bin rule of Algorithm.cpp:240-273): exact counts against the oracle."""
import numpy as np
import pytest
from helpers import GOLDEN, SIZES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", SIZES)
def test_histogram_reference_recipe(ctx, gbc, orc, n):
    host = orc.random_uints(n, 1000, n + 3)
    inp = gbc.DeviceBuffer.from_host(ctx, host)
    hist = gbc.DeviceBuffer(ctx, 10, np.uint32)
    gbc.histogram_even(ctx, inp, hist, 0.0, 1000.0)
    assert hist.to_host().tolist() == GOLDEN["histogram10"][str(n)]


def test_u8_256_bins(ctx, gbc, orc):
    rng = np.random.default_rng(3)
    x = rng.integers(0, 256, size=(1 << 22) + 13, dtype=np.uint8)
    inp = gbc.DeviceBuffer.from_host(ctx, x)
    hist = gbc.DeviceBuffer(ctx, 256, np.uint32)
    gbc.histogram_even(ctx, inp, hist, 0.0, 256.0)
    assert np.array_equal(hist.to_host(), np.bincount(x, minlength=256).astype(np.uint32))


@pytest.mark.parametrize("dtype", [np.int8, np.uint16, np.int32, np.int64, np.float32, np.float64])
@pytest.mark.parametrize("bins", [1, 7, 1000, 5000, 65536])
def test_types_and_bin_counts(ctx, gbc, orc, dtype, bins):
    rng = np.random.default_rng(bins)
    n = 300001
    if np.dtype(dtype).kind == "f":
        x = rng.uniform(-120, 130, size=n).astype(dtype)
        x[::1000] = np.array([-100.0, 100.0, 0.0, np.nan, -0.0], dtype=dtype)[rng.integers(0, 5)]
    else:
        info = np.iinfo(dtype)
        x = rng.integers(max(info.min, -120), min(info.max, 130), size=n).astype(dtype)
    lower, upper = -100.0, 100.0
    inp = gbc.DeviceBuffer.from_host(ctx, x)
    hist = gbc.DeviceBuffer(ctx, bins, np.uint32)
    gbc.histogram_even(ctx, inp, hist, lower, upper)
    assert np.array_equal(hist.to_host(), orc.histogram_even(x, bins, lower, upper))


def test_edges_and_errors(ctx, gbc, orc):
    x = np.linspace(0, 1, 100001, dtype=np.float32)
    inp = gbc.DeviceBuffer.from_host(ctx, x)
    hist = gbc.DeviceBuffer(ctx, 3, np.uint32)
    gbc.histogram_even(ctx, inp, hist, 0.0, 0.3)
    assert np.array_equal(hist.to_host(), orc.histogram_even(x, 3, 0.0, 0.3))
    with pytest.raises(ValueError):
        gbc.histogram_even(ctx, inp, hist, 1.0, 1.0)
    empty = gbc.DeviceBuffer(ctx, 0, np.float32)
    gbc.fill(ctx, hist, 5)
    gbc.histogram_even(ctx, empty, hist, 0.0, 1.0)
    assert hist.to_host().tolist() == [0, 0, 0]
