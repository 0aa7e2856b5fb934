"""The warm start's first layer as a 3x3x1 convolution, restated in numpy (float64, no GPU).

flf_ws_input writes the four input features of voxels x - 1, x and x + 1 as channels
0..11 (channel 4k + j = feature j at x + k - 1, zero outside the volume), and the
first layer keeps only its taps at the centre x offset (dx = 1).  Any 3x3x3 layer
over the four features is then the same function: the weight of tap (dz, dy, dx),
feature j moves to tap (dz, dy, 1), channel 4 dx + j.  This checks that identity,
with the volume's zero padding at the x edges."""

import numpy as np

from test_conv_wide_model import direct_conv


def shifted_channels(f):
    """f [B, Z, Y, X, 4] -> [B, Z, Y, X, 16]: channel 4k + j = f[..., x + k - 1, j], zero outside."""
    B, Z, Y, X, F = f.shape
    out = np.zeros((B, Z, Y, X, 16))
    for k in range(3):
        lo, hi = max(0, 1 - k), min(X, X + 1 - k)          # x with 0 <= x + k - 1 < X
        out[:, :, :, lo:hi, 4 * k:4 * k + F] = f[:, :, :, lo + k - 1:hi + k - 1]
    return out


def test_3x3x1_over_shifted_channels_equals_3x3x3():
    rng = np.random.default_rng(11)
    f = rng.standard_normal((2, 5, 6, 9, 4))
    w = rng.standard_normal((27, 4, 16))
    ref = direct_conv(f, w)
    w1 = np.zeros((27, 16, 16))
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                w1[dz * 9 + dy * 3 + 1, 4 * dx:4 * dx + 4] = w[dz * 9 + dy * 3 + dx]
    got = direct_conv(shifted_channels(f), w1)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    # the layer's off-centre x taps stay zero, so a full 3x3x3 kernel over the same input agrees
    assert not np.any(w1[[t for t in range(27) if t % 3 != 1]])
