"""The pooled output of k_conv3d_tma16<..., POOL> restated in numpy (float32, no GPU).

The epilogue of the 16-channel tcgen05 convolution walks work items of R = 2 output
rows x 128 voxels over a chunk of zc consecutive planes.  With POOL each lane keeps
the BF16 outputs it stored for its two rows, takes the neighbouring lane's values by
a shuffle (lane pairs are x pairs, since an item starts at a multiple of 128) and
adds, in k_pool2's order, (y0, x), (y0, x+1), (y0+1, x), (y0+1, x+1) of an even
plane and then of the next plane, times 1/8.  Plane pairs stay in one item because
the launcher rounds the chunk length zc up to an even number (its cost loop over 1..8
chunks is restated here).  The test checks, for the network's shapes, that every
chunk starts on an even plane and has an even length, and that the item-wise sums
give k_pool2's result bit for bit."""

import numpy as np
import pytest


def zc_choice(B, Z, Y, X, R=2, sms=152, pool=True):
    """The launcher's z chunk length (launch_tma16): fewest waves x slabs per item."""
    xsegs, yblocks = -(-X // 128), -(-Y // R)
    best, zc_best = -1, Z
    for c in range(1, min(8, Z) + 1):
        zc = -(-Z // c)
        if pool:
            zc += zc & 1
        items = B * (-(-Z // zc)) * yblocks * xsegs
        cost = -(-items // sms) * (zc + 2)
        if best < 0 or cost < best:
            best, zc_best = cost, zc
    return zc_best


def pool2_ref(y):
    """k_pool2: float32 sum over d = 0..7 (dz = d >> 2, dy = (d >> 1) & 1, dx = d & 1), times 1/8."""
    B, Z, Y, X, C = y.shape
    acc = np.zeros((B, Z // 2, Y // 2, X // 2, C), np.float32)
    for d in range(8):
        dz, dy, dx = d >> 2, (d >> 1) & 1, d & 1
        acc = acc + y[:, dz::2, dy::2, dx::2]
    return acc * np.float32(0.125)


def epilogue_pool(y, zc):
    """The epilogue's pooled output, item by item (lanes vectorised over x)."""
    B, Z, Y, X, C = y.shape
    out = np.full((B, Z // 2, Y // 2, X // 2, C), np.nan, np.float32)
    for b in range(B):
        for zlo in range(0, Z, zc):
            nz = min(Z - zlo, zc)
            assert zlo % 2 == 0 and nz % 2 == 0
            for y0 in range(0, Y, 2):
                for x0 in range(0, X, 128):
                    xs = np.arange(x0, min(x0 + 128, X))
                    for i in range(nz):
                        z = zlo + i
                        kept = y[b, z, y0:y0 + 2][:, xs]               # [2 rows, lanes, C]
                        nb = np.concatenate([kept[:, 1:], kept[:, -1:]], axis=1)   # shuffle down by one
                        if i % 2 == 0:
                            pacc = np.zeros((len(xs), C), np.float32)
                        pacc = pacc + kept[0]
                        pacc = pacc + nb[0]
                        pacc = pacc + kept[1]
                        pacc = pacc + nb[1]
                        if i % 2 == 1:
                            even = (xs % 2) == 0
                            out[b, z // 2, y0 // 2, xs[even] // 2] = (pacc * np.float32(0.125))[even]
    return out


@pytest.mark.parametrize("shape", [(2, 4, 6, 10), (1, 2, 2, 2), (1, 6, 8, 140), (1, 10, 12, 258),
                                   (1, 14, 20, 136)])
def test_epilogue_pool_matches_pool2(shape):
    rng = np.random.default_rng(sum(shape))
    y = rng.standard_normal(shape + (16,)).astype(np.float32)
    B, Z, Y, X = shape
    zc = zc_choice(B, Z, Y, X)
    got = epilogue_pool(y, zc)
    ref = pool2_ref(y)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("shape", [(1, 24, 456, 456), (4, 24, 128, 128), (1, 48, 1008, 1008), (1, 14, 40, 456),
                                   (2, 6, 16, 130), (8, 24, 128, 128)])
def test_chunks_hold_plane_pairs(shape):
    B, Z, Y, X = shape
    zc = zc_choice(B, Z, Y, X)
    assert zc % 2 == 0
    assert all(z % 2 == 0 for z in range(0, Z, zc))
    assert all(min(Z - z, zc) % 2 == 0 for z in range(0, Z, zc))
