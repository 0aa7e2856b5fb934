"""The padded-row decomposition k_conv3d_wide computes, restated in numpy and
checked against a direct 3x3x3 'same' convolution (float64, no GPU).

A work item is output plane z of volume b and rows y0 .. y0+R-1.  For every
input plane z+dz in the volume and every chunk of KC (<= 64) input channels a
slab of R+2 rows x Xp = X+2 voxels (the halo, zeros outside the volume) is laid
out as rows of 8 channels, the voxel at slab (r, c) being row r*Xp + c of each
8-channel group.  Output position q = yl*Xp + x of the item reads, for tap
(dy, dx), slab row q + dy*Xp + dx, so every tap is one product of a shifted
row window (M = nM x 128 positions) with the packed weight block of
(tap, 16 input channels), accumulated over taps, K steps and chunks:

    D[q][co] = sum_{dz,dy,dx,ci} slab_{dz}[q + dy*Xp + dx][ci] w[(dz+1)*9 + dy*3 + dx][ci][co]

Positions with x >= X or yl >= R are computed and dropped.  The rows a slab
load does not write hold stale data (NaN here); only dropped positions read
them.  (On the device a 64-channel chunk is one TMA load of 128-byte rows with
the 128-byte swizzle, which the operand descriptors undo; the logical rows, and
so this model, are the same.)  The item shapes follow the launcher (rows per item balanced over the y
blocks, nM = ceil(R*Xp / 128)), and the weights the packing kernel's layout.  With
splits, each input plane z+dz of an item is its own work unit writing an FP32
partial sum, and the three partials are added afterwards.
"""

import numpy as np
import pytest


def direct_conv(x, w):
    """x [B, Z, Y, X, CI], w [27, CI, CO] -> [B, Z, Y, X, CO], zero padding."""
    B, Z, Y, X, CI = x.shape
    CO = w.shape[2]
    xp = np.zeros((B, Z + 2, Y + 2, X + 2, CI))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    out = np.zeros((B, Z, Y, X, CO))
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                out += xp[:, dz:dz + Z, dy:dy + Y, dx:dx + X] @ w[dz * 9 + dy * 3 + dx]
    return out


def pack(w):
    """k_conv3d_pack_weights: wp[((tap*CI/16 + ks)*2 + k8)*CO + co][j] = w[tap][16 ks + 8 k8 + j][co]."""
    _, CI, CO = w.shape
    wp = np.zeros(27 * CI * CO)
    for tap in range(27):
        for ci in range(CI):
            ks, k8, j = ci >> 4, (ci >> 3) & 1, ci & 7
            for co in range(CO):
                wp[((((tap * (CI // 16) + ks) * 2 + k8) * CO + co) * 8) + j] = w[tap, ci, co]
    return wp


def item_shape(Y, X, CO, nM):
    """The launcher's wide_shape: (Xp, R, nM, nyb, slab_rows) or None."""
    Xp = X + 2
    rmax = nM * 128 // Xp
    if rmax < 1 or Xp > 256 or nM * CO > 256:
        return None
    nyb = -(-Y // rmax)
    R = -(-Y // nyb)
    nM = -(-(R * Xp) // 128)
    slab_rows = (nM * 128 + 2 * Xp + 2 + 7) // 8 * 8
    return Xp, R, nM, nyb, slab_rows


def wide_conv(x, w, nM_req, splits=1):
    B, Z, Y, X, CI = x.shape
    CO = w.shape[2]
    shp = item_shape(Y, X, CO, nM_req)
    assert shp is not None
    Xp, R, nM, nyb, slab_rows = shp
    KC = min(CI, 64)
    NCG, G8, KS = CI // KC, KC // 8, KC // 16
    wp = pack(w)
    out = np.full((B, Z, Y, X, CO), np.nan)
    for it in range(B * Z * nyb):
        yb, q = it % nyb, it // nyb
        z, b = q % Z, q // Z
        y0 = yb * R
        # with splits each input plane's partial is its own unit's output, summed afterwards
        parts = {}
        for dz in (-1, 0, 1):
            D = parts.setdefault(dz if splits > 1 else 0, np.zeros((nM * 128, CO)))
            if not 0 <= z + dz < Z:
                continue
            for cg in range(NCG):
                # one slab slot: G8 groups of slab_rows rows x 8 channels, stale rows NaN
                slab = np.full((G8, slab_rows, 8), np.nan)
                for g in range(G8):
                    for r in range(R + 2):
                        for c in range(Xp):
                            yy, xx = y0 - 1 + r, c - 1
                            ch = cg * KC + 8 * g
                            slab[g, r * Xp + c] = (x[b, z + dz, yy, xx, ch:ch + 8]
                                                   if 0 <= yy < Y and 0 <= xx < X else 0.0)
                for t9 in range(9):
                    dy, dx = t9 // 3, t9 % 3
                    tap = (dz + 1) * 9 + t9
                    for ks in range(KS):
                        blk = (tap * (CI // 16) + cg * KS + ks) * 16 * CO
                        Bk = wp[blk:blk + 16 * CO].reshape(2, CO, 8)             # [k8][co][j]
                        Bm = Bk.transpose(0, 2, 1).reshape(16, CO)                # [k][co]
                        for m in range(nM):
                            rows = m * 128 + np.arange(128) + dy * Xp + dx
                            A = np.concatenate([slab[2 * ks, rows], slab[2 * ks + 1, rows]], axis=1)
                            D[m * 128:(m + 1) * 128] += A @ Bm
        D = sum(parts[k] for k in sorted(parts))
        for qq in range(nM * 128):
            yl, xx = qq // Xp, qq % Xp
            y = y0 + yl
            if yl < R and y < Y and xx < X:
                out[b, z, y, xx] = D[qq]
    return out


@pytest.mark.parametrize("shape,CI,CO,nM", [
    ((1, 3, 7, 9), 32, 64, 1), ((1, 3, 7, 9), 32, 64, 3), ((2, 2, 5, 13), 64, 32, 1),
    ((1, 3, 11, 30), 128, 64, 2), ((1, 2, 4, 70), 64, 128, 2), ((1, 2, 3, 126), 64, 64, 1),
])
@pytest.mark.parametrize("splits", [1, 3])
def test_wide_decomposition_matches_direct_conv(shape, CI, CO, nM, splits):
    rng = np.random.default_rng(CI + CO + nM)
    x = rng.standard_normal(shape + (CI,))
    w = rng.standard_normal((27, CI, CO))
    got = wide_conv(x, w, nM, splits)
    ref = direct_conv(x, w)
    assert np.isfinite(got).all()
    assert np.abs(got - ref).max() <= 1e-9 * np.abs(ref).max()


def test_item_shapes():
    # the network's level 2 and 3 at the 24 x 456 x 456 volume, and a training crop
    assert item_shape(114, 114, 64, 3) == (116, 3, 3, 38, 624)
    assert item_shape(57, 57, 128, 1) == (59, 2, 1, 29, 248)
    assert item_shape(32, 32, 64, 2) == (34, 7, 2, 5, 328)
    # no full padded row in the tiles, or accumulators beyond 256 TMEM columns
    assert item_shape(10, 200, 64, 1) is None
    assert item_shape(10, 20, 128, 4) is None
