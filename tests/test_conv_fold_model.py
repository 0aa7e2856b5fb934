"""The decomposition k_conv3d_tma16 computes, restated in numpy and checked
against a direct 3x3x3 'same' convolution (float64, no GPU).

The kernel walks z over columns of R rows x W voxels.  For every input plane z'
of a column it forms, per output row r and (dy, dx), one product of the slab
row r+dy shifted by dx (M = voxels) with a packed weight block whose N index is
(dz, co), accumulating over (dy, dx) and the 16-channel K steps:

    D[z'][r][x][dz*CO + co] = sum_{dy,dx,ci} in[z'][y0+r+dy-1][x0+x+dx-1][ci] w[dz*9+dy*3+dx][ci][co]

and the epilogue adds three column groups of three slabs:

    out[z][r][x][co] = D[z-1][r][x][0*CO+co] + D[z][r][x][1*CO+co] + D[z+1][r][x][2*CO+co],

leaving out the planes z-1 < 0 and z+1 >= Z.  Columns may be split into z
chunks, each loading the halo planes zlo-1 and zlo+nz.  This test follows that
order exactly (slab layout, B block order blk*KS + kh, the N order, chunking),
so an edit that breaks the mapping fails here first.
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


def packed_b(w, CI, CO):
    """The shared-memory B operands: block (blk = dy*3+dx, K step kh) is an
    N x 16 matrix with row n = dz*CO + co and column k = ci - 16 kh."""
    KS = CI // 16
    blocks = np.zeros((9 * KS, 3 * CO, 16))
    for blk in range(9):
        for kh in range(KS):
            for n in range(3 * CO):
                dz, co = divmod(n, CO)
                blocks[blk * KS + kh, n, :] = w[dz * 9 + blk, kh * 16:(kh + 1) * 16, co]
    return blocks


def fold_model(x, w, R, W, zc):
    """out via the kernel's slabs, folded MMAs and epilogue sums (segment width W)."""
    B, Z, Y, X, CI = x.shape
    CO = w.shape[2]
    KS = CI // 16
    bops = packed_b(w, CI, CO)
    out = np.full((B, Z, Y, X, CO), np.nan)
    xsegs, yblocks, zchunks = -(-X // W), -(-Y // R), -(-Z // zc)
    for b in range(B):
        for zi in range(zchunks):
            zlo = zi * zc
            nz = min(Z - zlo, zc)
            for yb in range(yblocks):
                y0 = yb * R
                for xs in range(xsegs):
                    x0 = xs * W
                    # slabs zlo-1 .. zlo+nz: (R+2) rows x (W+2) voxels, zeros outside the volume
                    D = {}
                    for k in range(nz + 2):
                        zin = zlo - 1 + k
                        if not 0 <= zin < Z:
                            continue                       # MMAs skipped; the epilogue leaves it out
                        slab = np.zeros((R + 2, W + 2, CI))
                        for j in range(R + 2):
                            yy = y0 - 1 + j
                            if not 0 <= yy < Y:
                                continue
                            lo, hi = max(x0 - 1, 0), min(x0 - 1 + W + 2, X)
                            slab[j, lo - (x0 - 1):hi - (x0 - 1)] = x[b, zin, yy, lo:hi]
                        acc = np.zeros((R, W, 3 * CO))
                        for r in range(R):
                            for blk in range(9):
                                dy, dx = divmod(blk, 3)
                                for kh in range(KS):
                                    a = slab[r + dy, dx:dx + W, kh * 16:(kh + 1) * 16]   # M x K
                                    acc[r] += a @ bops[blk * KS + kh].T                  # M x N
                        D[zin] = acc
                    for i in range(nz):
                        z = zlo + i
                        o = D[z][:, :, CO:2 * CO].copy()
                        if z > 0:
                            o += D[z - 1][:, :, 0:CO]
                        if z + 1 < Z:
                            o += D[z + 1][:, :, 2 * CO:3 * CO]
                        for r in range(R):
                            y = y0 + r
                            if y >= Y:
                                continue
                            n = min(W, X - x0)
                            out[b, z, y, x0:x0 + n] = o[r, :n]
    return out


@pytest.mark.parametrize("ci,co,R", [(16, 16, 2), (16, 32, 1), (32, 16, 2), (32, 32, 1)])
@pytest.mark.parametrize("shape,W,zc", [((1, 5, 5, 13), 8, 5), ((2, 6, 4, 9), 4, 2), ((1, 7, 3, 6), 16, 3)])
def test_fold_model_matches_direct_convolution(ci, co, R, shape, W, zc):
    rng = np.random.default_rng(ci * 100 + co + sum(shape))
    x = rng.standard_normal(shape + (ci,))
    w = rng.standard_normal((27, ci, co)) / np.sqrt(27 * ci)
    got = fold_model(x, w, R, W, zc)
    assert not np.isnan(got).any()                       # every output voxel written once
    np.testing.assert_allclose(got, direct_conv(x, w), rtol=1e-12, atol=1e-12)


def head_model(x, w, R, W, zc):
    """The head variant (output channel 0 only): B block dx holds B[n = dz*3 + dy][ci] =
    w[dz*9 + dy*3 + dx][ci][0] (n < 9, zero above); one MMA per slab input row and dx
    accumulates D[z'][ri][x][n]; out[z][y0 + r][x] = sum over (dz, dy) of
    D[z - 1 + dz][r + dy][x][dz*3 + dy], planes outside the volume left out."""
    B, Z, Y, X, CI = x.shape
    KS = CI // 16
    blocks = np.zeros((3 * KS, 16, 16))
    for dx in range(3):
        for kh in range(KS):
            for n in range(9):
                dz, dy = divmod(n, 3)
                blocks[dx * KS + kh, n, :] = w[dz * 9 + dy * 3 + dx, kh * 16:(kh + 1) * 16, 0]
    out = np.full((B, Z, Y, X), np.nan)
    for b in range(B):
        for zlo in range(0, Z, zc):
            nz = min(Z - zlo, zc)
            for y0 in range(0, Y, R):
                for x0 in range(0, X, W):
                    D = {}
                    for k in range(nz + 2):
                        zin = zlo - 1 + k
                        if not 0 <= zin < Z:
                            continue
                        slab = np.zeros((R + 2, W + 2, CI))
                        for j in range(R + 2):
                            yy = y0 - 1 + j
                            if not 0 <= yy < Y:
                                continue
                            lo, hi = max(x0 - 1, 0), min(x0 - 1 + W + 2, X)
                            slab[j, lo - (x0 - 1):hi - (x0 - 1)] = x[b, zin, yy, lo:hi]
                        acc = np.zeros((R + 2, W, 16))
                        for ri in range(R + 2):
                            for dx in range(3):
                                for kh in range(KS):
                                    acc[ri] += slab[ri, dx:dx + W, kh * 16:(kh + 1) * 16] @ blocks[dx * KS + kh].T
                        D[zin] = acc
                    for i in range(nz):
                        z = zlo + i
                        o = np.zeros((R, W))
                        for dz in range(3):
                            if (z - 1 + dz) not in D:
                                continue
                            for r in range(R):
                                for dy in range(3):
                                    o[r] += D[z - 1 + dz][r + dy, :, dz * 3 + dy]
                        for r in range(R):
                            if y0 + r < Y:
                                n = min(W, X - x0)
                                out[b, z, y0 + r, x0:x0 + n] = o[r, :n]
    return out


@pytest.mark.parametrize("shape,W,zc", [((1, 5, 9, 13), 8, 5), ((2, 6, 6, 9), 4, 2), ((1, 7, 3, 6), 16, 3)])
def test_head_fold_model_matches_direct_convolution(shape, W, zc):
    rng = np.random.default_rng(sum(shape) + W)
    x = rng.standard_normal(shape + (16,))
    w = rng.standard_normal((27, 16, 16)) / np.sqrt(27 * 16)
    got = head_model(x, w, 4, W, zc)
    assert not np.isnan(got).any()
    np.testing.assert_allclose(got, direct_conv(x, w)[..., 0], rtol=1e-12, atol=1e-12)
