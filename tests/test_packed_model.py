"""CPU tests: the numpy model of the GPU algorithm equals the oracle.

The model (tests/packed_model.py) follows the CUDA kernels index for index
(kernel construction, packed symmetric storage, multiply-accumulate), so a
pass here means the kernels' mathematics is right; the GPU tests then check
the kernels themselves.
"""

import numpy as np
import pytest

import packed_model as M
from oracle import lf_oracle as O


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("N,hs,Y,X", [(3, [7, 11], 12, 15), (5, [21, 11], 23, 17), (7, [15], 21, 28)])
def test_packed_model_matches_oracle(N, hs, Y, X):
    rng = np.random.default_rng(N)
    nh = (N + 1) // 2
    H = [rng.random((nh, nh, h, h)) for h in hs]
    vol = rng.random((len(hs), Y, X))
    img = rng.random((Y, X))
    fw = M.forward_model(H, vol, N)
    fo = O.forward_project(H, vol[:, None], N, method="direct", dtype=np.float64)[0]
    assert rel(fw, fo) < 1e-12
    bk = M.backward_model(H, img, N)
    bo = O.backward_project(H, img[None], N, method="direct", dtype=np.float64)[:, 0]
    assert rel(bk, bo) < 1e-12


def test_packed_rows_and_slots():
    for N in (3, 5, 15, 19):
        tb = M.tables(N)
        c = N // 2
        assert sorted(tb["slotcol"]) == list(range(N * N))
        # one half block: c(c+1) generic rows, c + 1 row pairs (mirror + transpose symmetry)
        assert tb["nrow"] == (c + 1) * (c + 2)
        assert len(tb["okind"]) == (c + 1) ** 2
        # every input channel is a stored row, a mirror image of one, or the transpose of one
        seen = set()
        for ch, kind, row, trans, mx in tb["groups"]:
            orbit = {ch, tb["My"](ch), tb["Mx"](ch), tb["Mxy"](ch)}
            seen |= orbit
            if trans:
                seen |= {tb["Tr"](i) for i in orbit}
        assert seen == set(range(N * N))
    # stored rows per frequency pair: 72 of the 128 of the mirror-only layout at Nnum 15
    fq = 25
    q = M.quads(fq)
    assert len(q) == fq * (fq + 1) // 2 and q[-1][2] + 1 == fq * fq


def test_transform_size_rule():
    # f >= max(Ly, Lx) + R with R = floor((ch + N - 1)/N); smallest even 7-smooth
    assert M.kernel_radius(211, 15) == 7
    assert M.choose_f(450, 450, [211, 61], 15) == 40
    assert M.choose_f(1005, 1005, [841], 15) == 96
