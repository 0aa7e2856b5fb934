"""Seeded inputs of the golden cases (shared by make_golden.py and the tests).

Each case is regenerated bit-identically from its seed with numpy's PCG64
generator, so only the reference's outputs are committed.
"""

import numpy as np


def psf_quadrants(Nnum, hs, seed):
    """Per-plane ``[n_h, n_h, h, h]`` float32 H and Ht quadrants; each PSF sums to 1."""
    rng = np.random.default_rng(seed)
    nh = (Nnum + 1) // 2
    H, Ht = [], []
    for h in hs:
        a = rng.random((nh, nh, h, h)) ** 3
        a /= a.sum(axis=(2, 3), keepdims=True)
        b = rng.random((nh, nh, h, h)) ** 3
        b /= b.sum(axis=(2, 3), keepdims=True)
        H.append(a.astype(np.float32))
        Ht.append(b.astype(np.float32))
    return H, Ht


# name -> case description
CASES = {
    # The reference's projector self-test uses one plane, random [0,1) input and
    # non-square shapes on purpose (projector.py:1170-1212); Nnum 15.
    "selftest_sq": dict(Nnum=15, hs=[31], shape=(2, 90, 90), seed=11, kind="project"),
    "selftest_wide": dict(Nnum=15, hs=[31], shape=(1, 90, 180), seed=12, kind="project"),
    "selftest_tall": dict(Nnum=15, hs=[31], shape=(1, 180, 90), seed=13, kind="project"),
    # several planes, Nnum 7, ragged support sizes
    "planes_n7": dict(Nnum=7, hs=[29, 15, 43], shape=(1, 35, 49), seed=21, kind="project"),
    # full Richardson-Lucy runs (lfdeconv.DeconvRL), Nnum 5, three planes
    "rl_prevedel": dict(Nnum=5, hs=[21, 11, 21], shape=(1, 30, 30), seed=31, kind="rl",
                        iters=3, prevedel=True),
    "rl_standard": dict(Nnum=5, hs=[21, 11, 21], shape=(1, 30, 30), seed=32, kind="rl",
                        iters=2, prevedel=False),
}


def case_inputs(name):
    c = CASES[name]
    H, Ht = psf_quadrants(c["Nnum"], c["hs"], c["seed"])
    rng = np.random.default_rng(c["seed"] + 1000)
    T, Y, X = c["shape"]
    Z = len(c["hs"])
    img = rng.random((T, Y, X)).astype(np.float32)
    vol = rng.random((Z, T, Y, X)).astype(np.float32)
    if c["kind"] == "rl":
        img = (img * 1000.0 + 100.0).astype(np.float32)
    return dict(H=H, Ht=Ht, img=img, vol=vol, **c)
