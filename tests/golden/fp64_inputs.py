"""Inputs of the FP64-oracle fixtures at the benchmark configurations.

Each case fixes a geometry (Nnum, image size, z planes), a synthetic PSF set
with the shapes of that optical configuration (``synthetic.synthetic_psf``,
deterministic), a camera image built from integer arithmetic only (so it is
the same bits on every machine), the Richardson-Lucy run to check, and the
positions at which the FP64 outputs are stored.  ``make_fp64_fixtures.py``
computes the FP64 outputs; the GPU tests recompute the inputs from this file.

* ``450px_11planes``: 450 x 450 px, Nnum 15, 11 planes at -25..25 um: Htf and
  8 Prevedel RL iterations from a uniform volume, every plane.
* ``450px_21planes``: the same image size with 21 planes at -50..50 um (the
  learned warm start's configuration; PSF sizes 61..421): Htf and 8 Prevedel
  iterations, every plane.
* ``1005px_41planes``: 1005 x 1005 px, 41 planes at -100..100 um (PSF sizes up
  to 841): Htf and one Prevedel iteration (which needs the forward projection
  of all 41 planes) on 7 of the planes, from the edge to the centre.
"""

import numpy as np

M64 = (1 << 64) - 1

CASES = {
    "450px_11planes": dict(Nnum=15, Y=450, X=450, z=(-25, 25, 5), img_size_ref=7, iters=8, planes=None,
                           beads=200, seed=11),
    "450px_21planes": dict(Nnum=15, Y=450, X=450, z=(-50, 50, 5), img_size_ref=14, iters=8, planes=None,
                           beads=200, seed=21),
    "1005px_41planes": dict(Nnum=15, Y=1005, X=1005, z=(-100, 100, 5), img_size_ref=28, iters=1,
                            planes=[0, 7, 14, 20, 26, 33, 40], beads=2000, seed=41),
}

SAMPLES = 100_000


def splitmix64(x):
    """Vectorised splitmix64 on uint64 (wrapping arithmetic): a portable hash."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return x


def z_planes(case):
    z0, z1, dz = CASES[case]["z"]
    return np.arange(z0, z1 + dz / 2, dz)


def psf(case, only=None):
    import synthetic
    c = CASES[case]
    return synthetic.synthetic_psf(c["Nnum"], z_planes(case), c["img_size_ref"], only=only)


def image(case):
    """[1, Y, X] float32 camera image: background 100 with hash noise in [-10, 10],
    plus beads drawn as integer 5 x 5 stamps (outer product of 1 4 6 4 1) with
    amplitudes 1..8 at hashed positions.  Integer arithmetic throughout."""
    c = CASES[case]
    Y, X, seed = c["Y"], c["X"], c["seed"]
    idx = np.arange(Y * X, dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 40)
    img = 100 + (splitmix64(idx) % np.uint64(21)).astype(np.int64) - 10
    img = img.reshape(Y, X)
    k = np.arange(c["beads"], dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 50)
    hy = splitmix64(k * np.uint64(3) + np.uint64(1))
    hx = splitmix64(k * np.uint64(3) + np.uint64(2))
    ha = splitmix64(k * np.uint64(3) + np.uint64(3))
    ys = (hy % np.uint64(Y - 4)).astype(np.int64)
    xs = (hx % np.uint64(X - 4)).astype(np.int64)
    amps = (ha % np.uint64(8)).astype(np.int64) + 1
    w = np.array([1, 4, 6, 4, 1], np.int64)
    stamp = np.outer(w, w)
    for y, x, a in zip(ys, xs, amps):
        img[y:y + 5, x:x + 5] += a * stamp
    return img.astype(np.float32)[None]


def sample_positions(case, nplanes):
    """SAMPLES flat indices into a [nplanes, Y, X] array (hash-based, may repeat)."""
    c = CASES[case]
    n = nplanes * c["Y"] * c["X"]
    k = np.arange(SAMPLES, dtype=np.uint64) + np.uint64(c["seed"]) * np.uint64(1 << 44)
    return (splitmix64(k) % np.uint64(n)).astype(np.int64)


def checked_planes(case):
    c = CASES[case]
    return list(range(len(z_planes(case)))) if c["planes"] is None else list(c["planes"])


def load_fixture(case):
    import os
    with np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "fp64_%s.npz" % case)) as f:
        return {k: f[k] for k in f.files}


def compare(case, htf, x, fixture=None):
    """Errors of float32 results against the FP64 fixture of a case.

    htf, x: [Z, Y, X] arrays of all planes (numpy).  Returns the largest
    sampled absolute error over the FP64 array's maximum magnitude and the
    sampled relative L2 error, for Htf and for the RL result."""
    f = load_fixture(case) if fixture is None else fixture
    planes = list(f["planes"])
    pos = sample_positions(case, len(planes))
    out = {}
    for key, arr in (("htf", htf), ("x", x)):
        got = np.asarray(arr, np.float64)[planes].ravel()[pos]
        want = f[key].astype(np.float64)
        d = got - want
        out[key + "_max_rel"] = float(np.abs(d).max() / f[key + "_max"])
        out[key + "_rel_l2"] = float(np.linalg.norm(d) / np.linalg.norm(want))
    return out
