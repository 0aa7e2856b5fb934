"""Seeded synthetic inputs for tests and benchmarks: PSF sets, bead/filament volumes.

The reference generates light-field PSFs with a wave-optics model
(generate_psf.py:63-798), which is not part of the projection path and takes
minutes to hours.  ``synthetic_psf`` builds stand-in PSF sets with the same
array shapes (the per-plane support ``h_z`` follows the reference's CAindex
rule, generate_psf.py:624-630) and the properties the projection relies on:
non-negative, each forward PSF summing to 1 (generate_psf.py:606-612), mirror
symmetric across lenslet offsets, and an ``Ht`` that is the exact adjoint of
``H`` (the property the reference's "rubber stamp" transpose computes,
generate_psf.py:695-719).  Each PSF is a sum of two separable lenslet-periodic
spot patterns whose spread grows with |z|.
"""

import math

import numpy as np

__all__ = ["psf_sizes", "synthetic_psf", "bead_volume", "filament_volume", "poisson_image",
           "random_psf"]


def psf_sizes(Nnum, z_um, img_size_ref, zmax_um=None):
    """Per-plane PSF side ``h_z = 2*max(Nnum*ceil(R*|z|/zmax), 2*Nnum) + 1``."""
    z = np.asarray(z_um, dtype=np.float64)
    zmax = float(np.max(np.abs(z))) if zmax_um is None else float(zmax_um)
    out = []
    for zz in z:
        il = math.ceil(img_size_ref * abs(zz) / zmax - 1e-9) if zmax > 0 else 0
        hw = max(Nnum * il, 2 * Nnum)
        out.append(2 * hw + 1)
    return out


def _profiles(Nnum, h, spread_lenslets, sigma, gamma, alpha, n_terms):
    """Lenslet-periodic 1-D spot profiles u_b(d), d in [-ch, ch], b in [0, N); each sums to 1."""
    N = Nnum
    c = N // 2
    ch = (h - 1) // 2
    d = np.arange(-ch, ch + 1, dtype=np.float64)
    K = max(0, int(n_terms))
    ks = np.arange(-K, K + 1, dtype=np.float64)
    w = np.exp(-ks ** 2 / (2.0 * (0.5 + 0.6 * spread_lenslets) ** 2))
    u = np.zeros((N, h))
    for b in range(N):
        centres = ks * N + gamma * (b - c) + alpha * ks
        u[b] = np.sum(w[:, None] * np.exp(-(d[None, :] - centres[:, None]) ** 2 / (2.0 * sigma ** 2)), axis=0)
        u[b] /= u[b].sum()
    return u


def synthetic_psf(Nnum, z_um, img_size_ref, dtype=np.float32, only=None):
    """Stand-in PSF set: lists of per-plane ``H`` and ``Ht`` quadrants ``[n_h, n_h, h, h]``.

    ``Hfull[b][a] = sum_r u^r_b (x) u^r_a`` with mirror-symmetric profiles, so the
    reference's symmetry map reproduces the full set exactly; ``Ht`` is built
    by the adjoint relation ``Ht_ba(y, x) = H_{(b+y-ch)%N, (a+x-ch)%N}(2ch-y, 2ch-x)``.
    ``only``: plane indices to compute (the others are None in the lists).
    """
    N = int(Nnum)
    nh = (N + 1) // 2
    hs = psf_sizes(N, z_um, img_size_ref)
    zmax = float(np.max(np.abs(z_um))) or 1.0
    H_list, Ht_list = [], []
    for zi, (zz, h) in enumerate(zip(z_um, hs)):
        if only is not None and zi not in only:
            H_list.append(None)
            Ht_list.append(None)
            continue
        ch = (h - 1) // 2
        rel = abs(zz) / zmax
        spread = img_size_ref * rel
        nterm = max(1, (h // 2) // N - 1)
        sgn = 1.0 if zz >= 0 else -1.0
        comps = [
            (0.75, _profiles(N, h, spread, 0.9 + 0.8 * rel, 0.55, 0.35 * sgn * rel, nterm)),
            (0.25, _profiles(N, h, 0.5 * spread + 0.5, 1.6 + 1.2 * rel, -0.3, 0.15 * sgn * rel, nterm)),
        ]
        H = np.zeros((nh, nh, h, h))
        Ht = np.zeros((nh, nh, h, h))
        yy = np.arange(h)
        for wgt, u in comps:
            H += wgt * np.einsum("by,ax->bayx", u[:nh], u[:nh])
            # adjoint profiles: ut_b(y) = u_{(b + y - ch) mod N}(ch - y)
            ut = np.empty((nh, h))
            for b in range(nh):
                ut[b] = u[(b + yy - ch) % N, (2 * ch - yy)]
            Ht += wgt * np.einsum("by,ax->bayx", ut, ut)
        H_list.append(H.astype(dtype))
        Ht_list.append(Ht.astype(dtype))
    return H_list, Ht_list


def random_psf(Nnum, hs, seed=0, dtype=np.float32):
    """Unstructured PSF quadrants (uniform random, each PSF summing to 1) for parity tests.

    Unlike ``synthetic_psf`` these carry no symmetry beyond what the reference's
    symmetry map imposes, so they exercise every index map of the projector.
    """
    rng = np.random.default_rng(seed)
    nh = (int(Nnum) + 1) // 2
    H, Ht = [], []
    for h in hs:
        a = rng.random((nh, nh, h, h))
        a /= a.sum(axis=(2, 3), keepdims=True)
        b = rng.random((nh, nh, h, h))
        b /= b.sum(axis=(2, 3), keepdims=True)
        H.append(a.astype(dtype))
        Ht.append(b.astype(dtype))
    return H, Ht


def _splat(vol, zc, yc, xc, amp, sigma, radius=3):
    Z, Y, X = vol.shape
    z0, y0, x0 = int(round(zc)), int(round(yc)), int(round(xc))
    zs = np.arange(max(0, z0 - radius), min(Z, z0 + radius + 1))
    ys = np.arange(max(0, y0 - radius), min(Y, y0 + radius + 1))
    xs = np.arange(max(0, x0 - radius), min(X, x0 + radius + 1))
    if len(zs) == 0 or len(ys) == 0 or len(xs) == 0:
        return
    gz = np.exp(-(zs - zc) ** 2 / (2 * sigma ** 2))
    gy = np.exp(-(ys - yc) ** 2 / (2 * sigma ** 2))
    gx = np.exp(-(xs - xc) ** 2 / (2 * sigma ** 2))
    vol[np.ix_(zs, ys, xs)] += amp * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]


def bead_volume(shape, n_beads, seed=0, sigma=1.0, amp_range=(500.0, 1000.0), positions=None):
    """``[Z, Y, X]`` float32 volume of Gaussian beads (sigma in voxels, amplitude U(a, b))."""
    rng = np.random.default_rng(seed)
    Z, Y, X = shape
    vol = np.zeros(shape, dtype=np.float64)
    if positions is None:
        positions = np.stack([rng.uniform(0, Z - 1, n_beads), rng.uniform(0, Y - 1, n_beads),
                              rng.uniform(0, X - 1, n_beads)], axis=1)
    amps = rng.uniform(amp_range[0], amp_range[1], len(positions))
    for (zc, yc, xc), a in zip(positions, amps):
        _splat(vol, zc, yc, xc, a, sigma)
    return vol.astype(np.float32), positions


def filament_volume(shape, n_filaments, seed=0, width=1.5, intensity=500.0, steps=200):
    """``[Z, Y, X]`` float32 volume of random-walk filaments."""
    rng = np.random.default_rng(seed)
    Z, Y, X = shape
    vol = np.zeros(shape, dtype=np.float64)
    for _ in range(n_filaments):
        p = np.array([rng.uniform(0, Z - 1), rng.uniform(0, Y - 1), rng.uniform(0, X - 1)])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        for _ in range(steps):
            _splat(vol, p[0], p[1], p[2], intensity / 4.0, width, radius=3)
            d = d + 0.3 * rng.normal(size=3)
            d /= np.linalg.norm(d)
            p = np.clip(p + d * np.array([0.3, 1.0, 1.0]), 0, np.array([Z - 1, Y - 1, X - 1]))
    return vol.astype(np.float32)


def poisson_image(clean, background=100.0, seed=0):
    """Camera image: Poisson(clean + background), float32."""
    rng = np.random.default_rng(seed)
    lam = np.clip(np.asarray(clean, dtype=np.float64) + background, 0, None)
    return rng.poisson(lam).astype(np.float32)
