"""FP32 GPU Richardson-Lucy against the FP64 oracle at benchmark sizes.

The accuracy statement per configuration: max and relative L2 error of the
GPU's FP32 RL against an FP64 CPU restatement of the same iterations.  Runs
only with FLF_FP64_CHECK=1 (a few minutes of host CPU);
``python tests/test_gpu_fp64_rl.py`` prints the numbers.

* 450 x 450 px, Nnum 15, 11 planes at -25..25 um, 8 Prevedel
  iterations from a uniform volume;
* full field, cut to 3 planes (z = -100, 0, 100 um, PSF sizes 841 / 61 / 841)
  of the 1005 x 1005 workload, 4 iterations.

The FP64 side is the reference's special-FFT projection (oracle
project_plane_special, complex128), split by lenslet offset over a process
pool started with spawn; partial projections add up because the projection is
linear in the offsets.
"""

import multiprocessing as mp
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (ROOT, os.path.join(ROOT, "fast-light-field_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("FLF_FP64_CHECK") != "1", reason="set FLF_FP64_CHECK=1 (slow)")]

TOL = 1e-4


def _partial(args):
    """FP64 projection of src [T, Y, X] through the offsets `offs` of one plane."""
    from oracle import lf_oracle as O
    src, Hred, N, offs = args
    Hred = np.asarray(Hred, np.float64)
    T, Y, X = src.shape
    c = N // 2
    h = Hred.shape[-1]
    fshape, full = O.convolution_shape((Y, X), (h, h), N, True)
    FY, FX = fshape
    fy, fx, RX = FY // N, FX // N, FX // 2 + 1
    ky, kx = np.arange(FY), np.arange(RX)
    acc = np.zeros((T, FY, RX), np.complex128)
    for b, a in offs:
        bb, aa = min(b, N - 1 - b), min(a, N - 1 - a)
        P = Hred[bb, aa] if aa >= bb else Hred[aa, bb].T
        if b > c:
            P = P[::-1, :]
        if a > c:
            P = P[:, ::-1]
        S = np.fft.fft2(src[:, b::N, a::N], s=(fy, fx), axes=(1, 2))
        ph = np.exp(-2j * np.pi * b * ky / FY)[:, None] * np.exp(-2j * np.pi * a * kx / FX)[None, :]
        FH = np.fft.fft2(P, s=(FY, FX))[:, :RX]
        acc += S[:, ky % fy][:, :, kx % fx] * ph[None] * FH[None]
    img = np.fft.irfft2(acc, s=(FY, FX), axes=(1, 2))[:, :full[0], :full[1]]
    return O._centered(img, (Y, X))


class Fp64Projector:
    def __init__(self, H, Ht, N, pool, chunks=9):
        self.H, self.Ht, self.N, self.pool = H, Ht, N, pool
        offs = [(b, a) for b in range(N) for a in range(N)]
        k = -(-len(offs) // chunks)
        self.chunks = [offs[i:i + k] for i in range(0, len(offs), k)]

    def _run(self, mats, srcs):
        tasks = [(srcs[z], mats[z], self.N, ch) for z in range(len(mats)) for ch in self.chunks]
        parts = self.pool.map(_partial, tasks)
        n = len(self.chunks)
        return [sum(parts[z * n:(z + 1) * n]) for z in range(len(mats))]

    def forward(self, vol):
        return sum(self._run(self.H, [vol[z] for z in range(len(self.H))]))

    def backward(self, img):
        return np.stack(self._run(self.Ht, [img] * len(self.Ht)))


def rl_fp64(proj, img, iters):
    htf = proj.backward(img)
    x = np.ones_like(htf)
    with np.errstate(divide="ignore", invalid="ignore"):
        for _ in range(iters):
            x = x * (htf / proj.backward(proj.forward(x)))
            x[np.isnan(x)] = 0
    return x


def compare(workload, keep, iters, pool):
    import bench
    import lfdeconv
    import projector
    import torch
    hm, H, Ht, z, gt, Y, X = bench.build_problem(bench.WORKLOADS[workload], keep=keep)
    p = projector.Projector_gb300()
    clean = p.ForwardProjectACC(hm, gt[:, None], None)
    rng = np.random.default_rng(5)
    img = rng.poisson(np.clip(clean + 100.0, 0, None)).astype(np.float32)
    x_gpu = lfdeconv.DeconvRL(hm, None, iters, np.ones((len(z), 1, Y, X), np.float32), logPrint=False,
                              projector=p, im=img).astype(np.float64)
    del p
    torch.cuda.empty_cache()
    Hd = [np.asarray(hm.Hcc(c, False), np.float64) for c in range(hm.numZ)]
    Htd = [np.asarray(hm.Hcc(c, True), np.float64) for c in range(hm.numZ)]
    x64 = rl_fp64(Fp64Projector(Hd, Htd, hm.Nnum, pool), img.astype(np.float64), iters)
    err = np.abs(x_gpu - x64)
    return {"max_abs_rel": float(err.max() / np.abs(x64).max()),
            "rel_l2": float(np.linalg.norm(x_gpu - x64) / np.linalg.norm(x64)),
            "planes": int(len(z)), "image": [int(Y), int(X)], "iterations": iters}


def _pool():
    return mp.get_context("spawn").Pool(max(1, min(os.cpu_count() or 1, 32)))


def test_450px_11planes_fp32_rl_matches_fp64(built_lib):
    with _pool() as pool:
        r = compare("small", None, 8, pool)
    assert r["max_abs_rel"] < TOL and r["rel_l2"] < TOL, r


def test_full_field_cut_fp32_rl_matches_fp64(built_lib):
    with _pool() as pool:
        r = compare("fullfield", [0, 20, 40], 4, pool)
    assert r["max_abs_rel"] < TOL and r["rel_l2"] < TOL, r


if __name__ == "__main__":
    import time
    import build_lib
    build_lib.build()
    with _pool() as pool:
        for name, keep, it in (("small", None, 8), ("fullfield", [0, 20, 40], 4)):
            t0 = time.time()
            print(name, compare(name, keep, it, pool), "%.0f s" % (time.time() - t0), flush=True)
