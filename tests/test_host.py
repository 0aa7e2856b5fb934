"""CPU tests of the host-side logic: PSF store, plane handling, synthetic inputs,
the RL driver (through an oracle-backed stand-in projector) and frame sharding
over two gloo ranks."""

import os
import socket

import numpy as np
import pytest

from golden_inputs import case_inputs
from oracle import lf_oracle as O


class OracleProjector:
    """Stand-in projector with the reference interface, computing with the CPU oracle."""

    def __init__(self):
        self.storeVolumesOnGPU = False
        self.cacheFH = False
        self.name = "oracle"

    def asnative(self, m):
        return np.asarray(m)

    asnumpy = asnative

    def nativeZeros(self, shape, dtype=float):
        return np.zeros(shape, dtype)

    def nativeDivide(self, a, b, out):
        return np.divide(a, b, out=out)

    def assertNative(self, m):
        assert isinstance(m, np.ndarray)

    def BackwardProjectACC(self, hMatrix, projection, planes, progress, logPrint, numjobs, rlUpdateFunc=None):
        Ht = [hMatrix.Hcc(z, True) for z in range(hMatrix.numZ)]
        vol = O.backward_project(Ht, projection, hMatrix.Nnum, planes=list(planes))
        if rlUpdateFunc is not None:
            rlUpdateFunc(vol, slice(None))
            return None
        return vol

    def ForwardProjectACC(self, hMatrix, realspace, planes, progress, logPrint, numjobs):
        H = [hMatrix.Hcc(z, False) for z in range(hMatrix.numZ)]
        return O.forward_project(H, realspace, hMatrix.Nnum, planes=list(planes))


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / np.max(np.abs(b)))


def test_memmap_roundtrip(tmp_path):
    import psfmatrix
    c = case_inputs("planes_n7")
    stem = tmp_path / "fdnormPSFmatrix_test"
    psfmatrix.SaveReducedMatrices(str(stem), c["H"], c["Ht"])
    hm = psfmatrix.LoadMatrix(str(stem) + ".mat")
    assert hm.Nnum == 7 and hm.numZ == 3 and list(hm.iterableBRange) == [0, 1, 2, 3]
    for z in range(3):
        assert np.array_equal(hm.Hcc(z, False), c["H"][z])
        assert np.array_equal(hm.Hcc(z, True), c["Ht"][z])
        assert hm.PSFShape(z) == (c["hs"][z], c["hs"][z])
    sub = psfmatrix.LoadMatrix(str(stem) + ".mat", numZ=2, zStart=1)
    assert sub.numZ == 2 and np.array_equal(sub.Hcc(0, False), c["H"][1])


def test_hmatrix_arrays_validation():
    import psfmatrix
    c = case_inputs("planes_n7")
    with pytest.raises(ValueError):
        psfmatrix.HMatrixArrays(c["H"], c["Ht"][:2])
    with pytest.raises(ValueError):
        psfmatrix.HMatrixArrays([c["H"][0][:, :, :5]], [c["Ht"][0][:, :, :5]])
    a = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    b = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    assert a.identity() != b.identity()


def test_check_planes():
    import psfmatrix
    import projector
    c = case_inputs("planes_n7")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    assert projector.CheckPlanes(hm, None) == [0, 1, 2]
    assert projector.CheckPlanes(hm, range(1, 3)) == [1, 2]
    with pytest.raises(IndexError):
        projector.CheckPlanes(hm, [3])
    with pytest.raises(ValueError):
        projector.CheckPlanes(hm, [])
    assert projector.Projector_allC is projector.Projector_gb300
    assert projector.Projector_gpuHelpers is projector.Projector_gb300


def test_psf_sizes_follow_reference_rule():
    import synthetic
    # M40 optics, z -25..25 um: support sizes of the reference generator
    assert synthetic.psf_sizes(15, np.arange(-25, 26, 5), 7) == [211, 181, 151, 91, 61, 61, 61, 91, 151, 181, 211]


def test_synthetic_psf_properties():
    import synthetic
    H, Ht = synthetic.synthetic_psf(5, [-10, 0, 10], 2)
    for h in H:
        assert np.allclose(h.sum(axis=(2, 3)), 1.0, atol=1e-5) and h.min() >= 0
    rng = np.random.default_rng(0)
    x = rng.random((3, 1, 30, 35))
    y = rng.random((1, 30, 35))
    hx = O.forward_project(H, x, 5, method="direct", dtype=np.float64)
    hty = O.backward_project(Ht, y, 5, method="direct", dtype=np.float64)
    assert abs(np.sum(hx * y) - np.sum(x * hty)) / np.sum(hx * y) < 1e-12


def test_bead_and_poisson_inputs():
    import synthetic
    v, pos = synthetic.bead_volume((3, 20, 20), 5, seed=1)
    v2, _ = synthetic.bead_volume((3, 20, 20), 5, seed=1)
    assert np.array_equal(v, v2) and v.dtype == np.float32 and v.max() > 0 and len(pos) == 5
    img = synthetic.poisson_image(np.zeros((1, 4, 4)), background=100.0, seed=0)
    assert img.dtype == np.float32 and 50 < img.mean() < 150


@pytest.mark.parametrize("name", ["rl_prevedel", "rl_standard"])
def test_rl_driver_generic_path_matches_reference(name):
    import lfdeconv
    import psfmatrix
    c = case_inputs(name)
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    Z = len(c["hs"])
    x0 = None if c["prevedel"] else np.ones((Z,) + c["img"].shape, np.float32)
    r = lfdeconv.DeconvRL(hm, None, c["iters"], x0, logPrint=False, projector=OracleProjector(), im=c["img"],
                          prevedel=c["prevedel"])
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz"))[name + "/rl"]
    assert rel(r, g) < 1e-5


def test_rl_driver_writes_into_out():
    import lfdeconv
    import psfmatrix
    c = case_inputs("rl_prevedel")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    want = lfdeconv.DeconvRL(hm, None, 1, None, logPrint=False, projector=OracleProjector(), im=c["img"])
    out = np.empty_like(want)
    r = lfdeconv.DeconvRL(hm, None, 1, None, logPrint=False, projector=OracleProjector(), im=c["img"], out=out)
    assert r is out and np.array_equal(out, want)


def test_rl_driver_rejects_trust_mask_with_prevedel():
    import lfdeconv
    import psfmatrix
    c = case_inputs("rl_prevedel")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    with pytest.raises(ValueError):
        lfdeconv.DeconvRL(hm, None, 1, None, logPrint=False, projector=OracleProjector(), im=c["img"],
                          prevedel=True, trustMask=np.ones(c["img"].shape[1:], np.float32))


def test_frame_shard_partition():
    import sharding
    for T in (1, 5, 8, 13):
        for world in (1, 2, 3, 4):
            parts = [sharding.frame_shard(T, r, world) for r in range(world)]
            idx = [i for s in parts for i in range(s.start, s.stop)]
            assert idx == list(range(T))
            sizes = [s.stop - s.start for s in parts]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "fast-light-field_gb300"), os.path.join(root, "tests", "golden"),
              os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        import psfmatrix
        import sharding
        from test_host import OracleProjector
        c = case_inputs("rl_prevedel")
        hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
        rng = np.random.default_rng(4)
        im = (rng.random((3,) + c["img"].shape[1:]) * 1000 + 100).astype(np.float32)
        r = sharding.deconv_rl_sharded(hm, im, 2, OracleProjector())
        if rank == 0:
            np.save(out_path, r)
    finally:
        dist.destroy_process_group()


def test_frame_sharded_rl_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    import lfdeconv
    import psfmatrix
    out = str(tmp_path / "r0.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    c = case_inputs("rl_prevedel")
    hm = psfmatrix.HMatrixArrays(c["H"], c["Ht"])
    rng = np.random.default_rng(4)
    im = (rng.random((3,) + c["img"].shape[1:]) * 1000 + 100).astype(np.float32)
    single = lfdeconv.DeconvRL(hm, None, 2, None, logPrint=False, projector=OracleProjector(), im=im)
    sharded = np.load(out)
    assert sharded.shape == single.shape
    assert rel(sharded, single) < 1e-6


def test_warm_start_learning_rate_schedule():
    """The warm start's training schedule: linear ramp, then the cosine to zero."""
    import warmstart
    lr = warmstart.learning_rate
    assert lr(0, 1600, 1e-3, 100) == pytest.approx(1e-5 * 0.5 * (1 + np.cos(0.0)))
    assert lr(49, 1600, 1e-3, 100) == pytest.approx(0.5e-3 * 0.5 * (1 + np.cos(np.pi * 49 / 1599)))
    assert lr(99, 1600, 1e-3, 100) == pytest.approx(1e-3 * 0.5 * (1 + np.cos(np.pi * 99 / 1599)))
    assert lr(1599, 1600, 1e-3, 100) == pytest.approx(0.0, abs=1e-15)
    assert lr(0, 10, 2e-3, 0) == pytest.approx(2e-3)
    assert lr(0, 1, 2e-3, 0) == pytest.approx(2e-3)      # a single step: no division by zero
    rates = [lr(k, 1600, 1e-3, 100) for k in range(1600)]
    assert max(rates) <= 1e-3 and int(np.argmax(rates)) == 99
