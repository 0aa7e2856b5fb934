"""GPU test of the time-series driver (the reference's deconvolve_time_series.py):
TIFF frames of mixed sizes in, one deconvolved [Z, Y, X] TIFF per frame out."""

import os

import numpy as np
import pytest

from oracle import lf_oracle as O

pytestmark = pytest.mark.gpu

RL_TOL = 1e-4


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def test_time_series_driver_mixed_sizes(tmp_path, built_lib):
    import deconvolve_time_series as dts
    import lfdeconv
    import projector
    import psfmatrix
    import synthetic
    import tiffio
    N, iters = 5, 3
    H, Ht = synthetic.synthetic_psf(N, [-10, 0, 10], 2)
    # the time-series CLI takes the .mat path; its memmap folder (same name, no extension) is read
    psfmatrix.SaveReducedMatrices(str(tmp_path / "psf"), H, Ht)
    rng = np.random.default_rng(11)
    shapes = [(40, 35), (30, 30), (40, 35), (30, 30), (40, 35)]     # interleaved sizes
    files, images = [], []
    for k, s in enumerate(shapes):
        im = (rng.random(s) * 500 + 100).astype(np.uint16)
        path = str(tmp_path / ("frame%d.tif" % k))
        tiffio.imwrite(path, im)
        files.append(path)
        images.append(im.astype(np.float32))
    out = tmp_path / "out"
    written = dts.main(["-p", str(tmp_path / "psf.mat"), "-d", str(out), "-b", "2", "-i", str(iters),
                        "-t"] + files)
    assert sorted(written) == sorted(str(out / ("frame%d_deconvolved.tif" % k)) for k in range(len(files)))
    hm = psfmatrix.HMatrixArrays(H, Ht)
    p = projector.Projector_gb300()
    for k, im in enumerate(images):
        vol = tiffio.imread(str(out / ("frame%d_deconvolved.tif" % k)))
        assert vol.dtype == np.float32 and vol.shape == (3,) + im.shape
        Htf = lfdeconv.BackwardProjectACC(hm, im[np.newaxis], projector=p, logPrint=False)
        ref = lfdeconv.DeconvRL(hm, Htf, iters, Htf.copy(), logPrint=False, projector=p)
        assert rel(vol, ref[:, 0]) < RL_TOL
    o = O.deconv_rl(H, Ht, N, iters, im=images[1][np.newaxis], method="direct", dtype=np.float64)
    assert rel(tiffio.imread(str(out / "frame1_deconvolved.tif")), o[:, 0]) < RL_TOL


def test_time_series_driver_rejects_bad_arguments(tmp_path, built_lib):
    import deconvolve_time_series as dts
    with pytest.raises(SystemExit):
        dts.main(["-p", str(tmp_path / "psf.mat"), "-b", "0", "-t", "x.tif"])
    with pytest.raises(SystemExit):
        dts.main(["-p", str(tmp_path / "psf.mat"), "-i", "0", "-t", "x.tif"])


def test_time_series_driver_with_warm_start(tmp_path, built_lib):
    """--warm-start: a network trained for one frame size (warmstart.py command line)
    starts RL for frames of that size; other sizes start from Htf; saved weights come
    back unchanged and refuse another image size."""
    import deconvolve_time_series as dts
    import lfdeconv
    import projector
    import psfmatrix
    import synthetic
    import tiffio
    import warmstart
    N = 5
    H, Ht = synthetic.synthetic_psf(N, [-10, 0, 10], 2)
    psfmatrix.SaveReducedMatrices(str(tmp_path / "psf"), H, Ht)
    net = str(tmp_path / "net.npz")
    warmstart.main(["-p", str(tmp_path / "psf.mat"), "-s", "40", "40", "-o", net, "--steps", "40", "--beads", "20"])
    assert warmstart.WarmStart.trained_shape(net) == (3, 40, 40)
    hm = psfmatrix.LoadMatrix(str(tmp_path / "psf.mat"))
    p = projector.Projector_gb300()
    ws = warmstart.WarmStart(p, hm, 40, 40).load(net)
    with np.load(net) as f:
        assert np.array_equal(ws.net.state_dict()["e0a.w"], f["e0a.w"])
    with pytest.raises(ValueError, match="trained for"):
        warmstart.WarmStart(p, hm, 30, 30).load(net)
    rng = np.random.default_rng(2)
    files, images = [], []
    for k, s in enumerate([(40, 40), (30, 30)]):
        im = (rng.random(s) * 500 + 100).astype(np.uint16)
        path = str(tmp_path / ("w%d.tif" % k))
        tiffio.imwrite(path, im)
        files.append(path)
        images.append(im.astype(np.float32))
    out = dts.main(["-p", str(tmp_path / "psf.mat"), "-t"] + files + ["-d", str(tmp_path / "out"), "-i", "2",
                                                                     "-w", net])
    vols = {os.path.basename(o): tiffio.imread(o) for o in out}
    # the 40 x 40 frame: RL from the network's start volume
    htf = lfdeconv.BackwardProjectACC(hm, images[0][None], None, projector=p, logPrint=False)
    import torch
    x0 = ws.initial_volume(torch.as_tensor(htf, device="cuda"))
    want = lfdeconv.DeconvRL(hm, htf, 2, x0, logPrint=False, projector=p)
    assert rel(vols["w0_deconvolved.tif"], want[:, 0]) < RL_TOL
    # the 30 x 30 frame: RL from Htf, as without the option
    htf1 = lfdeconv.BackwardProjectACC(hm, images[1][None], None, projector=p, logPrint=False)
    want1 = lfdeconv.DeconvRL(hm, htf1, 2, htf1, logPrint=False, projector=p)
    assert rel(vols["w1_deconvolved.tif"], want1[:, 0]) < RL_TOL
