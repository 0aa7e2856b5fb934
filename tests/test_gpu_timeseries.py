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
    # the driver takes the .mat path; its memmap folder (same name, no extension) is read
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
